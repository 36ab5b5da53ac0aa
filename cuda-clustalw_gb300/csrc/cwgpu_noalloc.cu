// Allocation-free entry point: cwgpu_align_pairs_noalloc.
//
// Some callers cannot call cudaMalloc: code running inside a host framework
// that owns all device memory through its own pool (and forbids side
// allocations), processes with a fixed device-memory budget reserved at
// start-up, or callers between a memory-pool reservation and its use. They
// can still hand over device buffers they already own. This entry point runs
// the same pair kernel as cwgpu_align_pairs, but every byte of working memory
// it needs (per-warp boundary rows and residue copies, the queue head, the cell
// counters, the status words and the gap-open table) lives in one file-scope static device
// array, g_noalloc_scratch, of CWGPU_NOALLOC_SCRATCH_BYTES (16 MiB). Every GPU that
// loads this library holds that array until the process exits.
//
// In host code g_noalloc_scratch names a host-side stand-in, not a device
// address; a kernel given it would fault or read the wrong memory. So the
// first call on each device, with that device current, looks the address up
// with cudaGetSymbolAddress (and the occupancy of the kernel) and caches both
// per device.
//
// All calls share the one array and keep the last call's contents; the
// control words are cleared at the start of each call. Calls whose GPU work
// overlaps (from different host threads or streams) race on the array.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "cwgpu.h"
#include "cwgpu_device.cuh"
#include "cwgpu_layout.h"

namespace {

constexpr int kNaWarpsPerBlock = 4;
constexpr size_t kNaRegionBytes = (size_t)cwgpu::warp_region_bytes(CWGPU_NUMRES);  // per warp, dynamic smem
constexpr size_t kNaScratchBytes = (size_t)CWGPU_NOALLOC_SCRATCH_BYTES;
// Control words: [0] queue head, [1..3] cell counts, then three status words
// (int): rejected input, matrix entry outside int16, device-side limit.
constexpr size_t kNaCtrlBytes = 256;
constexpr int kNaStatusInput = 0, kNaStatusMatrix = 1, kNaStatusLimit = 2;
constexpr size_t kNaTableBytes = ((size_t)(CWGPU_NOALLOC_MAX_LEN + 1) * sizeof(int32_t) + 255) & ~(size_t)255;
constexpr size_t kNaRowsOffset = kNaCtrlBytes + kNaTableBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

struct NaArgs {
    const int8_t* codes;
    const int64_t* offs;
    const int32_t* lens;
    const int32_t* pairs;
    const int32_t* matrix;
    float* dist;
    cwgpu_pair_stats* stats;
    unsigned char* scratch;  // device address of g_noalloc_scratch
    long long npairs;
    int nseqs;
    int max_len;
    int ge;
    int gp1, gp2;
};

__device__ __forceinline__ int* na_status(unsigned char* scratch, int which) {
    return reinterpret_cast<int*>(scratch + 4 * sizeof(unsigned long long)) + which;
}

// Bytes of one warp slot: the two boundary rows, then the pair's residues in
// the pair kernels' layout (guards, forward and reversed copy of each
// sequence; cwgpu_layout.h), rounded to 256.
__host__ __device__ inline size_t na_slot_bytes(int max_len) {
    const size_t rows = 2 * (size_t)(max_len + 1) * sizeof(int2);
    const size_t codes = 2 * (size_t)cwgpu::kGuard + 4 * (size_t)cwgpu::rev_offset(max_len);
    return (rows + codes + 255) & ~(size_t)255;
}

// One pair (FullPairwiseAlign.cpp:112-183) with device-side input checks: a
// pair index, a negative sequence offset, a length above max_len or a residue
// code outside [0, 31] sets the input status word and the pair is skipped. The
// residue counts len1/len2 of :100-127 are counted here instead of being
// uploaded. The two sequences are copied into the slot (forward and reversed)
// and read back from there with plain loads, since the kernel wrote them.
__device__ void na_align_pair(const NaArgs& a, long long q, const cwgpu::Env& X, int2* bufA, int2* bufB,
                              int8_t* slot_codes, unsigned long long (&acc)[3]) {
    const int lane = threadIdx.x & 31;
    int* status = na_status(a.scratch, kNaStatusInput);
    const int32_t* go_table = reinterpret_cast<const int32_t*>(a.scratch + kNaCtrlBytes);
    const int si = a.pairs[2 * q], sj = a.pairs[2 * q + 1];
    if (si < 0 || si >= a.nseqs || sj < 0 || sj >= a.nseqs) {
        if (lane == 0) atomicExch(status, 1);
        return;
    }
    const int n = a.lens[si], m = a.lens[sj];
    if (n < 0 || m < 0 || n > a.max_len || m > a.max_len || (n > 0 && a.offs[si] < 0) || (m > 0 && a.offs[sj] < 0)) {
        if (lane == 0) atomicExch(status, 1);
        return;
    }
    const int8_t* s1 = a.codes + a.offs[si];
    const int8_t* s2 = a.codes + a.offs[sj];
    int bad = 0, r1 = 0, r2 = 0;
    for (int i = lane; i < n; i += 32) {
        const int c = s1[i];
        bad |= (c < 0 || c >= CWGPU_NUMRES);
        r1 += (c != a.gp1 && c != a.gp2);
    }
    for (int i = lane; i < m; i += 32) {
        const int c = s2[i];
        bad |= (c < 0 || c >= CWGPU_NUMRES);
        r2 += (c != a.gp1 && c != a.gp2);
    }
    if (__any_sync(cwgpu::kFull, bad)) {
        if (lane == 0) atomicExch(status, 1);
        return;
    }
    const int len1 = __reduce_add_sync(cwgpu::kFull, r1), len2 = __reduce_add_sync(cwgpu::kFull, r2);
    int8_t* p1 = slot_codes + cwgpu::kGuard;
    int8_t* p1r = p1 + cwgpu::rev_offset(n);
    int8_t* p2 = p1r + cwgpu::rev_offset(n);
    int8_t* p2r = p2 + cwgpu::rev_offset(m);
    __syncwarp();  // the previous pair's reads of the slot are done
    for (int i = lane; i < n; i += 32) {
        const int8_t c = s1[i];
        p1[i] = c;
        p1r[n - 1 - i] = c;
    }
    for (int i = lane; i < m; i += 32) {
        const int8_t c = s2[i];
        p2[i] = c;
        p2r[m - 1 - i] = c;
    }
    __syncwarp();  // copies visible to the whole warp
    cwgpu_pair_stats st;
    const float dist = cwgpu::align_one<cwgpu::kR, false>(p1, n, p2, m, len1, len2, go_table[min(n, m)], a.ge, bufA,
                                                          bufB, X, st, acc);
    if (lane == 0) {
        a.dist[q] = dist;
        if (a.stats) a.stats[q] = st;
    }
}

// The matrix is checked while it is staged: the score profile holds int16
// entries, so an entry outside [-32768, 32767] sets the matrix status word and
// every block returns before aligning anything (cwgpu_set_matrix makes the same
// check on the host for the allocating entry points).
__global__ void __launch_bounds__(kNaWarpsPerBlock * 32) k_pairwise_noalloc(NaArgs a) {
    __shared__ int smat[CWGPU_NUMRES * CWGPU_NUMRES];
    extern __shared__ __align__(16) uint16_t na_region[];
    int bad_entry = 0;
    for (int i = threadIdx.x; i < CWGPU_NUMRES * CWGPU_NUMRES; i += blockDim.x) {
        const int v = a.matrix[i];
        bad_entry |= (v < -32768 || v > 32767);
        smat[i] = v;
    }
    if (__syncthreads_or(bad_entry)) {
        if (threadIdx.x == 0) atomicExch(na_status(a.scratch, kNaStatusMatrix), 1);
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * kNaWarpsPerBlock + warp;
    cwgpu::Env X;
    X.smat = smat;
    X.region = na_region + (size_t)warp * (kNaRegionBytes / sizeof(uint16_t));
    X.K = CWGPU_NUMRES;
    X.gp1 = (a.gp1 >= 0 && a.gp1 < CWGPU_NUMRES) ? a.gp1 : -1;
    X.gp2 = (a.gp2 >= 0 && a.gp2 < CWGPU_NUMRES) ? a.gp2 : -1;
    X.tiny_m = 32;
    X.tiny_n = cwgpu::kTinyMaxN;
    unsigned long long* ctrl = reinterpret_cast<unsigned long long*>(a.scratch);
    X.err = na_status(a.scratch, kNaStatusLimit);
    unsigned char* my_slot = a.scratch + kNaRowsOffset + (size_t)slot * na_slot_bytes(a.max_len);
    int2* bufA = reinterpret_cast<int2*>(my_slot);
    int2* bufB = bufA + (a.max_len + 1);
    int8_t* slot_codes = reinterpret_cast<int8_t*>(bufB + (a.max_len + 1));
    unsigned long long acc[3] = {0, 0, 0};
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(ctrl, 1ULL);
        k = __shfl_sync(cwgpu::kFull, k, 0);
        if (k >= (unsigned long long)a.npairs) break;
        na_align_pair(a, (long long)k, X, bufA, bufB, slot_codes, acc);
    }
    if (lane == 0 && (acc[0] | acc[1] | acc[2])) {
        atomicAdd(ctrl + 1, acc[0]);
        atomicAdd(ctrl + 2, acc[1]);
        atomicAdd(ctrl + 3, acc[2]);
    }
}

struct NaDevice {
    bool ready = false;
    unsigned char* scratch = nullptr;
    int sm_count = 0;
    int blocks_per_sm = 0;
};

constexpr int kNaMaxDevices = 64;
NaDevice g_na_devices[kNaMaxDevices];
std::mutex g_na_mutex;

int na_reject(const char* why) {
    fprintf(stderr, "cwgpu_align_pairs_noalloc: %s\n", why);
    return CWGPU_ERR_ARG;
}

// Once per device, with that device current: the device address of the static
// scratch array, and the occupancy of the kernel.
int na_setup(int dev, NaDevice** out) {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    NaDevice& d = g_na_devices[dev];
    if (!d.ready) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            fprintf(stderr, "cwgpu_align_pairs_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return CWGPU_ERR_CUDA;
        }
        int sms = 0, per_sm = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_pairwise_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(kNaRegionBytes * kNaWarpsPerBlock));
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairwise_noalloc, kNaWarpsPerBlock * 32,
                                                              kNaRegionBytes * kNaWarpsPerBlock);
        if (e != cudaSuccess) {
            fprintf(stderr, "cwgpu_align_pairs_noalloc: set-up failed: %s\n", cudaGetErrorString(e));
            return CWGPU_ERR_CUDA;
        }
        d.scratch = static_cast<unsigned char*>(ptr);
        d.sm_count = sms;
        d.blocks_per_sm = per_sm < 1 ? 1 : per_sm;
        d.ready = true;
    }
    *out = &d;
    return CWGPU_OK;
}

}  // namespace

extern "C" int cwgpu_align_pairs_noalloc(const int8_t* d_codes, const int64_t* d_offsets, const int32_t* d_lens,
                                         int32_t nseqs, int32_t max_len, const int32_t* d_matrix,
                                         const cwgpu_params* params, const int32_t* d_pairs, int64_t npairs,
                                         float* d_dist, cwgpu_pair_stats* d_stats, void* stream) {
    if (!params || nseqs < 0 || npairs < 0) return na_reject("bad argument");
    if (max_len < 0 || max_len > CWGPU_NOALLOC_MAX_LEN)
        return na_reject("max_len is above CWGPU_NOALLOC_MAX_LEN (8191 residues), the limit of this entry point");
    if (npairs == 0) return CWGPU_OK;
    if (!d_codes || !d_offsets || !d_lens || !d_matrix || !d_pairs || !d_dist) return na_reject("null device pointer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return na_reject("no usable current device");
    NaDevice* d = nullptr;
    int rc = na_setup(dev, &d);
    if (rc) return rc;

    // Gap-open penalty by min(n, m), with the reference's expression types
    // (FullPairwiseAlign.cpp:129-146); entry 0 is never used.
    int32_t table[CWGPU_NOALLOC_MAX_LEN + 1];
    int32_t ge = 0;
    cwgpu_gap_penalties(params, 1, 1, &table[0], &ge);
    table[0] = 0;
    for (int L = 1; L <= max_len; ++L) {
        int32_t unused = 0;
        cwgpu_gap_penalties(params, L, L, &table[L], &unused);
    }

    const long long slots = (long long)((kNaScratchBytes - kNaRowsOffset) / na_slot_bytes(max_len));
    long long grid = slots / kNaWarpsPerBlock;
    const long long full = (long long)d->sm_count * d->blocks_per_sm;
    if (grid > full) grid = full;
    const long long need = (npairs + kNaWarpsPerBlock - 1) / kNaWarpsPerBlock;
    if (grid > need) grid = need;
    if (grid < 1) return na_reject("max_len leaves no room for one block of scratch rows");

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = cudaMemsetAsync(d->scratch, 0, kNaCtrlBytes, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d->scratch + kNaCtrlBytes, table, sizeof(int32_t) * (size_t)(max_len + 1),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        NaArgs a;
        a.codes = d_codes;
        a.offs = d_offsets;
        a.lens = d_lens;
        a.pairs = d_pairs;
        a.matrix = d_matrix;
        a.dist = d_dist;
        a.stats = d_stats;
        a.scratch = d->scratch;
        a.npairs = npairs;
        a.nseqs = nseqs;
        a.max_len = max_len;
        a.ge = ge;
        a.gp1 = params->gap_pos1;
        a.gp2 = params->gap_pos2;
        k_pairwise_noalloc<<<(unsigned)grid, kNaWarpsPerBlock * 32, kNaRegionBytes * kNaWarpsPerBlock, s>>>(a);
        e = cudaGetLastError();
    }
    int status[3] = {0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(status, d->scratch + 4 * sizeof(unsigned long long), sizeof(status),
                            cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        fprintf(stderr, "cwgpu_align_pairs_noalloc: %s\n", cudaGetErrorString(e));
        return CWGPU_ERR_CUDA;
    }
    if (status[kNaStatusMatrix]) {
        fprintf(stderr, "cwgpu_align_pairs_noalloc: matrix entry outside the int16 profile range\n");
        return CWGPU_ERR_MATRIX;
    }
    if (status[kNaStatusInput])
        return na_reject("input rejected on the device (pair index, sequence offset, length above max_len, or "
                         "residue code)");
    if (status[kNaStatusLimit]) {
        fprintf(stderr, "cwgpu_align_pairs_noalloc: device-side limit reached (Myers-Miller stack depth)\n");
        return CWGPU_ERR_DEVICE;
    }
    return CWGPU_OK;
}
