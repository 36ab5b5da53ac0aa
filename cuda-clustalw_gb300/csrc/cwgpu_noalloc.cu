// Allocation-free entry point: cwgpu_align_pairs_noalloc.
//
// Some callers cannot call cudaMalloc: code running inside a host framework
// that owns all device memory through its own pool (and forbids side
// allocations), processes with a fixed device-memory budget reserved at
// start-up, or callers between a memory-pool reservation and its use. They
// can still hand over device buffers they already own. This entry point runs
// the same pair kernel as cwgpu_align_pairs, but every byte of working memory
// it needs (per-warp boundary rows, the queue head, the cell counters, the
// status word and the gap-open table) lives in one file-scope static device
// array, g_noalloc_scratch, of CWGPU_NOALLOC_SCRATCH_BYTES (16 MiB). Every GPU that
// loads this library holds that array until the process exits.
//
// In host code g_noalloc_scratch names a host-side stand-in, not a device
// address; a kernel given it would fault or read the wrong memory. So the
// first call on each device, with that device current, looks the address up
// with cudaGetSymbolAddress (and the occupancy of the kernel) and caches both
// per device. That first call should come before any stream capture.
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

namespace {

constexpr int kNaWarpsPerBlock = 4;
constexpr size_t kNaProfBytesPerWarp = 32 * 32 * 4 * sizeof(uint16_t);
constexpr size_t kNaScratchBytes = (size_t)CWGPU_NOALLOC_SCRATCH_BYTES;
constexpr size_t kNaCtrlBytes = 256;  // [0] queue head, [1..3] cell counts, [4] status word
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

// One pair (FullPairwiseAlign.cpp:112-183) with device-side input checks: a
// pair index, a length above max_len or a residue code outside [0, 31] sets
// the status word and the pair is skipped. The residue counts len1/len2 of
// :100-127 are counted here instead of being uploaded.
template <int R>
__device__ void na_align_pair(const NaArgs& a, long long q, uint16_t* prof, const int* smat, int2* bufA,
                              int2* bufB, unsigned long long (&acc)[3]) {
    const int lane = threadIdx.x & 31;
    unsigned long long* ctrl = reinterpret_cast<unsigned long long*>(a.scratch);
    int* status = reinterpret_cast<int*>(ctrl + 4);
    const int32_t* go_table = reinterpret_cast<const int32_t*>(a.scratch + kNaCtrlBytes);
    const int si = a.pairs[2 * q], sj = a.pairs[2 * q + 1];
    if (si < 0 || si >= a.nseqs || sj < 0 || sj >= a.nseqs) {
        if (lane == 0) atomicExch(status, 1);
        return;
    }
    const int n = a.lens[si], m = a.lens[sj];
    if (n < 0 || m < 0 || n > a.max_len || m > a.max_len) {
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
    const int go = go_table[min(n, m)];
    const int ge = a.ge;
    cwgpu_pair_stats st = {0, 0, 0, 0, 0, 0, 0, 0};
    float dist = 1.0f;
    if (n > 0 && m > 0) {
        cwgpu::Task t;
        t.rseq = s1;
        t.rdir = 1;
        t.cseq = s2;
        t.cdir = 1;
        t.rows = n;
        t.cols = m;
        t.ht0 = 0;
        t.hts = 0;
        t.eo = go;
        t.hl0 = 0;
        t.hls = 0;
        t.fo = go;
        t.buf = bufA;
        cwgpu::Best fb;
        cwgpu::sweep<R, 32, cwgpu::MODE_LOCAL_FWD>(t, go, ge, 0, prof, smat, fb);
        const int max_score = fb.val;
        const int se1 = max_score > 0 ? (int)(fb.key >> 16) + 1 : 0;
        const int se2 = max_score > 0 ? (int)(fb.key & 0xffffu) : 0;
        __syncwarp();
        int sb1 = 1, sb2 = 1;
        if (se1 > 0) {
            cwgpu::Task r;
            r.rseq = s1 + se1 - 1;
            r.rdir = -1;
            r.cseq = s2 + se2 - 1;
            r.cdir = -1;
            r.rows = se1;
            r.cols = se2;
            r.ht0 = -1;
            r.hts = 0;
            r.eo = 0;
            r.hl0 = -1;
            r.hls = 0;
            r.fo = 0;
            r.buf = bufA;
            cwgpu::Best rb;
            cwgpu::sweep<R, 32, cwgpu::MODE_LOCAL_REV>(r, go, ge, max_score, prof, smat, rb);
            if (rb.val > 0) {
                sb1 = se1 - (int)(rb.key >> 16);
                sb2 = se2 - (int)(rb.key & 0xffffu) + 1;
            }
            if (rb.val >= max_score)
                acc[1] += (unsigned long long)(se1 - sb1) * se2 + (unsigned long long)(se2 - sb2 + 1);
            else
                acc[1] += (unsigned long long)se1 * se2;
            __syncwarp();
        }
        acc[0] += (unsigned long long)n * m;
        int mm = 0, ident = 0, matches = 0;
        long long dcells = 0;
        cwgpu::mm_align<R>(s1, s2, sb1 - 1, sb2 - 1, se1 - sb1 + 1, se2 - sb2 + 1, go, ge, a.gp1, a.gp2, bufA,
                           bufB, prof, smat, status, mm, ident, matches, dcells);
        acc[2] += (unsigned long long)dcells;
        float mmv = (float)(100 * ident);
        if (len1 == 0 || len2 == 0)
            mmv = 0.0f;
        else
            mmv = __fdiv_rn(mmv, (float)min(len1, len2));
        dist = __fdiv_rn(__fsub_rn(100.0f, mmv), 100.0f);
        st.fwd_score = max_score;
        st.se1 = se1;
        st.se2 = se2;
        st.sb1 = sb1;
        st.sb2 = sb2;
        st.mm_score = mm;
        st.n_ident = ident;
        st.n_match = matches;
    }
    if (lane == 0) {
        a.dist[q] = dist;
        if (a.stats) a.stats[q] = st;
    }
}

__global__ void __launch_bounds__(kNaWarpsPerBlock * 32) k_pairwise_noalloc(NaArgs a) {
    __shared__ int smat[CWGPU_NUMRES * CWGPU_NUMRES];
    __shared__ __align__(16) uint16_t prof_all[kNaWarpsPerBlock * kNaProfBytesPerWarp / sizeof(uint16_t)];
    for (int i = threadIdx.x; i < CWGPU_NUMRES * CWGPU_NUMRES; i += blockDim.x) smat[i] = a.matrix[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * kNaWarpsPerBlock + warp;
    uint16_t* prof = prof_all + (size_t)warp * (kNaProfBytesPerWarp / sizeof(uint16_t));
    int2* rows = reinterpret_cast<int2*>(a.scratch + kNaRowsOffset);
    int2* bufA = rows + (size_t)slot * 2 * (a.max_len + 1);
    int2* bufB = bufA + (a.max_len + 1);
    unsigned long long* ctrl = reinterpret_cast<unsigned long long*>(a.scratch);
    unsigned long long acc[3] = {0, 0, 0};
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(ctrl, 1ULL);
        k = __shfl_sync(cwgpu::kFull, k, 0);
        if (k >= (unsigned long long)a.npairs) break;
        na_align_pair<4>(a, (long long)k, prof, smat, bufA, bufB, acc);
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
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairwise_noalloc, kNaWarpsPerBlock * 32, 0);
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

    const size_t row_bytes = 2 * (size_t)(max_len + 1) * sizeof(int2);
    const long long slots = (long long)((kNaScratchBytes - kNaRowsOffset) / row_bytes);
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
        k_pairwise_noalloc<<<(unsigned)grid, kNaWarpsPerBlock * 32, 0, s>>>(a);
        e = cudaGetLastError();
    }
    int status = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&status, d->scratch + 4 * sizeof(unsigned long long), sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        fprintf(stderr, "cwgpu_align_pairs_noalloc: %s\n", cudaGetErrorString(e));
        return CWGPU_ERR_CUDA;
    }
    if (status) return na_reject("input rejected on the device (pair index, length above max_len, or residue code)");
    return CWGPU_OK;
}
