// Host side of the C ABI (include/cwgpu.h): context, device layout, pair
// ordering, persistent graph-captured launch, plain one-launch-per-pair form.
//
// Device layout in HBM (all resident for the life of the context):
//   codes   int8 residues remapped to the K codes that occur: guard bytes, then
//           per sequence its codes and their reversed copy, each starting at a
//           16-byte boundary, then guard bytes (cwgpu_layout.h)
//   poffs   int64 start of each sequence's forward copy in `codes`
//   offs    int64 start of each sequence in the packed original codes (the
//           quick path uploads those itself)
//   lens    int32 sequence lengths n (getSeqLength)
//   nres    int32 residues that are not gapPos1/gapPos2 (len1/len2 of :100-127)
//   go_tab  int32 gap-open penalty per min(n, m) (FullPairwiseAlign.cpp:129-146)
//   matrix  int32[32*32] pairwise substitution matrix
//   scratch int2[slots][2][lmax+1]: per warp slot, the boundary rows of the
//           forward and reverse sweeps (HH/DD and RR/SS of diff()).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "cwgpu.h"
#include "cwgpu_context.h"
#include "cwgpu_device.cuh"
#include "cwgpu_layout.h"
#include "cwgpu_ranges.h"

namespace {

constexpr int kWarpsPerBlock = 4;  // warps (= concurrent pairs) per CTA
constexpr int kCounterWords = 8;   // cwgpu_context::d_counter

// RS = rows per lane of every sweep: cwgpu::kR for the long-pair kernel,
// cwgpu::kRShort for pairs whose first sequence has at most
// cwgpu_tuning::short_rows residues (128 by default: one 4-row stripe).
// Separate kernels keep the long-pair code exactly as tuned. Both are held to
// 5 CTAs (20 warps) per SM, i.e. 96 registers: measured faster than the 113
// registers and 4 CTAs per SM the compiler picks for the long-pair kernel
// unbounded (1000 x 1523 protein family, 200 sequences: 110.3 vs 114.7 ms).
template <int RS>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 5)
    k_pairwise(cwgpu::PairArgs g, long long single) {
    __shared__ int smat[CWGPU_NUMRES * CWGPU_NUMRES];
    extern __shared__ __align__(16) uint16_t region_all[];
    for (int i = threadIdx.x; i < CWGPU_NUMRES * CWGPU_NUMRES; i += blockDim.x) smat[i] = g.matrix[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const long long slot = (long long)blockIdx.x * wpb + warp;
    cwgpu::Env X;
    X.smat = smat;
    X.region = region_all + (size_t)warp * (cwgpu::warp_region_bytes(g.K) / sizeof(uint16_t));
    X.K = g.K;
    X.gp1 = g.gp1;
    X.gp2 = g.gp2;
    X.tiny_m = g.tiny_m;
    X.tiny_n = g.tiny_n;
    X.err = g.err;
    int2* bufA = g.scratch + (size_t)slot * 2 * (g.lmax + 1);
    int2* bufB = bufA + (g.lmax + 1);
    unsigned long long acc[3] = {0, 0, 0};
    if (single >= 0) {
        if (slot == 0) cwgpu::align_pair<RS>(g, single, X, bufA, bufB, acc);
    } else {
        for (;;) {
            unsigned long long k = 0;
            if (lane == 0) k = atomicAdd(g.counter, 1ULL);
            k = __shfl_sync(cwgpu::kFull, k, 0);
            if (k >= (unsigned long long)g.npairs) break;
            cwgpu::align_pair<RS>(g, (long long)g.order[k], X, bufA, bufB, acc);
        }
    }
    if (lane == 0 && g.cells && (acc[0] | acc[1] | acc[2])) {
        atomicAdd(g.cells + 0, acc[0]);
        atomicAdd(g.cells + 1, acc[1]);
        atomicAdd(g.cells + 2, acc[2]);
    }
}

}  // namespace

// struct cwgpu_context: cwgpu_context.h (shared with the quick-distance path).

struct cwgpu_plan {
    cwgpu_context* ctx = nullptr;
    int64_t npairs = 0;
    int32_t* d_pairs = nullptr;
    int32_t* d_order = nullptr;
    float* d_dist = nullptr;
    cwgpu_pair_stats* d_stats = nullptr;
    int64_t nlong = 0;  // order[0, nlong): long-pair kernel; order[nlong, npairs): short-pair kernel
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    cudaStream_t fork_stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    unsigned generation = 0;
};

namespace {

int fail(cwgpu_context* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_fail(cwgpu_context* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA, m);
}

#define CW_CUDA(ctx, call)                                      \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Grow-only device array: reallocates (contents lost) only when `need`
// elements exceed the capacity.
template <class T>
cudaError_t grow(T*& p, int64_t& cap, int64_t need) {
    if (need <= cap && p) return cudaSuccess;
    dfree(p);
    cap = 0;
    const int64_t n = std::max<int64_t>(need, 1);
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)n);
    if (e == cudaSuccess) cap = n;
    return e;
}

// Recomputes nres and the gap-open table after sequences or params changed.
int refresh_derived(cwgpu_context* ctx) {
    if (!ctx->derived_dirty) return CWGPU_OK;
    if (!ctx->has_params || !ctx->has_seqs) return fail(ctx, CWGPU_ERR_STATE, "params or sequences not set");
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<int32_t> nres(ctx->nseqs);
    for (int s = 0; s < ctx->nseqs; ++s) {
        int c = 0;
        const int8_t* p = ctx->host_codes.data() + ctx->offs[s];
        for (int i = 0; i < ctx->lens[s]; ++i)
            if (p[i] != ctx->params.gap_pos1 && p[i] != ctx->params.gap_pos2) ++c;
        nres[s] = c;
    }
    if (ctx->nseqs)
        CW_CUDA(ctx, cudaMemcpy(ctx->d_nres, nres.data(), sizeof(int32_t) * ctx->nseqs, cudaMemcpyHostToDevice));
    std::vector<int32_t> go(ctx->lmax + 1);
    for (int L = 1; L <= ctx->lmax; ++L) {  // L = 0 pairs never reach the penalties (:113-118)
        int32_t g = 0, e = 0;
        cwgpu_gap_penalties(&ctx->params, L, L, &g, &e);
        go[L] = g;
    }
    CW_CUDA(ctx, grow(ctx->d_go, ctx->cap_go, (int64_t)go.size()));
    CW_CUDA(ctx, cudaMemcpy(ctx->d_go, go.data(), sizeof(int32_t) * go.size(), cudaMemcpyHostToDevice));
    ctx->go_len = (int)go.size();
    // Matrix over the dense codes, row stride 32 (entries past K unused).
    if (ctx->has_matrix) {
        std::vector<int32_t> dm(CWGPU_NUMRES * CWGPU_NUMRES, 0);
        for (int a = 0; a < ctx->K; ++a)
            for (int b = 0; b < ctx->K; ++b)
                dm[a * CWGPU_NUMRES + b] = ctx->matrix[ctx->code_of[a] * CWGPU_NUMRES + ctx->code_of[b]];
        CW_CUDA(ctx, cudaMemcpy(ctx->d_matrix, dm.data(), sizeof(int32_t) * dm.size(), cudaMemcpyHostToDevice));
    }
    ctx->derived_dirty = false;
    ctx->generation++;
    return CWGPU_OK;
}

int gap_extend_of(const cwgpu_params& p) {
    int32_t g = 0, e = 0;
    cwgpu_gap_penalties(&p, 1, 1, &g, &e);
    return e;
}

size_t block_smem(int K, int warps) { return (size_t)cwgpu::warp_region_bytes(K) * warps; }

template <int RS>
int persistent_grid(cwgpu_context* ctx, int* grid) {
    int per_sm = 0;
    const size_t smem = block_smem(ctx->K, kWarpsPerBlock);
    CW_CUDA(ctx, cudaFuncSetAttribute(k_pairwise<RS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)block_smem(CWGPU_NUMRES, kWarpsPerBlock)));
    CW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairwise<RS>, kWarpsPerBlock * 32, smem));
    *grid = (per_sm < 1 ? 1 : per_sm) * ctx->sm_count;
    return CWGPU_OK;
}

bool has_short_seqs(const cwgpu_context* ctx) {
    for (int s = 0; s < ctx->nseqs; ++s)
        if (ctx->lens[s] <= ctx->short_rows) return true;
    return false;
}

// Persistent grids: as many CTAs as fit on every SM at once, per kernel. The
// scratch holds one (bufA, bufB) pair per warp slot of the long-pair grid,
// followed by the short-pair grid's slots when the set has short sequences
// (the two kernels of a plan can run at the same time).
int ensure_scratch(cwgpu_context* ctx) {
    if (ctx->grid == 0 || ctx->grid_K != ctx->K) {
        int rc = persistent_grid<cwgpu::kR>(ctx, &ctx->grid);
        if (!rc) rc = persistent_grid<cwgpu::kRShort>(ctx, &ctx->grid_short);
        if (rc) return rc;
        ctx->grid_K = ctx->K;
        ctx->scratch_bytes = 0;  // grid changed: resize below
        dfree(ctx->d_scratch);
    }
    const int64_t slots = (int64_t)(ctx->grid + (has_short_seqs(ctx) ? ctx->grid_short : 0)) * kWarpsPerBlock;
    const size_t need = (size_t)slots * 2 * (size_t)(ctx->lmax + 1) * sizeof(int2);
    if (need > ctx->scratch_bytes) {
        dfree(ctx->d_scratch);
        ctx->scratch_bytes = 0;
        CW_CUDA(ctx, cudaMalloc(&ctx->d_scratch, need));
        ctx->scratch_bytes = need;
        ctx->generation++;
    }
    return CWGPU_OK;
}

cwgpu::PairArgs make_args(cwgpu_context* ctx, const int32_t* d_pairs, const int32_t* d_order, int64_t npairs,
                          float* d_dist, cwgpu_pair_stats* d_stats) {
    cwgpu::PairArgs g;
    g.codes = ctx->d_codes;
    g.offs = ctx->d_poffs;
    g.lens = ctx->d_lens;
    g.nres = ctx->d_nres;
    g.pairs = d_pairs;
    g.order = d_order;
    g.go_table = ctx->d_go;
    g.matrix = ctx->d_matrix;
    g.dist = d_dist;
    g.stats = d_stats;
    g.scratch = ctx->d_scratch;
    g.counter = ctx->d_counter;
    g.cells = ctx->d_counter + 1;
    g.err = ctx->d_err;
    g.npairs = npairs;
    g.lmax = ctx->lmax;
    g.ge = gap_extend_of(ctx->params);
    const int gp1 = ctx->params.gap_pos1, gp2 = ctx->params.gap_pos2;
    g.gp1 = (gp1 >= 0 && gp1 < CWGPU_NUMRES) ? ctx->dense_of[gp1] : -1;
    g.gp2 = (gp2 >= 0 && gp2 < CWGPU_NUMRES) ? ctx->dense_of[gp2] : -1;
    g.K = ctx->K;
    g.tiny_m = ctx->tiny_m;
    g.tiny_n = ctx->tiny_n;
    return g;
}

int check_ready(cwgpu_context* ctx) {
    if (!ctx) return CWGPU_ERR_ARG;
    if (!ctx->has_matrix) return fail(ctx, CWGPU_ERR_STATE, "matrix not set");
    if (!ctx->has_params) return fail(ctx, CWGPU_ERR_STATE, "params not set");
    if (!ctx->has_seqs) return fail(ctx, CWGPU_ERR_STATE, "sequences not uploaded");
    int rc = refresh_derived(ctx);
    if (rc) return rc;
    return ensure_scratch(ctx);
}

int validate_pairs(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs) {
    if (npairs < 0 || (npairs > 0 && !pairs)) return fail(ctx, CWGPU_ERR_ARG, "bad pair list");
    if (npairs > CWGPU_MAX_PAIRS_PER_CALL)
        return fail(ctx, CWGPU_ERR_ARG, "more than CWGPU_MAX_PAIRS_PER_CALL pairs in one call");
    for (int64_t q = 0; q < npairs; ++q) {
        const int32_t a = pairs[2 * q], b = pairs[2 * q + 1];
        if (a < 0 || a >= ctx->nseqs || b < 0 || b >= ctx->nseqs)
            return fail(ctx, CWGPU_ERR_ARG, "pair index out of range");
    }
    return CWGPU_OK;
}

bool short_pair(const cwgpu_context* ctx, const int32_t* pairs, int64_t q) {
    return ctx->lens[pairs[2 * q]] <= ctx->short_rows;
}

// Pairs for the long-pair kernel first, then those for the short-pair kernel
// (*nlong of them are long); each part longest first (by n*m), so the tail of
// each persistent queue holds its shortest work. The order only balances the
// load, so a counting sort on a coarse key does: the top 12 bits of n*m as a
// float (exponent and 4 mantissa bits, 1/16 relative resolution), stable.
std::vector<int32_t> work_order(const cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, int64_t* nlong) {
    constexpr int kKeyBits = 12, kBuckets = 1 << kKeyBits;
    std::vector<uint16_t> key((size_t)npairs);
    std::vector<int64_t> start(2 * kBuckets + 1, 0);
    for (int64_t q = 0; q < npairs; ++q) {
        const float w = (float)((double)ctx->lens[pairs[2 * q]] * (double)ctx->lens[pairs[2 * q + 1]]);
        uint32_t bits;
        memcpy(&bits, &w, sizeof(bits));  // w >= 0: the bit pattern grows with w
        const int b = (int)(bits >> (31 - kKeyBits));
        const int k = (short_pair(ctx, pairs, q) ? kBuckets : 0) + (kBuckets - 1 - b);
        key[(size_t)q] = (uint16_t)k;
        ++start[k + 1];
    }
    for (int k = 0; k < 2 * kBuckets; ++k) start[k + 1] += start[k];
    *nlong = start[kBuckets];
    std::vector<int32_t> order((size_t)npairs);
    for (int64_t q = 0; q < npairs; ++q) order[(size_t)start[key[(size_t)q]]++] = (int32_t)q;
    return order;
}

// One persistent launch of k_pairwise<RS> over g's queue with a kernel-node
// priority (honoured by graphs instantiated with UseNodePriority).
template <int RS>
cudaError_t launch_persistent(const cwgpu::PairArgs& g, int max_grid, size_t smem, int priority, cudaStream_t s) {
    const int grid = (int)std::min<int64_t>(max_grid, (g.npairs + kWarpsPerBlock - 1) / kWarpsPerBlock);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kWarpsPerBlock * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = priority;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_pairwise<RS>, g, -1LL);
}

// The queue-counter reset and one persistent launch per kernel: long pairs
// on s, short pairs on s2 forked from s when both kinds are present (joined
// back into s), else on s. The short-pair kernel runs at lower priority so
// that its CTAs take the SM slots long-pair CTAs leave as the long queue
// drains. Works the same under stream capture.
cudaError_t enqueue_pairs(cwgpu_context* ctx, const cwgpu::PairArgs& gl, const cwgpu::PairArgs& gs, cudaStream_t s,
                          cudaStream_t s2, cudaEvent_t fork, cudaEvent_t join) {
    const size_t smem = block_smem(ctx->K, kWarpsPerBlock);
    const bool both = gl.npairs > 0 && gs.npairs > 0;
    cudaError_t e = cudaMemsetAsync(ctx->d_counter, 0, kCounterWords * sizeof(unsigned long long), s);
    cudaStream_t short_stream = s;
    if (e == cudaSuccess && both) {
        e = cudaEventRecord(fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, fork, 0);
        short_stream = s2;
    }
    if (e == cudaSuccess && gl.npairs > 0) e = launch_persistent<cwgpu::kR>(gl, ctx->grid, smem, ctx->prio_high, s);
    if (e == cudaSuccess && gs.npairs > 0)
        e = launch_persistent<cwgpu::kRShort>(gs, ctx->grid_short, smem, ctx->prio_low, short_stream);
    if (e == cudaSuccess && both) {
        e = cudaEventRecord(join, s2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    }
    return e;
}

// Arguments of the two kernels over one ordered pair list (long pairs first).
void split_args(cwgpu_context* ctx, const int32_t* d_pairs, const int32_t* d_order, int64_t npairs, int64_t nlong,
                float* d_dist, cwgpu_pair_stats* d_stats, cwgpu::PairArgs* gl, cwgpu::PairArgs* gs) {
    *gl = make_args(ctx, d_pairs, d_order, nlong, d_dist, d_stats);
    *gs = make_args(ctx, d_pairs, d_order + nlong, npairs - nlong, d_dist, d_stats);
    gs->counter = ctx->d_counter + 4;
    if (nlong > 0) gs->scratch += (size_t)ctx->grid * kWarpsPerBlock * 2 * (size_t)(ctx->lmax + 1);
}

int check_kernel_error(cwgpu_context* ctx) {
    int err = 0;
    CW_CUDA(ctx, cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        CW_CUDA(ctx, cudaMemset(ctx->d_err, 0, sizeof(int)));
        return fail(ctx, CWGPU_ERR_DEVICE, "kernel reported an internal limit (Myers-Miller stack depth)");
    }
    return CWGPU_OK;
}

}  // namespace

extern "C" {

const char* cwgpu_status_string(int status) {
    switch (status) {
        case CWGPU_OK: return "ok";
        case CWGPU_ERR_ARG: return "invalid argument";
        case CWGPU_ERR_CUDA: return "CUDA error";
        case CWGPU_ERR_OOM: return "out of device memory";
        case CWGPU_ERR_STATE: return "inputs not set";
        case CWGPU_ERR_RANGE: return "the range for pairwise alignment is incorrect";
        case CWGPU_ERR_TIMEOUT: return "bounded device wait timed out";
        case CWGPU_ERR_DEVICE: return "device-side limit exceeded";
        case CWGPU_ERR_MATRIX: return "matrix entry outside int16";
        case CWGPU_ERR_NOT_FOUND: return "unknown job";
        default: return "unknown status";
    }
}

const char* cwgpu_last_error(const cwgpu_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int cwgpu_gap_penalties(const cwgpu_params* p, int32_t n, int32_t m, int32_t* gap_open, int32_t* gap_extend) {
    if (!p || !gap_open || !gap_extend) return CWGPU_ERR_ARG;
    // FullPairwiseAlign.cpp:129-148 with the reference's operand types: float
    // members times int intScale stay float; the protein gap-open goes through
    // double because log() returns double.
    if (p->dna) {
        *gap_open = static_cast<int>(2 * p->pw_gap_open * p->int_scale * p->gap_open_scale);
        *gap_extend = static_cast<int>(p->pw_gap_extend * p->int_scale * p->gap_extend_scale);
    } else {
        const int mn = n < m ? n : m;
        if (p->mat_avg <= 0)
            *gap_open = 2 * static_cast<int>((p->pw_gap_open + log(static_cast<double>(mn))) * p->int_scale);
        else
            *gap_open = static_cast<int>(2 * p->mat_avg * (p->pw_gap_open + log(static_cast<double>(mn))) *
                                         p->gap_open_scale);
        *gap_extend = static_cast<int>(p->pw_gap_extend * p->int_scale);
    }
    return CWGPU_OK;
}

int64_t cwgpu_range_pair_count(int32_t nseqs, int32_t i_start, int32_t i_end, int32_t j_start, int32_t j_end) {
    int64_t c = 0;
    const int64_t hi = std::min(nseqs, j_end);
    for (int32_t si = std::max(0, i_start); si < nseqs && si < i_end; ++si) {
        const int64_t lo = cwgpu::range_col_lo(si, j_start);
        if (hi > lo) c += hi - lo;
    }
    return c;
}

int cwgpu_create(int device, cwgpu_context** out) {
    if (!out) return CWGPU_ERR_ARG;
    *out = nullptr;
    cwgpu_context* ctx = new (std::nothrow) cwgpu_context();
    if (!ctx) return CWGPU_ERR_OOM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&ctx->prio_low, &ctx->prio_high);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counter, kCounterWords * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_counter, 0, kCounterWords * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_matrix, sizeof(int32_t) * CWGPU_NUMRES * CWGPU_NUMRES);
    if (e != cudaSuccess) {
        cwgpu_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA;
    }
    memset(&ctx->params, 0, sizeof(ctx->params));
    *out = ctx;
    return CWGPU_OK;
}

void cwgpu_destroy(cwgpu_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    dfree(ctx->d_codes);
    dfree(ctx->d_poffs);
    dfree(ctx->d_offs);
    dfree(ctx->d_lens);
    dfree(ctx->d_nres);
    dfree(ctx->d_matrix);
    dfree(ctx->d_go);
    dfree(ctx->d_scratch);
    dfree(ctx->d_counter);
    dfree(ctx->d_err);
    dfree(ctx->d_pairs1);
    dfree(ctx->d_order1);
    dfree(ctx->d_dist1);
    dfree(ctx->d_stats1);
    if (ctx->stream_short) cudaStreamSynchronize(ctx->stream_short);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->stream_short) cudaStreamDestroy(ctx->stream_short);
    cwgpu_fast_release(ctx);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int cwgpu_set_matrix(cwgpu_context* ctx, const int32_t* matrix) {
    if (!ctx || !matrix) return CWGPU_ERR_ARG;
    for (int i = 0; i < CWGPU_NUMRES * CWGPU_NUMRES; ++i)
        if (matrix[i] < -32768 || matrix[i] > 32767)
            return fail(ctx, CWGPU_ERR_MATRIX, "matrix entry outside the int16 profile range");
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    memcpy(ctx->matrix, matrix, sizeof(ctx->matrix));
    ctx->has_matrix = true;
    ctx->derived_dirty = true;  // the device copy is remapped to the dense codes
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_set_params(cwgpu_context* ctx, const cwgpu_params* params) {
    if (!ctx || !params) return CWGPU_ERR_ARG;
    ctx->params = *params;
    ctx->has_params = true;
    ctx->derived_dirty = true;
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_upload_seqs(cwgpu_context* ctx, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                      const int32_t* lens) {
    if (!ctx || nseqs < 0 || (nseqs > 0 && (!offsets || !lens))) return CWGPU_ERR_ARG;
    std::vector<int64_t> doffs(nseqs);
    int64_t total = 0;
    int lmax = 0;
    for (int s = 0; s < nseqs; ++s) {
        if (lens[s] < 0 || lens[s] > CWGPU_MAX_SEQ_LEN)
            return fail(ctx, CWGPU_ERR_ARG, "sequence length outside [0, CWGPU_MAX_SEQ_LEN]");
        if (lens[s] > 0 && (!codes || offsets[s] < 0)) return fail(ctx, CWGPU_ERR_ARG, "bad sequence offset");
        for (int i = 0; i < lens[s]; ++i) {
            const int8_t c = codes[offsets[s] + i];
            if (c < 0 || c >= CWGPU_NUMRES) return fail(ctx, CWGPU_ERR_ARG, "residue code outside [0, 31]");
        }
        doffs[s] = total;
        total += (lens[s] + 15) & ~15;
        lmax = std::max(lmax, (int)lens[s]);
    }
    std::vector<int8_t> packed((size_t)std::max<int64_t>(total, 16), 0);
    for (int s = 0; s < nseqs; ++s)
        if (lens[s] > 0) memcpy(packed.data() + doffs[s], codes + offsets[s], lens[s]);
    // Remap residue codes to the dense alphabet of the codes that occur, so the
    // per-stripe score profile holds K rows instead of 32.
    bool present[CWGPU_NUMRES] = {false};
    for (int s = 0; s < nseqs; ++s)
        for (int i = 0; i < lens[s]; ++i) present[codes[offsets[s] + i]] = true;
    int K = 0, dense_of[CWGPU_NUMRES], code_of[CWGPU_NUMRES];
    for (int c = 0; c < CWGPU_NUMRES; ++c) {
        dense_of[c] = present[c] ? K : -1;
        if (present[c]) code_of[K++] = c;
    }
    if (K == 0) {  // no residues at all: keep one code so launches stay well-formed
        dense_of[0] = 0;
        code_of[0] = 0;
        K = 1;
    }
    std::vector<int8_t> dense;
    std::vector<int64_t> poffs;
    cwgpu::build_layout(
        nseqs, lens, [&](int s, int i) { return (int8_t)dense_of[codes[offsets[s] + i]]; }, dense, poffs);
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->has_seqs = false;
    CW_CUDA(ctx, grow(ctx->d_codes, ctx->cap_codes, (int64_t)dense.size()));
    if (nseqs > ctx->cap_seqs || !ctx->d_offs || !ctx->d_poffs || !ctx->d_lens || !ctx->d_nres) {
        int64_t c1 = 0, c2 = 0, c3 = 0, c4 = 0;
        dfree(ctx->d_offs);
        dfree(ctx->d_poffs);
        dfree(ctx->d_lens);
        dfree(ctx->d_nres);
        ctx->cap_seqs = 0;
        CW_CUDA(ctx, grow(ctx->d_offs, c1, nseqs));
        CW_CUDA(ctx, grow(ctx->d_poffs, c4, nseqs));
        CW_CUDA(ctx, grow(ctx->d_lens, c2, nseqs));
        CW_CUDA(ctx, grow(ctx->d_nres, c3, nseqs));
        ctx->cap_seqs = c1;
    }
    CW_CUDA(ctx, cudaMemcpy(ctx->d_codes, dense.data(), dense.size(), cudaMemcpyHostToDevice));
    if (nseqs) {
        CW_CUDA(ctx, cudaMemcpy(ctx->d_offs, doffs.data(), sizeof(int64_t) * nseqs, cudaMemcpyHostToDevice));
        CW_CUDA(ctx, cudaMemcpy(ctx->d_poffs, poffs.data(), sizeof(int64_t) * nseqs, cudaMemcpyHostToDevice));
        CW_CUDA(ctx, cudaMemcpy(ctx->d_lens, lens, sizeof(int32_t) * nseqs, cudaMemcpyHostToDevice));
    }
    ctx->nseqs = nseqs;
    ctx->lmax = lmax;
    ctx->lens.assign(lens, lens + nseqs);
    ctx->offs = doffs;
    ctx->host_codes.swap(packed);
    ctx->K = K;
    memcpy(ctx->dense_of, dense_of, sizeof(dense_of));
    memcpy(ctx->code_of, code_of, sizeof(code_of));
    ctx->has_seqs = true;
    ctx->derived_dirty = true;
    ctx->generation++;
    return CWGPU_OK;
}

// ---- plans: device-resident pair list + captured launch -------------------

int cwgpu_plan_create(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, cwgpu_plan** out) {
    if (!ctx || !out) return CWGPU_ERR_ARG;
    *out = nullptr;
    int rc = check_ready(ctx);
    if (rc) return rc;
    rc = validate_pairs(ctx, pairs, npairs);
    if (rc) return rc;
    cwgpu_plan* p = new (std::nothrow) cwgpu_plan();
    if (!p) return CWGPU_ERR_OOM;
    p->ctx = ctx;
    p->npairs = npairs;
    const size_t np = (size_t)std::max<int64_t>(npairs, 1);
    cudaError_t e = cudaMalloc(&p->d_pairs, sizeof(int32_t) * 2 * np);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_order, sizeof(int32_t) * np);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_dist, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_stats, sizeof(cwgpu_pair_stats) * np);
    if (e == cudaSuccess && npairs > 0) {
        std::vector<int32_t> order = work_order(ctx, pairs, npairs, &p->nlong);
        e = cudaMemcpy(p->d_pairs, pairs, sizeof(int32_t) * 2 * npairs, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(p->d_order, order.data(), sizeof(int32_t) * npairs, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        // Capture: reset the queue counters, then one persistent launch per kernel.
        cwgpu::PairArgs gl, gs;
        split_args(ctx, p->d_pairs, p->d_order, npairs, p->nlong, p->d_dist, p->d_stats, &gl, &gs);
        const bool both = gl.npairs > 0 && gs.npairs > 0;
        e = cudaStreamCreateWithFlags(&p->graph_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess && both) e = cudaStreamCreateWithFlags(&p->fork_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess && both) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
        if (e == cudaSuccess && both) e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(p->graph_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t ce = enqueue_pairs(ctx, gl, gs, p->graph_stream, p->fork_stream, p->fork, p->join);
            e = cudaStreamEndCapture(p->graph_stream, &p->graph);
            if (e == cudaSuccess) e = ce;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiateWithFlags(&p->exec, p->graph, cudaGraphInstantiateFlagUseNodePriority);
    }
    if (e != cudaSuccess) {
        cwgpu_plan_destroy(p);
        return cuda_fail(ctx, e, "cwgpu_plan_create");
    }
    p->generation = ctx->generation;
    *out = p;
    return CWGPU_OK;
}

int cwgpu_plan_launch(cwgpu_plan* p, void* stream) {
    if (!p) return CWGPU_ERR_ARG;
    cwgpu_context* ctx = p->ctx;
    if (p->generation != ctx->generation || ctx->derived_dirty)
        return fail(ctx, CWGPU_ERR_STATE, "plan is stale: inputs changed after cwgpu_plan_create");
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    CW_CUDA(ctx, cudaGraphLaunch(p->exec, s));
    return CWGPU_OK;
}

int cwgpu_plan_results(cwgpu_plan* p, float* dist_out, cwgpu_pair_stats* stats_out) {
    if (!p) return CWGPU_ERR_ARG;
    cwgpu_context* ctx = p->ctx;
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    CW_CUDA(ctx, cudaDeviceSynchronize());
    int rc = check_kernel_error(ctx);
    if (rc) return rc;
    if (p->npairs > 0 && dist_out)
        CW_CUDA(ctx, cudaMemcpy(dist_out, p->d_dist, sizeof(float) * p->npairs, cudaMemcpyDeviceToHost));
    if (p->npairs > 0 && stats_out)
        CW_CUDA(ctx, cudaMemcpy(stats_out, p->d_stats, sizeof(cwgpu_pair_stats) * p->npairs, cudaMemcpyDeviceToHost));
    return CWGPU_OK;
}

void* cwgpu_plan_device_dist(cwgpu_plan* p) { return p ? (void*)p->d_dist : nullptr; }

int cwgpu_plan_cell_counts(cwgpu_plan* p, int64_t* counts) {
    if (!p || !counts) return CWGPU_ERR_ARG;
    cwgpu_context* ctx = p->ctx;
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    CW_CUDA(ctx, cudaDeviceSynchronize());
    unsigned long long c[3];
    CW_CUDA(ctx, cudaMemcpy(c, ctx->d_counter + 1, sizeof(c), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 3; ++i) counts[i] = (int64_t)c[i];
    return CWGPU_OK;
}

int cwgpu_plan_kernel_count(const cwgpu_plan* p) {
    if (!p) return 0;
    return (p->nlong > 0 ? 1 : 0) + (p->npairs > p->nlong ? 1 : 0);
}

void cwgpu_plan_destroy(cwgpu_plan* p) {
    if (!p) return;
    if (p->ctx) cudaSetDevice(p->ctx->device);
    if (p->graph_stream) cudaStreamSynchronize(p->graph_stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->graph_stream) cudaStreamDestroy(p->graph_stream);
    if (p->fork_stream) cudaStreamDestroy(p->fork_stream);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->join) cudaEventDestroy(p->join);
    dfree(p->d_pairs);
    dfree(p->d_order);
    dfree(p->d_dist);
    dfree(p->d_stats);
    delete p;
}

// One-shot form: the same launches as a plan, enqueued directly (no graph to
// build for a single run) on the context's streams and grow-only arrays.
int cwgpu_align_pairs(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, float* dist_out,
                      cwgpu_pair_stats* stats_out) {
    if (!ctx || (npairs > 0 && !dist_out)) return CWGPU_ERR_ARG;
    int rc = check_ready(ctx);
    if (rc) return rc;
    rc = validate_pairs(ctx, pairs, npairs);
    if (rc) return rc;
    if (npairs == 0) return CWGPU_OK;
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (npairs > ctx->cap_pairs1) {
        int64_t c1 = 0, c2 = 0, c3 = 0, c4 = 0;
        ctx->cap_pairs1 = 0;
        CW_CUDA(ctx, grow(ctx->d_pairs1, c1, 2 * npairs));
        CW_CUDA(ctx, grow(ctx->d_order1, c2, npairs));
        CW_CUDA(ctx, grow(ctx->d_dist1, c3, npairs));
        CW_CUDA(ctx, grow(ctx->d_stats1, c4, npairs));
        ctx->cap_pairs1 = npairs;
    }
    // Created on first use; each handle on its own, so a call after a failed
    // creation retries what is missing.
    if (!ctx->stream_short) CW_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream_short, cudaStreamNonBlocking));
    if (!ctx->ev_fork) CW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    if (!ctx->ev_join) CW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    int64_t nlong = 0;
    const std::vector<int32_t> order = work_order(ctx, pairs, npairs, &nlong);
    cudaStream_t s = ctx->stream;
    CW_CUDA(ctx, cudaMemcpyAsync(ctx->d_pairs1, pairs, sizeof(int32_t) * 2 * npairs, cudaMemcpyHostToDevice, s));
    CW_CUDA(ctx, cudaMemcpyAsync(ctx->d_order1, order.data(), sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, s));
    cwgpu::PairArgs gl, gs;
    split_args(ctx, ctx->d_pairs1, ctx->d_order1, npairs, nlong, ctx->d_dist1, stats_out ? ctx->d_stats1 : nullptr,
               &gl, &gs);
    CW_CUDA(ctx, enqueue_pairs(ctx, gl, gs, s, ctx->stream_short, ctx->ev_fork, ctx->ev_join));
    CW_CUDA(ctx, cudaMemcpyAsync(dist_out, ctx->d_dist1, sizeof(float) * npairs, cudaMemcpyDeviceToHost, s));
    if (stats_out)
        CW_CUDA(ctx, cudaMemcpyAsync(stats_out, ctx->d_stats1, sizeof(cwgpu_pair_stats) * npairs,
                                     cudaMemcpyDeviceToHost, s));
    CW_CUDA(ctx, cudaStreamSynchronize(s));
    return check_kernel_error(ctx);
}

int cwgpu_align_pairs_plain(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, float* dist_out,
                            cwgpu_pair_stats* stats_out) {
    if (!ctx || (npairs > 0 && !dist_out)) return CWGPU_ERR_ARG;
    int rc = check_ready(ctx);
    if (rc) return rc;
    rc = validate_pairs(ctx, pairs, npairs);
    if (rc) return rc;
    if (npairs == 0) return CWGPU_OK;
    int32_t* d_pairs = nullptr;
    float* d_dist = nullptr;
    cwgpu_pair_stats* d_stats = nullptr;
    cudaError_t e = cudaMalloc(&d_pairs, sizeof(int32_t) * 2 * npairs);
    if (e == cudaSuccess) e = cudaMalloc(&d_dist, sizeof(float) * npairs);
    if (e == cudaSuccess) e = cudaMalloc(&d_stats, sizeof(cwgpu_pair_stats) * npairs);
    if (e == cudaSuccess) e = cudaMemcpy(d_pairs, pairs, sizeof(int32_t) * 2 * npairs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_counter, 0, kCounterWords * sizeof(unsigned long long), ctx->stream);
    if (e == cudaSuccess) {
        cwgpu::PairArgs g = make_args(ctx, d_pairs, nullptr, npairs, d_dist, d_stats);
        for (int64_t q = 0; q < npairs && e == cudaSuccess; ++q) {
            if (short_pair(ctx, pairs, q))
                k_pairwise<cwgpu::kRShort><<<1, 32, block_smem(ctx->K, 1), ctx->stream>>>(g, (long long)q);
            else
                k_pairwise<cwgpu::kR><<<1, 32, block_smem(ctx->K, 1), ctx->stream>>>(g, (long long)q);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) {
        rc = check_kernel_error(ctx);
        if (!rc) {
            e = cudaMemcpy(dist_out, d_dist, sizeof(float) * npairs, cudaMemcpyDeviceToHost);
            if (e == cudaSuccess && stats_out)
                e = cudaMemcpy(stats_out, d_stats, sizeof(cwgpu_pair_stats) * npairs, cudaMemcpyDeviceToHost);
        }
    }
    dfree(d_pairs);
    dfree(d_dist);
    dfree(d_stats);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cwgpu_align_pairs_plain");
    return rc;
}

int cwgpu_pairwise_align(cwgpu_context* ctx, int32_t i_start, int32_t i_end, int32_t j_start, int32_t j_end,
                         double* elements, int32_t dist_size, cwgpu_pair_stats* stats_out) {
    if (!ctx || !elements) return CWGPU_ERR_ARG;
    if (!ctx->has_seqs) return fail(ctx, CWGPU_ERR_STATE, "sequences not uploaded");
    // FullPairwiseAlign.cpp:47-52
    if (dist_size != ctx->nseqs + 1) return fail(ctx, CWGPU_ERR_ARG, "The distance matrix is not the right size!");
    // FullPairwiseAlign.cpp:53-58
    if (i_start < 0 || i_end < i_start || j_start < 0 || j_end < j_start)
        return fail(ctx, CWGPU_ERR_RANGE, "The range for pairwise Alignment is incorrect.");
    const int n = ctx->nseqs;
    if (n == 0) return CWGPU_OK;  // :63-66
    std::vector<float> dist;
    return cwgpu::for_range_blocks(
        n, i_start, i_end, j_start, j_end, cwgpu::kRangeBlockPairs, [&](const int32_t* pairs, int64_t np, int64_t first) {
            dist.resize((size_t)std::max<int64_t>(np, 1));
            const int rc = cwgpu_align_pairs(ctx, pairs, np, dist.data(), stats_out ? stats_out + first : nullptr);
            if (rc) return rc;
            for (int64_t q = 0; q < np; ++q) {
                // SymMatrix::getIndex for (si+1, sj+1), si < sj: ((_j*(_j+1))>>1) + _i.
                const int64_t i = pairs[2 * q], j = pairs[2 * q + 1];
                elements[((j * (j + 1)) >> 1) + i] = (double)dist[q];
            }
            return (int)CWGPU_OK;
        });
}

int cwgpu_set_tuning(cwgpu_context* ctx, const cwgpu_tuning* tuning) {
    if (!ctx || !tuning) return CWGPU_ERR_ARG;
    if (tuning->tiny_m < 0 || tuning->tiny_m > 256 || tuning->tiny_n < 0 || tuning->tiny_n > cwgpu::kTinyMaxN ||
        tuning->short_rows < 0 || tuning->short_rows > CWGPU_MAX_SEQ_LEN)
        return fail(ctx, CWGPU_ERR_ARG, "tiny_m must be in [0, 256], tiny_n in [0, 16], short_rows in [0, 65535]");
    ctx->tiny_m = tuning->tiny_m;
    ctx->tiny_n = tuning->tiny_n;
    ctx->short_rows = tuning->short_rows;
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_get_tuning(const cwgpu_context* ctx, cwgpu_tuning* tuning) {
    if (!ctx || !tuning) return CWGPU_ERR_ARG;
    tuning->tiny_m = ctx->tiny_m;
    tuning->tiny_n = ctx->tiny_n;
    tuning->short_rows = ctx->short_rows;
    return CWGPU_OK;
}

int cwgpu_synchronize(cwgpu_context* ctx) {
    if (!ctx) return CWGPU_ERR_ARG;
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    CW_CUDA(ctx, cudaDeviceSynchronize());
    return check_kernel_error(ctx);
}

}  // extern "C"
