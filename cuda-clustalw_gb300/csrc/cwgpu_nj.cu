// cwgpu_nj.cu - guide tree by neighbour joining on sm_103a.
//
// Computes what clustalw::NJTree::generateTree does
// (CPU/clustalw-2.0.11/src/tree/NJTree.cpp:161-748), bit-identically: the
// same double rounding in every sum, the same criterion
//   total = fnseqs2 * d(ii,jj) + 2 * sumd - diq - djq      (NJTree.cpp:331-376)
// minimised with the first-minimum rule of the reference's scan (jj ascending,
// ii ascending, strict <), the same branch lengths and the same in-place
// updates of the packed DistMatrix.
//
// One cooperative persistent kernel runs all n-3 cycles. Each cycle is
//   search   every CTA scans its share of the packed lower triangle (row jj is
//            contiguous, so the reference's scan order is memory order) and
//            keeps the lexicographic minimum of (total, element index);
//   barrier  the per-CTA minima are published;
//   update   CTA 0 picks the join, writes branch lengths and the treeDesc
//            row, updates the row sums and the joined row/column of the
//            matrix, and forms the next cycle's sums; the sequential sums of
//            the reference are replayed in the reference's order;
//   barrier  the new sums and matrix entries are published.
// The hand-offs between CTA 0 and the other CTAs are bounded spins: if one runs
// out the kernel records a timeout status and every CTA returns. Comparisons
// of doubles use order-preserving integer keys: on this part every double
// instruction, a compare included, occupies a sub-partition's double unit for
// about 70 cycles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cwgpu_nj.h"

namespace cwnj {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kPer = 8;             // elements per lane per work item
constexpr int kChunk = 32 * kPer;   // elements of one row per work item
constexpr unsigned long long kBarrierTimeoutNs = 4000000000ull;
constexpr unsigned kSpinLimit = 1u << 27;
constexpr int kMaxGrid = 256;       // CTAs (one per SM)

enum { ST_OK = 0, ST_TIMEOUT = 1, ST_NOJOIN = 2, ST_INTERNAL = 3 };

struct Args {
    double* d;  // packed matrix, joined in place
    int n;
    double* left;
    double* right;
    int* desc;   // (n+1) x (n+1)
    int* joins;  // 2*(n-3) or null
    double* sumCols;
    double* sumRows;
    double* av;
    double* join;
    double* r;  // sumCols + sumRows of the valid nodes, for the search
    unsigned char* valid;
    int* rep;  // cycle that last formed the cluster node i stands for (0: leaf)
    int* vlist;  // two buffers of n + 1 entries: the valid nodes in ascending order
    unsigned long long* cand_k;  // order key of the criterion
    long long* cand_idx;
    int2* cand_ij;
    double* cand_d;
    double* scal;  // [0] 2*sumd, [1] fnseqs2, [2] fnseqs
    const int2* items;
    int n_items;
    unsigned* arrive;   // candidates written, summed over cycles (other CTAs)
    unsigned* release;  // cycles CTA 0 has published
    int* status;
    bool node_shared;   // CTA 0 keeps the per-node arrays in shared memory
    unsigned long long wait_ns;  // limit of every wait between CTAs
};

__device__ __forceinline__ size_t tri(int a) { return ((size_t)a * (size_t)(a + 1)) >> 1; }
// SymMatrix::getIndex (general/SymMatrix.h:166-197) for 1-based i, j.
__device__ __forceinline__ size_t sym(int i, int j) {
    return i < j ? tri(j - 1) + (size_t)(i - 1) : tri(i - 1) + (size_t)(j - 1);
}

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_status(const int* p) { return *(const volatile int*)p; }

// Order-preserving key of a double: key(a) < key(b) exactly when a < b, with
// -0.0 and +0.0 equal and NaN above everything (never a minimum).
__device__ __forceinline__ unsigned long long okey(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0) return 0x8000000000000000ull;
    if ((b & 0x7FF0000000000000ull) == 0x7FF0000000000000ull && (b & ((1ull << 52) - 1))) return ~0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// x * 0.5 and x * 2.0 without a double instruction where the result is a
// normal number (then both are exact: only the exponent changes).
__device__ __forceinline__ double half_of(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    if (e > 1u && e < 2047u) return __longlong_as_double((long long)(b - (1ull << 52)));
    return __dmul_rn(x, 0.5);
}
__device__ __forceinline__ double twice(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    if (e >= 1u && e < 2046u) return __longlong_as_double((long long)(b + (1ull << 52)));
    return __dmul_rn(2.0, x);
}

// (key, idx) lexicographic order; idx -1 marks "no candidate" at the cut-off
// tmin, which any real candidate (t < tmin) beats.
__device__ __forceinline__ bool better(unsigned long long k, long long i, unsigned long long bk, long long bi) {
    return k < bk || (k == bk && i < bi);
}

// ---------------------------------------------------------------------------
// Exact replay of a sequentially rounded double sum by one warp.
//
// The reference adds its row sums one term at a time, each addition rounded to
// nearest-even. A dependent double add costs about 70 cycles on this part, so
// a chain of n adds per cycle would dominate the whole tree. The warp instead
// takes 32 terms at a time. While the running sum s = m * 2^q (m a 53-bit
// integer) stays in one binade and a term x >= 0, the rounded step adds
// a = floor(x / 2^q) plus a rounding bit: 1 above half an ulp, 0 below, and at
// exactly half (a tie) the bit that makes m + a + bit even. So a step is a
// function of the parity of m alone, m -> m + delta(m & 1), and such functions
// compose: a warp reduction over lanes in order (or a scan, when a step must
// be located) gives the block's total from the incoming parity. Without ties
// delta does not depend on the parity and a plain integer reduction suffices.
// The first lane whose step leaves the binade, or whose term is negative,
// non-finite or of a higher binade, is done with one hardware add (which rounds
// exactly as the reference's add) and the warp resumes after it. Terms of +0.0
// (skipped nodes) change nothing: adding +0.0 to a sum that is never -0.0.
// ---------------------------------------------------------------------------
constexpr unsigned long long kFracMask = (1ull << 52) - 1;
constexpr unsigned long long kTwo52 = 1ull << 52, kTwo53 = 1ull << 53;

// (d0, d1): the step's increment of m when m is even / odd. compose(L, R) is
// "L, then R".
__device__ __forceinline__ void compose(unsigned long long& l0, unsigned long long& l1, unsigned long long r0,
                                        unsigned long long r1) {
    const unsigned long long o0 = l0 + ((l0 & 1ull) ? r1 : r0);
    const unsigned long long o1 = l1 + ((l1 & 1ull) ? r0 : r1);
    l0 = o0;
    l1 = o1;
}

__device__ __forceinline__ double assemble(int Es, unsigned long long m) {
    return __longlong_as_double((long long)(((unsigned long long)Es << 52) | (m & kFracMask)));
}

// Adds the 32 lanes' terms xv (lane order) to the warp-uniform sum s.
__device__ __forceinline__ double block_add(double s, double xv, int lane) {
    const unsigned long long xb = (unsigned long long)__double_as_longlong(xv);
    const int Ex = (int)(xb >> 52);  // sign bit included: negative terms read >= 2048
    int start = 0;
    while (true) {
        const unsigned long long sb = (unsigned long long)__double_as_longlong(s);
        const int Es = (int)(sb >> 52);
        const bool s_fast = Es >= 1 && Es <= 2046;  // positive normal
        bool bad = false, tie = false;
        unsigned long long a = 0, ru = 0;
        if (lane >= start && xb != 0) {
            if (!s_fast || Ex >= 2047) {
                bad = true;
            } else {
                const int Exe = Ex == 0 ? 1 : Ex;
                const unsigned long long mant = Ex == 0 ? (xb & kFracMask) : ((xb & kFracMask) | kTwo52);
                const int d = Es - Exe;
                if (d < 0) {
                    bad = true;
                } else if (d == 0) {
                    a = mant;
                } else if (d < 54) {
                    const unsigned long long r = mant & ((1ull << d) - 1);
                    const unsigned long long half = 1ull << (d - 1);
                    tie = r == half;
                    ru = r > half ? 1ull : 0ull;
                    a = mant >> d;
                }  // d >= 54: the term is below half an ulp of s
            }
        }
        const unsigned badmask = __ballot_sync(0xffffffffu, bad);
        if (!s_fast) {
            if (badmask == 0) return s;  // only +0.0 terms remain
            const int k = __ffs(badmask) - 1;
            s = __dadd_rn(s, __shfl_sync(0xffffffffu, xv, k));
            start = k + 1;
            if (start >= 32) return s;
            continue;
        }
        const unsigned long long m = (sb & kFracMask) | kTwo52;
        const unsigned tiemask = __ballot_sync(0xffffffffu, tie);
        // Increments for an even / odd incoming m.
        unsigned long long d0 = a + (tie ? (a & 1ull) : ru);
        unsigned long long d1 = a + (tie ? ((a & 1ull) ^ 1ull) : ru);
        if (badmask == 0) {
            unsigned long long tot;
            if (tiemask == 0) {
                tot = ((unsigned long long)__reduce_add_sync(0xffffffffu, (unsigned)(d0 >> 26)) << 26) +
                      (unsigned long long)__reduce_add_sync(0xffffffffu, (unsigned)(d0 & ((1u << 26) - 1)));
            } else {
                unsigned long long t0 = d0, t1 = d1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long r0 = __shfl_down_sync(0xffffffffu, t0, o);
                    const unsigned long long r1 = __shfl_down_sync(0xffffffffu, t1, o);
                    if (lane + o < 32) compose(t0, t1, r0, r1);
                }
                tot = __shfl_sync(0xffffffffu, (m & 1ull) ? t1 : t0, 0);
            }
            if (m + tot < kTwo53) return assemble(Es, m + tot);
        }
        // Locate the first lane that cannot take the step in integers: a bad
        // term or the first step whose rounded sum reaches the next binade.
        unsigned long long i0 = d0, i1 = d1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long l0 = __shfl_up_sync(0xffffffffu, i0, o);
            unsigned long long l1 = __shfl_up_sync(0xffffffffu, i1, o);
            if (lane >= o) {
                compose(l0, l1, i0, i1);
                i0 = l0;
                i1 = l1;
            }
        }
        const unsigned long long mk = m + ((m & 1ull) ? i1 : i0);  // m after this lane's step
        const unsigned over = __ballot_sync(0xffffffffu, lane >= start && mk >= kTwo53);
        const int k = __ffs(badmask | over) - 1;
        if (k < 0) {  // cannot happen: the step above failed for some lane; add the rest in hardware
            for (int l = start; l < 32; ++l) s = __dadd_rn(s, __shfl_sync(0xffffffffu, xv, l));
            return s;
        }
        const unsigned long long prev = __shfl_sync(0xffffffffu, mk, k > 0 ? k - 1 : 0);
        s = assemble(Es, k > 0 ? prev : m);
        s = __dadd_rn(s, __shfl_sync(0xffffffffu, xv, k));
        start = k + 1;
        if (start >= 32) return s;
    }
}

// s + get(lo) + ... + get(hi-1), each addition rounded as the reference's
// sequential loop rounds it; get(j) returns +0.0 for skipped terms. Called by
// a whole warp, 32 terms per step; loads run kDepth steps ahead of the adds.
template <class Get>
__device__ double warp_seq_sum(const Get& get, int lo, int hi, double s) {
    constexpr int kDepth = 4;
    const int lane = threadIdx.x & 31;
    double buf[kDepth];
#pragma unroll
    for (int p = 0; p < kDepth; ++p) {
        const int j = lo + 32 * p + lane;
        buf[p] = j < hi ? get(j) : 0.0;
    }
    for (int base = lo; base < hi; base += 32 * kDepth) {
#pragma unroll
        for (int p = 0; p < kDepth; ++p) {
            const double xv = buf[p];
            const int jn = base + 32 * (p + kDepth) + lane;
            buf[p] = jn < hi ? get(jn) : 0.0;
            if (base + 32 * p < hi) s = block_add(s, xv, lane);
        }
    }
    return s;
}

struct ValidTerms {  // x[j] where node j is still valid (generic loads: shared or global)
    const double* x;
    const unsigned char* valid;
    __device__ double operator()(int j) const { return valid[j] ? x[j] : 0.0; }
};
struct PlainTerms {
    const double* x;
    __device__ double operator()(int j) const { return __ldg(x + j); }
};
struct RowTerms {  // d(i, j) for i < j: row j of the packed triangle
    const double* row;
    __device__ double operator()(int i) const { return __ldcg(row + (i - 1)); }
};
struct ListTerms {  // x[list[k]]: the terms of the valid nodes only, in ascending node order
    const double* x;
    const int* list;
    __device__ double operator()(int k) const { return x[list[k]]; }
};
struct ListSkipTerms {  // the same with entry `skip` (a node that just left) read as +0.0
    const double* x;
    const int* list;
    int skip;
    __device__ double operator()(int k) const { return k == skip ? 0.0 : x[list[k]]; }
};
struct ColTerms {  // d(j, i) for i > j: column j of the packed triangle
    const double* d;
    int j;
    __device__ double operator()(int i) const { return __ldcg(d + tri(i - 1) + (j - 1)); }
};

// Shared memory of a CTA: the search inputs r[] (diq/djq terms) and v[]
// (valid flags), the CTA's reduction scratch, and, in CTA 0 when they fit, the
// per-node working arrays of the joins.
struct Smem {
    double* r;
    unsigned char* v;
    unsigned long long* red_k;
    long long* red_i;
    int2* red_ij;
    double* red_d;
    double* ext;  // sumCols, sumRows, av, join (n+1 each), then rep and two lists (n+1 ints each)
};

__host__ __device__ inline size_t smem_layout(int n, bool node_shared, size_t* ext_off, size_t* v_off) {
    size_t off = sizeof(double) * (size_t)(n + 1);                          // r
    off += (2 * sizeof(double) + sizeof(long long) + sizeof(int2)) * kWarps;  // reduction scratch
    *ext_off = off;
    if (node_shared) off += 4 * sizeof(double) * (size_t)(n + 1) + 3 * sizeof(int) * (size_t)(n + 1);
    *v_off = off;
    return off + (size_t)(n + 1) + 16;
}

__device__ Smem carve(int n, bool node_shared) {
    extern __shared__ __align__(16) unsigned char smem[];
    size_t ext_off, v_off;
    smem_layout(n, node_shared, &ext_off, &v_off);
    Smem S;
    S.r = reinterpret_cast<double*>(smem);
    size_t off = sizeof(double) * (size_t)(n + 1);
    S.red_k = reinterpret_cast<unsigned long long*>(smem + off);
    off += sizeof(unsigned long long) * kWarps;
    S.red_d = reinterpret_cast<double*>(smem + off);
    off += sizeof(double) * kWarps;
    S.red_i = reinterpret_cast<long long*>(smem + off);
    off += sizeof(long long) * kWarps;
    S.red_ij = reinterpret_cast<int2*>(smem + off);
    S.ext = reinterpret_cast<double*>(smem + ext_off);
    S.v = smem + v_off;
    return S;
}

// CTA 0's per-node state: shared memory when it fits, else the global arrays
// of Args. r and valid are also published to global memory for the search.
struct Node {
    double* sumCols;
    double* sumRows;
    double* av;
    double* join;
    double* r;
    unsigned char* valid;
    int* rep;
    int* vlist;  // valid nodes, ascending: the terms of the sequential sums
    int* vnext;  // the other list buffer (the list without this cycle's minj)
};

// A search candidate: criterion, element index (scan order), (ii, jj) and
// d(ii, jj), which the join needs first.
struct Cand {
    unsigned long long k;
    long long i;
    int2 ij;
    double d;
};

__device__ __forceinline__ void warp_min(Cand& c) {
    for (int o = 16; o > 0; o >>= 1) {
        Cand o2;
        o2.k = __shfl_down_sync(0xffffffffu, c.k, o);
        o2.i = __shfl_down_sync(0xffffffffu, c.i, o);
        o2.ij.x = __shfl_down_sync(0xffffffffu, c.ij.x, o);
        o2.ij.y = __shfl_down_sync(0xffffffffu, c.ij.y, o);
        o2.d = __shfl_down_sync(0xffffffffu, c.d, o);
        if (better(o2.k, o2.i, c.k, c.i)) c = o2;
    }
}

// ---------------------------------------------------------------------------
// Cycle hand-off between CTA 0 and the rest: one-way signals instead of full
// grid barriers. Every other CTA adds 1 to `arrive` when its candidate is
// written; CTA 0 waits for the count, joins, publishes, and raises `release`
// to the next cycle number. Both counters only grow. Waits are bounded and
// also end when any CTA has set an error status.
// ---------------------------------------------------------------------------
// Every thread of the CTA returns the same verdict (read once by thread 0).
__device__ bool wait_geq(const Args& A, const unsigned* p, unsigned target) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        const unsigned long long t0 = gtimer();
        unsigned it = 0;
        while ((int)(ld_acquire(p) - target) < 0) {
            if (ld_status(A.status) != ST_OK) break;
            if (++it > kSpinLimit || gtimer() - t0 > A.wait_ns) {
                atomicCAS(A.status, ST_OK, ST_TIMEOUT);
                break;
            }
            if (it > 256) __nanosleep(32);
        }
        __threadfence();
        s_ok = ld_status(A.status) == ST_OK;
    }
    __syncthreads();
    const bool ok = s_ok;
    __syncthreads();  // s_ok is rewritten by the next wait
    return ok;
}
// Every thread fences its own global writes before the CTA signals.
__device__ void signal_add(unsigned* p) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(p, 1u);
}
__device__ void signal_set(unsigned* p, unsigned v) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) st_release(p, v);
}

// One cycle's search over this CTA's work items; writes the CTA minimum.
__device__ void search(const Args& A, const Smem& S, bool reload) {
    const int n = A.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (reload) {
        for (int j = threadIdx.x; j <= n; j += blockDim.x) {
            S.r[j] = __ldcg(A.r + j);
            S.v[j] = __ldcg(A.valid + j);
        }
    }
    const double c = __ldcg(A.scal + 0);
    const double f = __ldcg(A.scal + 1);
    const unsigned long long kmin0 = okey(__dmul_rn(__dmul_rn(99999.0, 2.0), f));  // NJTree.cpp:334
    __syncthreads();
    Cand b{kmin0, -1, make_int2(0, 0), 0.0};
    const int gw = warp * gridDim.x + blockIdx.x, nw = kWarps * gridDim.x;
    for (int t = gw; t < A.n_items; t += nw) {
        const int2 it = __ldg(A.items + t);
        const int jj = it.x;
        if (!S.v[jj]) continue;
        const double rj = S.r[jj];
        const size_t base = tri(jj - 1);
        const int e0 = it.y * kChunk + lane;
        double dv[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int e = e0 + 32 * u;
            dv[u] = e < jj - 1 ? __ldcg(A.d + base + e) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int e = e0 + 32 * u;
            if (e < jj - 1 && S.v[e + 1]) {
                const double tot = __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(f, dv[u]), c), S.r[e + 1]), rj);
                const unsigned long long kt = okey(tot);
                if (kt < b.k) {  // items and elements come in scan order per lane
                    b.k = kt;
                    b.i = (long long)(base + e);
                    b.ij = make_int2(e + 1, jj);
                    b.d = dv[u];
                }
            }
        }
    }
    warp_min(b);
    if (lane == 0) {
        S.red_k[warp] = b.k;
        S.red_i[warp] = b.i;
        S.red_ij[warp] = b.ij;
        S.red_d[warp] = b.d;
    }
    __syncthreads();
    if (warp == 0) {
        b = Cand{kmin0, -1, make_int2(0, 0), 0.0};
        if (lane < kWarps) b = Cand{S.red_k[lane], S.red_i[lane], S.red_ij[lane], S.red_d[lane]};
        warp_min(b);
        if (lane == 0) {
            A.cand_k[blockIdx.x] = b.k;
            A.cand_idx[blockIdx.x] = b.i;
            A.cand_ij[blockIdx.x] = b.ij;
            A.cand_d[blockIdx.x] = b.d;
        }
    }
    __syncthreads();
}

// Writes r[j] = sumCols[j] + sumRows[j] for the valid j other than j_skip,
// on this CTA's threads t0 and up, to the node array and, when that is in
// shared memory, to the global copy the other CTAs read.
__device__ void publish_r(const Args& A, const Node& N, bool shared, int t0, int j_skip) {
    const int n = A.n;
    for (int j = 1 + (int)threadIdx.x - t0; j <= n; j += blockDim.x - t0) {
        if (!N.valid[j] || j == j_skip) continue;
        const double v = __dadd_rn(N.sumCols[j], N.sumRows[j]);
        N.r[j] = v;
        if (shared) A.r[j] = v;
    }
}

// Branch lengths of cycle nc (NJTree.cpp:378-470), av and rep of the joined
// node. Nothing else in the cycle reads what this writes, so one thread does
// it beside the sums.
__device__ void branch_lengths(const Args& A, const Node& N, int nc, int mini, int minj, double dmin, double dio_sum,
                               double djo_sum, double avi, double avj) {
    const double fnseqs = A.scal[2];
    const double fnseqs2 = A.scal[1];
    const double dio = __ddiv_rn(__dsub_rn(dio_sum, dmin), fnseqs2);
    const double djo = __ddiv_rn(__dsub_rn(djo_sum, dmin), fnseqs2);
    double bi = __dmul_rn(__dsub_rn(__dadd_rn(dmin, dio), djo), 0.5);
    double bj = __dsub_rn(dmin, bi);
    bi = __dsub_rn(bi, avi);
    bj = __dsub_rn(bj, avj);
    if (fabs(bi) < 0.0001) bi = 0.0;
    if (fabs(bj) < 0.0001) bj = 0.0;
    A.left[nc] = bi;
    A.right[nc] = bj;
    if (dmin <= 0.0) dmin = 0.000001;
    N.av[mini] = __dmul_rn(dmin, 0.5);
    A.scal[2] = __dsub_rn(fnseqs, 1.0);
    N.rep[mini] = nc;
    if (A.joins) {
        A.joins[2 * (nc - 1)] = mini;
        A.joins[2 * (nc - 1) + 1] = minj;
    }
}

// One join (CTA 0): NJTree.cpp:378-641 as restated in the oracle.
__device__ bool update(const Args& A, Node& N, bool shared, int nc) {
    const int n = A.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ int s_mini, s_minj, s_repi, s_repj;
    __shared__ double s_sR, s_sC, s_sumd, s_dio, s_djo, s_avi, s_avj, s_dmin;
    Cand b;
    {
        // Every CTA's candidate, one per thread of this CTA (all loads in one
        // round trip), reduced per warp and then across the warps.
        __shared__ Cand s_cand[kWarps];
        const double f = __ldcg(A.scal + 1);
        const Cand none{okey(__dmul_rn(__dmul_rn(99999.0, 2.0), f)), -1, make_int2(0, 0), 0.0};
        b = none;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
            const Cand o{__ldcg(A.cand_k + k), __ldcg(A.cand_idx + k), __ldcg(A.cand_ij + k), __ldcg(A.cand_d + k)};
            if (better(o.k, o.i, b.k, b.i)) b = o;
        }
        warp_min(b);
        if (lane == 0) s_cand[warp] = b;
        __syncthreads();
        if (warp == 0) {
            b = lane < kWarps ? s_cand[lane] : none;
            warp_min(b);
        }
    }
    if (warp == 0) {
        if (lane == 0) {
            const int mi = b.i >= 0 ? b.ij.x : 0, mj = b.i >= 0 ? b.ij.y : 0;
            s_mini = mi;
            s_minj = mj;
            if (mi) {  // everything the scalar step reads before the loop changes it
                s_dio = __dadd_rn(N.sumCols[mi], N.sumRows[mi]);
                s_djo = __dadd_rn(N.sumCols[mj], N.sumRows[mj]);
                s_avi = N.av[mi];
                s_avj = N.av[mj];
                s_repi = N.rep[mi];
                s_repj = N.rep[mj];
                s_dmin = b.d;
            }
        }
    }
    __syncthreads();
    const int mini = s_mini, minj = s_minj;
    if (mini == 0) {
        if (threadIdx.x == 0) atomicCAS(A.status, ST_OK, ST_NOJOIN);
        return false;
    }
    // Invariants every index below relies on; a violation ends the kernel
    // with a status instead of an out-of-range access.
    if (!(mini >= 1 && mini < minj && minj <= n) || s_repi < 0 || s_repi >= nc || s_repj < 0 || s_repj >= nc) {
        if (threadIdx.x == 0) atomicCAS(A.status, ST_OK, ST_INTERNAL);
        return false;
    }
    const int typei = s_avi > 0.0 ? 0 : 1, typej = s_avj > 0.0 ? 0 : 1;
    // treeDesc row nc (NJTree.cpp:478-531) and the joined row (NJTree.cpp:541-641),
    // one node per thread: each node's sums, join value and matrix entries are
    // touched only by its own iteration, so the reference's two loops fuse.
    int* row = A.desc + (size_t)nc * (n + 1);
    const int* rowi = A.desc + (size_t)s_repi * (n + 1);
    const int* rowj = A.desc + (size_t)s_repj * (n + 1);
    for (int j = 1 + threadIdx.x; j <= n; j += blockDim.x) {
        const bool live = N.valid[j] && j != minj;
        const double d_jj = live && j != minj ? __ldcg(A.d + sym(j, minj)) : 0.0;
        const double d_ji = live && j != mini ? __ldcg(A.d + sym(j, mini)) : 0.0;
        int v = typei == 0 ? (rowi[j] == 1) : (j == mini);
        v |= typej == 0 ? (rowj[j] == 1) : (j == minj);
        row[j] = v;
        if (live) {
            double sc = N.sumCols[j], sr = N.sumRows[j];
            if (j < minj) sc = __dsub_rn(sc, d_jj);
            else sr = __dsub_rn(sr, d_jj);
            if (j < mini) sc = __dsub_rn(sc, d_ji);
            else if (j > mini) sr = __dsub_rn(sr, d_ji);
            const double jv = half_of(__dadd_rn(d_jj, d_ji));
            N.join[j] = jv;
            if (j < mini) {
                A.d[sym(j, mini)] = jv;
                sc = __dadd_rn(sc, jv);
            } else if (j > mini) {
                A.d[sym(mini, j)] = jv;
                sr = __dadd_rn(sr, jv);
            }
            N.sumCols[j] = sc;
            N.sumRows[j] = sr;
        }
        A.d[sym(minj, j)] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        N.valid[minj] = 0;
        if (shared) A.valid[minj] = 0;
    }
    __syncthreads();
    // minj leaves the list of valid nodes (nv of them before this join: one
    // node leaves per cycle). The reference's sums run over the valid nodes in
    // ascending order, skipping the others, which add +0.0 and change nothing,
    // so the sums below walk the list instead of all n nodes. The list
    // without minj is written to the other buffer beside the first sums.
    const int nv = n - nc + 1;
    __shared__ int s_pi, s_pj, s_bad;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nv;  // first k with vlist[k] >= mini, then minj
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (N.vlist[mid] < mini) lo = mid + 1; else hi = mid;
        }
        s_pi = lo;
        hi = nv;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (N.vlist[mid] < minj) lo = mid + 1; else hi = mid;
        }
        s_pj = lo;
        s_bad = !(s_pi < nv && N.vlist[s_pi] == mini && lo < nv && N.vlist[lo] == minj);
        if (s_bad) atomicCAS(A.status, ST_OK, ST_INTERNAL);
    }
    __syncthreads();
    if (s_bad) return false;
    const int pi = s_pi, pj = s_pj;
    // The reference's three sequential sums on three warps (three SM
    // sub-partitions): sumRows[mini] and sumCols[mini] over the joined row
    // (NJTree.cpp:590-616) and the next cycle's sumd over sumCols
    // (NJTree.cpp:314-321), whose terms after mini wait for sumCols[mini].
    // The other warps meanwhile form the next search's diq/djq terms, the
    // list without minj and the branch lengths.
    double sumd_part = 0.0;
    if (warp == 0) {
        const double v = warp_seq_sum(ListTerms{N.join, N.vlist}, 0, pi, 0.0);
        if (lane == 0) s_sR = v;
    } else if (warp == 1) {
        const double v = warp_seq_sum(ListSkipTerms{N.join, N.vlist, pj}, pi + 1, nv, 0.0);
        if (lane == 0) s_sC = v;
    } else if (warp == 2) {
        sumd_part = warp_seq_sum(ListTerms{N.sumCols, N.vlist}, 0, pi, 0.0);
    } else {
        if (threadIdx.x == 96)
            branch_lengths(A, N, nc, mini, minj, s_dmin, s_dio, s_djo, s_avi, s_avj);
        for (int k = (int)threadIdx.x - 96; k < nv - 1; k += blockDim.x - 96)
            N.vnext[k] = N.vlist[k < pj ? k : k + 1];
        publish_r(A, N, shared, 96, mini);
    }
    __syncthreads();
    if (warp == 2) {
        double v = __dadd_rn(sumd_part, s_sC);
        v = warp_seq_sum(ListTerms{N.sumCols, N.vnext}, pi + 1, nv - 1, v);
        if (lane == 0) s_sumd = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        N.sumRows[mini] = s_sR;
        N.sumCols[mini] = s_sC;
        N.sumCols[minj] = 0.0;
        N.sumRows[minj] = 0.0;
        const double rm = __dadd_rn(s_sC, s_sR);
        N.r[mini] = rm;
        if (shared) A.r[mini] = rm;
        const double fnseqs = A.scal[2];
        A.scal[0] = twice(s_sumd);
        A.scal[1] = __dsub_rn(fnseqs, 2.0);
    }
    __syncthreads();
    int* const t = N.vlist;  // the next cycle reads the list without minj
    N.vlist = N.vnext;
    N.vnext = t;
    return true;
}

// The last cycle: three nodes, a trichotomy (NJTree.cpp:646-737).
__device__ void last_cycle(const Args& A, const Node& N) {
    const int n = A.n;
    __shared__ int s_l[4], s_node[4], s_rep[4], s_ok;
    if (threadIdx.x == 0) {
        int k = 1;
        for (int i = 1; i <= n && k <= 3; ++i)
            if (N.valid[i]) s_l[k++] = i;
        s_ok = k == 4;
        for (int i = 1; i < k; ++i) s_ok = s_ok && N.rep[s_l[i]] >= 0 && N.rep[s_l[i]] <= n - 3;
        if (!s_ok) atomicCAS(A.status, ST_OK, ST_INTERNAL);
    }
    __syncthreads();
    if (!s_ok) return;
    if (threadIdx.x == 0) {
        const int l1 = s_l[1], l2 = s_l[2], l3 = s_l[3];
        const double d12 = __ldcg(A.d + sym(l1, l2)), d13 = __ldcg(A.d + sym(l1, l3)), d23 = __ldcg(A.d + sym(l2, l3));
        const double b1 = __dmul_rn(__dsub_rn(__dadd_rn(d12, d13), d23), 0.5);
        const double b2 = __dsub_rn(d12, b1);
        const double b3 = __dsub_rn(d13, b1);
        double br[4];
        br[1] = __dsub_rn(b1, N.av[l1]);
        br[2] = __dsub_rn(b2, N.av[l2]);
        br[3] = __dsub_rn(b3, N.av[l3]);
        for (int i = 1; i <= 3; ++i) {
            if (fabs(br[i]) < 0.0001) br[i] = 0.0;
            s_node[i] = N.av[s_l[i]] > 0.0;
            s_rep[i] = N.rep[s_l[i]];
        }
        A.left[n - 2] = br[1];
        A.left[n - 1] = br[2];
        A.left[n] = br[3];
    }
    __syncthreads();
    int* row = A.desc + (size_t)(n - 2) * (n + 1);
    for (int j = 1 + threadIdx.x; j <= n; j += blockDim.x) {
        int v = 0;
        for (int i = 1; i <= 3; ++i) {
            const bool in = s_node[i] ? A.desc[(size_t)s_rep[i] * (n + 1) + j] == 1 : j == s_l[i];
            if (in) v = i;
        }
        row[j] = v;
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_nj(Args A) {
    const int n = A.n;
    const bool shared = A.node_shared;
    const Smem S = carve(n, shared);
    const int lane = threadIdx.x & 31;
    const unsigned others = gridDim.x - 1;
    // Initialisation (NJTree.cpp:250-293): zero diagonal, row and column sums,
    // one warp per node.
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = gridDim.x * kWarps;
    for (int j = 1 + gwarp; j <= n; j += nwarps) {
        const double sr = warp_seq_sum(RowTerms{A.d + tri(j - 1)}, 1, j, 0.0);
        const double sc = warp_seq_sum(ColTerms{A.d, j}, j + 1, n + 1, 0.0);
        if (lane == 0) {
            A.sumRows[j] = sr;
            A.sumCols[j] = sc;
            A.d[sym(j, j)] = 0.0;
            A.av[j] = 0.0;
            A.rep[j] = 0;
            A.valid[j] = 1;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.valid[0] = 0;
    __syncthreads();
    if (blockIdx.x != 0) {
        signal_add(A.arrive);
        if (!wait_geq(A, A.release, 1u)) return;
        for (int nc = 1; nc <= n - 3; ++nc) {
            search(A, S, true);
            signal_add(A.arrive);
            if (!wait_geq(A, A.release, (unsigned)nc + 1u)) return;
        }
        return;
    }
    // CTA 0: gathers the node state, then joins.
    if (!wait_geq(A, A.arrive, others)) return;
    Node N;
    if (shared) {
        N.sumCols = S.ext;
        N.sumRows = S.ext + (n + 1);
        N.av = S.ext + 2 * (size_t)(n + 1);
        N.join = S.ext + 3 * (size_t)(n + 1);
        N.rep = reinterpret_cast<int*>(S.ext + 4 * (size_t)(n + 1));
        N.vlist = N.rep + (n + 1);
        N.vnext = N.vlist + (n + 1);
        N.r = S.r;
        N.valid = S.v;
        for (int j = threadIdx.x; j <= n; j += blockDim.x) {
            N.sumCols[j] = __ldcg(A.sumCols + j);
            N.sumRows[j] = __ldcg(A.sumRows + j);
            N.av[j] = 0.0;
            N.join[j] = 0.0;
            N.rep[j] = 0;
            N.valid[j] = j > 0;
        }
    } else {
        N = Node{A.sumCols, A.sumRows, A.av, A.join, A.r, A.valid, A.rep, A.vlist, A.vlist + (n + 1)};
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) N.vlist[k] = k + 1;  // every node starts valid
    __syncthreads();
    {
        __shared__ double s_sumd0;
        if (threadIdx.x < 32) {
            const double v = warp_seq_sum(ValidTerms{N.sumCols, N.valid}, 1, n + 1, 0.0);
            if (lane == 0) s_sumd0 = v;
        } else {
            publish_r(A, N, shared, 32, 0);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            A.scal[0] = twice(s_sumd0);
            A.scal[1] = __dsub_rn((double)n, 2.0);
            A.scal[2] = (double)n;
        }
        __syncthreads();
        signal_set(A.release, 1u);
    }
    for (int nc = 1; nc <= n - 3; ++nc) {
        search(A, S, !shared);
        if (!wait_geq(A, A.arrive, others * (unsigned)(nc + 1))) return;
        if (!update(A, N, shared, nc)) return;
        signal_set(A.release, (unsigned)nc + 1u);
    }
    last_cycle(A, N);
}

// Diagnostic: one CTA waits, with the tree's wait, for a counter that nothing
// raises; the wait must end at its limit with ST_TIMEOUT.
__global__ void k_wait_probe(Args A, unsigned target) { wait_geq(A, A.arrive, target); }

// One warp replays s0 + x[0] + ... + x[count-1] (diagnostic entry point).
__global__ void k_seq_sum(const double* x, int count, double s0, double* out) {
    const double v = warp_seq_sum(PlainTerms{x}, 0, count, s0);
    if (threadIdx.x == 0) *out = v;
}

}  // namespace cwnj

using namespace cwnj;

struct cwgpu_nj {
    int device = 0;
    int sm_count = 0;
    int grid = 0;
    cudaStream_t stream = nullptr;
    int cap_n = 0;
    double* d_work = nullptr;
    double* d_left = nullptr;
    double* d_right = nullptr;
    int* d_desc = nullptr;
    int* d_joins = nullptr;
    double* d_vec = nullptr;  // sumCols, sumRows, av, join, r
    unsigned char* d_valid = nullptr;
    int* d_rep = nullptr;
    unsigned long long* d_cand_k = nullptr;
    long long* d_cand_idx = nullptr;
    int2* d_cand_ij = nullptr;
    double* d_cand_d = nullptr;
    double* d_scal = nullptr;
    int2* d_items = nullptr;
    int items_n = -1;
    int n_items = 0;
    unsigned* d_sig = nullptr;  // [0] arrive, [1] release
    int* d_status = nullptr;
    size_t smem_set = 0;
    size_t smem_optin = 0;   // dynamic shared memory a CTA may use
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_kernel_s = 0.0;
    int64_t last_pairs = 0;
    std::string last_error;
};

namespace {

int fail(cwgpu_nj* h, cudaError_t e, const char* what) {
    h->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA;
}

#define NJ_CHECK(h, call)                                  \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return fail((h), e_, #call); \
    } while (0)

size_t smem_bytes(int n, bool node_shared) {
    size_t a, b;
    return smem_layout(n, node_shared, &a, &b);
}

// CTA 0 keeps the per-node arrays in shared memory when they fit.
bool node_shared_for(const cwgpu_nj* h, int n) { return smem_bytes(n, true) <= h->smem_optin; }

void free_buffers(cwgpu_nj* h) {
    void* ptrs[] = {h->d_work, h->d_left, h->d_right, h->d_desc, h->d_joins, h->d_vec, h->d_valid, h->d_rep,
                    h->d_items};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    h->d_work = h->d_left = h->d_right = h->d_vec = nullptr;
    h->d_desc = h->d_joins = h->d_rep = nullptr;
    h->d_valid = nullptr;
    h->d_items = nullptr;
    h->items_n = -1;
    h->cap_n = 0;
}

int ensure(cwgpu_nj* h, int n) {
    if (n > h->cap_n) {
        free_buffers(h);
        const size_t nel = (size_t)(n + 1) * (n + 2) / 2;
        NJ_CHECK(h, cudaMalloc(&h->d_work, nel * sizeof(double)));
        NJ_CHECK(h, cudaMalloc(&h->d_left, (n + 2) * sizeof(double)));
        NJ_CHECK(h, cudaMalloc(&h->d_right, (n + 2) * sizeof(double)));
        NJ_CHECK(h, cudaMalloc(&h->d_desc, (size_t)(n + 1) * (n + 1) * sizeof(int)));
        NJ_CHECK(h, cudaMalloc(&h->d_joins, (size_t)2 * (n + 1) * sizeof(int)));
        NJ_CHECK(h, cudaMalloc(&h->d_vec, 5 * (size_t)(n + 1) * sizeof(double)));
        NJ_CHECK(h, cudaMalloc(&h->d_valid, (size_t)(n + 1)));
        NJ_CHECK(h, cudaMalloc(&h->d_rep, 3 * (size_t)(n + 1) * sizeof(int)));  // rep, then two valid lists
        h->cap_n = n;
    }
    const size_t sm = smem_bytes(n, node_shared_for(h, n));
    if (sm > h->smem_optin) {
        h->last_error = "matrix too large for the search's shared memory";
        return CWGPU_ERR_ARG;
    }
    if (sm > h->smem_set) {
        NJ_CHECK(h, cudaFuncSetAttribute(k_nj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        h->smem_set = sm;
    }
    if (h->items_n != n) {
        std::vector<int2> items;
        for (int jj = 2; jj <= n; ++jj)
            for (int c = 0; c * kChunk < jj - 1; ++c) items.push_back(make_int2(jj, c));
        if (h->d_items) cudaFree(h->d_items);
        h->d_items = nullptr;
        NJ_CHECK(h, cudaMalloc(&h->d_items, std::max<size_t>(1, items.size()) * sizeof(int2)));
        NJ_CHECK(h, cudaMemcpy(h->d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
        h->n_items = (int)items.size();
        h->items_n = n;
    }
    return CWGPU_OK;
}

int64_t pairs_evaluated(int n) {
    int64_t s = 0;
    for (int nc = 1; nc <= n - 3; ++nc) {
        const int64_t m = n - nc + 1;
        s += m * (m - 1) / 2;
    }
    return s;
}

// Runs the kernel on h->d_work (already holding the input matrix).
int run(cwgpu_nj* h, int n, cudaStream_t st, double* d_left, double* d_right, int* d_desc, int* d_joins) {
    NJ_CHECK(h, cudaMemsetAsync(d_left, 0, (n + 2) * sizeof(double), st));
    NJ_CHECK(h, cudaMemsetAsync(d_right, 0, (n + 2) * sizeof(double), st));
    NJ_CHECK(h, cudaMemsetAsync(d_desc, 0, (size_t)(n + 1) * (n + 1) * sizeof(int), st));
    NJ_CHECK(h, cudaMemsetAsync(h->d_sig, 0, 2 * sizeof(unsigned), st));
    NJ_CHECK(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), st));
    Args A;
    A.d = h->d_work;
    A.n = n;
    A.left = d_left;
    A.right = d_right;
    A.desc = d_desc;
    A.joins = d_joins;
    A.sumCols = h->d_vec;
    A.sumRows = h->d_vec + (n + 1);
    A.av = h->d_vec + 2 * (size_t)(n + 1);
    A.join = h->d_vec + 3 * (size_t)(n + 1);
    A.r = h->d_vec + 4 * (size_t)(n + 1);
    A.valid = h->d_valid;
    A.rep = h->d_rep;
    A.vlist = h->d_rep + (n + 1);
    A.cand_k = h->d_cand_k;
    A.cand_idx = h->d_cand_idx;
    A.cand_ij = h->d_cand_ij;
    A.cand_d = h->d_cand_d;
    A.scal = h->d_scal;
    A.items = h->d_items;
    A.n_items = h->n_items;
    A.arrive = h->d_sig;
    A.release = h->d_sig + 1;
    A.status = h->d_status;
    A.node_shared = node_shared_for(h, n);
    A.wait_ns = kBarrierTimeoutNs;
    void* args[] = {&A};
    NJ_CHECK(h, cudaEventRecord(h->ev0, st));
    NJ_CHECK(h, cudaLaunchCooperativeKernel((const void*)k_nj, dim3(h->grid), dim3(kThreads), args,
                                            smem_bytes(n, A.node_shared), st));
    NJ_CHECK(h, cudaEventRecord(h->ev1, st));
    return CWGPU_OK;
}

int finish(cwgpu_nj* h, int n) {
    int status = 0;
    NJ_CHECK(h, cudaMemcpy(&status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    float ms = 0.f;
    NJ_CHECK(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->last_kernel_s = ms * 1e-3;
    h->last_pairs = pairs_evaluated(n);
    if (status == ST_TIMEOUT) {
        h->last_error = "a bounded wait between CTAs ran out";
        return CWGPU_ERR_TIMEOUT;
    }
    if (status == ST_INTERNAL) {
        h->last_error = "internal consistency check failed in the join kernel";
        return CWGPU_ERR_DEVICE;
    }
    if (status == ST_NOJOIN) {
        h->last_error = "no pair below the cut-off 2*99999*(n-2) (non-finite distances)";
        return CWGPU_ERR_ARG;
    }
    return CWGPU_OK;
}

}  // namespace

extern "C" {

int cwgpu_nj_create(int device, cwgpu_nj** out) {
    if (!out) return CWGPU_ERR_ARG;
    *out = nullptr;
    cwgpu_nj* h = new cwgpu_nj();
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
    int coop = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cand_k, h->sm_count * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cand_idx, h->sm_count * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cand_ij, h->sm_count * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cand_d, h->sm_count * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_scal, 4 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_sig, 2 * sizeof(unsigned));
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nj);
    if (e == cudaSuccess) h->smem_optin = (size_t)optin > fa.sharedSizeBytes ? optin - fa.sharedSizeBytes : 0;
    if (e == cudaSuccess) e = cudaMalloc(&h->d_status, sizeof(int));
    if (e != cudaSuccess || !coop) {
        cwgpu_nj_destroy(h);
        return e == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA;
    }
    // One CTA per SM (512 threads); CTA 0 and the others wait on each other,
    // so the launch is cooperative: every CTA is resident.
    h->grid = std::min(h->sm_count, kMaxGrid);
    *out = h;
    return CWGPU_OK;
}

void cwgpu_nj_destroy(cwgpu_nj* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_buffers(h);
    void* ptrs[] = {h->d_cand_k, h->d_cand_idx, h->d_cand_ij, h->d_cand_d, h->d_scal, h->d_sig, h->d_status};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

const char* cwgpu_nj_last_error(const cwgpu_nj* h) { return h ? h->last_error.c_str() : ""; }

int cwgpu_nj_tree(cwgpu_nj* h, int32_t n, double* elements, double* left_branch, double* right_branch,
                  int32_t* tree_desc, int32_t* joins) {
    if (!h || !elements || !left_branch || !right_branch || !tree_desc) return CWGPU_ERR_ARG;
    if (n < 2 || n > CWGPU_NJ_MAX_N) return CWGPU_ERR_ARG;
    if (n == 2) return CWGPU_OK;  // NJTree.cpp:218-229
    NJ_CHECK(h, cudaSetDevice(h->device));
    int rc = ensure(h, n);
    if (rc) return rc;
    const size_t nel = (size_t)(n + 1) * (n + 2) / 2;
    cudaStream_t st = h->stream;
    NJ_CHECK(h, cudaMemcpyAsync(h->d_work, elements, nel * sizeof(double), cudaMemcpyHostToDevice, st));
    rc = run(h, n, st, h->d_left, h->d_right, h->d_desc, joins ? h->d_joins : nullptr);
    if (rc) return rc;
    NJ_CHECK(h, cudaMemcpyAsync(elements, h->d_work, nel * sizeof(double), cudaMemcpyDeviceToHost, st));
    NJ_CHECK(h, cudaMemcpyAsync(left_branch, h->d_left, (n + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
    NJ_CHECK(h, cudaMemcpyAsync(right_branch, h->d_right, (n + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
    NJ_CHECK(h, cudaMemcpyAsync(tree_desc, h->d_desc, (size_t)(n + 1) * (n + 1) * sizeof(int),
                                cudaMemcpyDeviceToHost, st));
    if (joins)
        NJ_CHECK(h, cudaMemcpyAsync(joins, h->d_joins, (size_t)2 * (n - 3) * sizeof(int), cudaMemcpyDeviceToHost, st));
    NJ_CHECK(h, cudaStreamSynchronize(st));
    return finish(h, n);
}

int cwgpu_nj_tree_device(cwgpu_nj* h, int32_t n, const double* d_elements_in, double* d_elements_out,
                         double* d_left_branch, double* d_right_branch, int32_t* d_tree_desc, int32_t* d_joins,
                         void* stream) {
    if (!h || !d_elements_in || !d_left_branch || !d_right_branch || !d_tree_desc) return CWGPU_ERR_ARG;
    if (n < 2 || n > CWGPU_NJ_MAX_N) return CWGPU_ERR_ARG;
    if (n == 2) return CWGPU_OK;
    NJ_CHECK(h, cudaSetDevice(h->device));
    int rc = ensure(h, n);
    if (rc) return rc;
    const size_t nel = (size_t)(n + 1) * (n + 2) / 2;
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    NJ_CHECK(h, cudaMemcpyAsync(h->d_work, d_elements_in, nel * sizeof(double), cudaMemcpyDeviceToDevice, st));
    rc = run(h, n, st, d_left_branch, d_right_branch, d_tree_desc, d_joins);
    if (rc) return rc;
    if (d_elements_out)
        NJ_CHECK(h, cudaMemcpyAsync(d_elements_out, h->d_work, nel * sizeof(double), cudaMemcpyDeviceToDevice, st));
    NJ_CHECK(h, cudaStreamSynchronize(st));
    return finish(h, n);
}

int cwgpu_nj_wait_probe(cwgpu_nj* h, int64_t timeout_ns, int32_t* timed_out) {
    if (!h || !timed_out || timeout_ns <= 0 || timeout_ns > (int64_t)kBarrierTimeoutNs) return CWGPU_ERR_ARG;
    NJ_CHECK(h, cudaSetDevice(h->device));
    NJ_CHECK(h, cudaMemsetAsync(h->d_sig, 0, 2 * sizeof(unsigned), h->stream));
    NJ_CHECK(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    Args A;
    memset(&A, 0, sizeof(A));
    A.arrive = h->d_sig;
    A.release = h->d_sig + 1;
    A.status = h->d_status;
    A.wait_ns = (unsigned long long)timeout_ns;
    k_wait_probe<<<1, 32, 0, h->stream>>>(A, 1u);
    NJ_CHECK(h, cudaGetLastError());
    NJ_CHECK(h, cudaStreamSynchronize(h->stream));
    int status = 0;
    NJ_CHECK(h, cudaMemcpy(&status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    NJ_CHECK(h, cudaMemset(h->d_status, 0, sizeof(int)));
    *timed_out = status == ST_TIMEOUT ? 1 : 0;
    return CWGPU_OK;
}

int cwgpu_nj_seq_sum(cwgpu_nj* h, const double* x, int64_t count, double s0, double* out) {
    if (!h || !out || count < 0 || count > (1ll << 30) || (count && !x)) return CWGPU_ERR_ARG;
    NJ_CHECK(h, cudaSetDevice(h->device));
    double* d = nullptr;
    NJ_CHECK(h, cudaMalloc(&d, (size_t)(count + 1) * sizeof(double)));
    cudaError_t e = count ? cudaMemcpy(d + 1, x, (size_t)count * sizeof(double), cudaMemcpyHostToDevice) : cudaSuccess;
    if (e == cudaSuccess) {
        k_seq_sum<<<1, 32, 0, h->stream>>>(d + 1, (int)count, s0, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(h, e, "cwgpu_nj_seq_sum");
    return CWGPU_OK;
}

int cwgpu_nj_last_stats(const cwgpu_nj* h, int64_t* pairs_evaluated_out, double* kernel_seconds) {
    if (!h) return CWGPU_ERR_ARG;
    if (pairs_evaluated_out) *pairs_evaluated_out = h->last_pairs;
    if (kernel_seconds) *kernel_seconds = h->last_kernel_s;
    return CWGPU_OK;
}

}  // extern "C"
