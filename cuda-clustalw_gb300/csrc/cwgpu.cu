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
#include <climits>
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

// ---- one CTA per pair: the pair's stripes shared by the warps of a CTA ------
//
// For launches with fewer long pairs than the long-pair kernel has warps, one
// warp per pair leaves most of the GPU idle. Here a CTA of nw warps aligns one
// pair: forwardPass and reversePass are shared sweeps (cwgpu::sweep_mw) over
// all nw warps, whose results are reduced across the warps; Myers-Miller
// frames of at least large_rows rows (0: the larger of 512 and a third of the
// pair's diff() box) are divided by the two halves of the CTA at once (forward
// half on warps [0, nw/2), reverse half on [nw/2, nw)), or two such frames at
// once on half the CTA each, and the smaller frames they leave go to a shared
// stack that every warp takes frames from (cwgpu::mm_align) and gives the
// children it makes back to. Frames are independent once (A, B, M, N, tb, te) are
// known and diff()'s identity and match counts are sums over its M == 1
// leaves, so results equal those of the one-warp form.
constexpr int kCtaMaxWarps = 16;
constexpr int kCtaStack = 64;
constexpr int kCtaSmall = 256;
constexpr int kRootBit = 1 << 30;  // in Frame.z (M < 2^17): the pair's top frame

struct CtaCtl {
    unsigned long long prog[kCtaMaxWarps];  // cwgpu::MwSync progress words
    int abort;
    int stop;  // reversePass: lowest stripe that reached maxScore
    long long q;
    int bval[kCtaMaxWarps];
    unsigned bkey[kCtaMaxWarps];
    long long dcells[kCtaMaxWarps];
    int ident[kCtaMaxWarps], match[kCtaMaxWarps];
    int mm;  // diff()'s score of the pair
    int nstack, nsmall, small_next;
    int lock, active;  // the shared frame stack `small`: its lock, warps holding a frame from it
    int4 stack[kCtaStack];  // large frames: (A, B, M | root, N | tb << 29 | te << 30)
    int4 small[kCtaSmall];  // frames for one warp each
};

struct CtaArgs {
    int large_rows;
    unsigned long long limit_ns;
};

// Maximum value, then lowest key, over the warps' results in C.
__device__ __forceinline__ cwgpu::Best cta_reduce(const CtaCtl& C, int nw) {
    cwgpu::Best b;
    b.val = C.bval[0];
    b.key = C.bkey[0];
    for (int w = 1; w < nw; ++w) {
        if (C.bval[w] > b.val || (C.bval[w] == b.val && C.bkey[w] < b.key)) {
            b.val = C.bval[w];
            b.key = C.bkey[w];
        }
    }
    return b;
}

__device__ __forceinline__ bool cta_large(int M, int N, int large_rows) { return M >= large_rows && N >= 64; }

constexpr int kShareRows = 64;  // frames with fewer rows stay with the warp that divided them

// The frames of C.small (every thread calls). C.small is a stack that every
// warp takes frames from and gives frames to: a warp takes a frame, runs the
// one-warp Myers-Miller on it, and after each division gives the right child
// back to the stack (if it has kShareRows rows or more and there is room) so
// that idle warps can take it. The phase ends when the stack is empty and no
// warp holds a frame. A warp that finds the stack empty while others still
// hold frames waits (bounded, like the stripe hand-overs).
template <int RS>
__device__ void cta_small_frames(CtaCtl& C, const int8_t* s1, const int8_t* s1r, int n, const int8_t* s2,
                                 const int8_t* s2r, int m, int go, int ge, int2* bufA, int2* bufB, const cwgpu::Env& X,
                                 const CtaArgs& ca, int& ident, int& match, long long& cells) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        C.active = 0;
        C.lock = 0;
    }
    __syncthreads();
    cwgpu::FrameShare fs;
    fs.frames = C.small;
    fs.count = &C.nsmall;
    fs.lock = &C.lock;
    fs.cap = kCtaSmall;
    fs.min_rows = kShareRows;
    volatile int* vcount = &C.nsmall;
    volatile int* vactive = &C.active;
    volatile int* vabort = &C.abort;
    unsigned long long t_wait = 0;
    for (;;) {
        int state = 0;  // 0: nothing to take yet, 1: took a frame, 2: phase over
        int fa = 0, fb = 0, fm = 0, fn = 0;
        if (lane == 0) {
            if (*vabort) {
                state = 2;
            } else if (atomicCAS(&C.lock, 0, 1) == 0) {
                __threadfence_block();
                const int c = *vcount;
                if (c > 0) {
                    volatile int* e = reinterpret_cast<volatile int*>(&C.small[c - 1]);
                    fa = e[0];
                    fb = e[1];
                    fm = e[2];
                    fn = e[3];
                    *vcount = c - 1;
                    atomicAdd(&C.active, 1);
                    state = 1;
                } else if (*vactive == 0) {
                    state = 2;
                }
                __threadfence_block();
                atomicExch(&C.lock, 0);
            }
            if (state == 0) {  // bounded wait for frames other warps still hold
                const unsigned long long now = cwgpu::global_ns();
                if (t_wait == 0) {
                    t_wait = now;
                } else if (now - t_wait > ca.limit_ns) {
                    *vabort = 1;
                    atomicExch(X.err, cwgpu::kStatusTimeout);
                    state = 2;
                }
            } else {
                t_wait = 0;
            }
        }
        state = __shfl_sync(cwgpu::kFull, state, 0);
        if (state == 2) break;
        if (state == 0) continue;
        fa = __shfl_sync(cwgpu::kFull, fa, 0);
        fb = __shfl_sync(cwgpu::kFull, fb, 0);
        fm = __shfl_sync(cwgpu::kFull, fm, 0);
        fn = __shfl_sync(cwgpu::kFull, fn, 0);
        int mmf = 0, id = 0, mt = 0;
        long long ce = 0;
        cwgpu::mm_align<RS, true, true>(s1, s1r, n, s2, s2r, m, fa, fb, fm & ~kRootBit, fn, go, ge, bufA, bufB, X, mmf,
                                        id, mt, ce, &fs);
        ident += id;
        match += mt;
        cells += ce;
        if ((fm & kRootBit) && lane == 0) C.mm = mmf;
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            atomicSub(&C.active, 1);  // after every frame this one gave to the stack
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) C.nsmall = 0;
    __syncthreads();
}

// diff() + tracePath of one pair by the whole CTA (every thread calls).
template <int RS>
__device__ void cta_diff(CtaCtl& C, const int8_t* s1, const int8_t* s1r, int n, const int8_t* s2, const int8_t* s2r,
                         int m, int A0, int B0, int M0, int N0, int go, int ge, int2* bufs, size_t stride, int nw,
                         const cwgpu::Env& X, cwgpu::MwSync& mw, unsigned long long& epoch, const CtaArgs& ca,
                         int& mm_score, int& n_ident, int& n_match, long long& cells) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* bufA = bufs + (size_t)warp * stride;
    int2* bufB = bufA + stride / 2;
    int ident = 0, match = 0;
    long long ncell = 0;
    // Frames divided by the CTA: at least large_rows rows; automatically the
    // top two levels of the recursion (measured on one-column calls of 1523
    // residues and sets of 3000: both faster than a fixed 512 or 1024).
    const int large_rows = ca.large_rows > 0 ? ca.large_rows : max(512, M0 / 3);
    if (threadIdx.x == 0) {
        C.nstack = 0;
        C.nsmall = 0;
        C.mm = 0;
        const int4 root = make_int4(A0, B0, M0 | kRootBit, N0);
        if (cta_large(M0, N0, large_rows))
            C.stack[C.nstack++] = root;
        else
            C.small[C.nsmall++] = root;
    }
    __syncthreads();
    for (;;) {
        const int ns = C.nstack;
        if (ns == 0) break;
        // One large frame by the whole CTA, or, when two are waiting, both at
        // once: frame f on warps [f * nw / 2, (f + 1) * nw / 2), forward half
        // on the first half of those warps, reverse half on the second.
        const int k = (ns >= 2 && nw >= 4) ? 2 : 1;
        const int gw = nw / (2 * k);  // warps per half
        const int fi = warp / (2 * gw);
        const int4 F = C.stack[ns - 1 - fi];
        int4 Fs[2];
        Fs[0] = C.stack[ns - 1];
        Fs[1] = k > 1 ? C.stack[ns - 2] : Fs[0];
        __syncthreads();  // every thread has its frames before they are popped
        if (threadIdx.x == 0) C.nstack = ns - k;
        const int A = F.x, B = F.y, M = F.z & ~kRootBit;
        const int N = F.w & ((1 << 29) - 1);
        const int tbf = (F.w >> 29) & 1, tef = (F.w >> 30) & 1;
        const int tb = tbf ? go : 0, te = tef ? go : 0;
        const int midi = M / 2;
        const bool fwd_group = warp - fi * 2 * gw < gw;
        const int slot0 = fi * 2 * gw + (fwd_group ? 0 : gw);
        cwgpu::Task t;
        if (fwd_group) {
            t.rseq = s1 + A;
            t.cseq = s2 + B;
            t.rows = midi;
            t.ht0 = t.hl0 = -tb;
        } else {
            t.rseq = s1r + (n - A - M);
            t.cseq = s2r + (m - B - N);
            t.rows = M - midi;
            t.ht0 = t.hl0 = -te;
        }
        t.buf = nullptr;
        t.cols = N;
        t.hts = ge;
        t.eo = go;
        t.hls = ge;
        t.fo = go;
        mw.epoch = (++epoch) << 32;
        cwgpu::Best unused;
        cwgpu::sweep_mw<RS, cwgpu::MODE_GLOBAL>(t, go, ge, 0, X, unused, bufs, stride, slot0, warp - slot0, gw, mw,
                                                &C.stop);
        __syncthreads();
        if (warp == 0) {
            for (int f = 0; f < k; ++f) {
                const int4 G = Fs[f];
                const int GA = G.x, GB = G.y, GM = G.z & ~kRootBit;
                const int GN = G.w & ((1 << 29) - 1);
                const int gtbf = (G.w >> 29) & 1, gtef = (G.w >> 30) & 1;
                const int gmidi = GM / 2;
                ncell += (long long)GM * GN;
                const int2* fwd = bufs + (size_t)(f * 2 * gw + cwgpu::mw_last_rank(gmidi, RS, gw)) * stride;
                const int2* rev = bufs + (size_t)(f * 2 * gw + gw + cwgpu::mw_last_rank(GM - gmidi, RS, gw)) * stride;
                int midh, midj;
                bool type2;
                cwgpu::midpoint_scan(fwd, rev, GM, GN, gmidi, gtbf ? go : 0, gtef ? go : 0, go, ge, midh, midj, type2);
                if (lane == 0) {
                    if (G.z & kRootBit) C.mm = midh;
                    int4 ch[2];  // right, then left, as diff() pushes them (:598-609)
                    if (!type2) {
                        ch[0] = make_int4(GA + gmidi, GB + midj, GM - gmidi, (GN - midj) | (1 << 29) | (gtef << 30));
                        ch[1] = make_int4(GA, GB, gmidi, midj | (gtbf << 29) | (1 << 30));
                    } else {
                        ch[0] = make_int4(GA + gmidi + 1, GB + midj, GM - gmidi - 1, (GN - midj) | (gtef << 30));
                        ch[1] = make_int4(GA, GB, gmidi - 1, midj | (gtbf << 29));
                    }
                    for (int c = 0; c < 2; ++c) {
                        if (cta_large(ch[c].z, ch[c].w & ((1 << 29) - 1), large_rows) && C.nstack < kCtaStack)
                            C.stack[C.nstack++] = ch[c];
                        else
                            C.small[C.nsmall++] = ch[c];
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();
        if (C.nsmall > kCtaSmall - 4)
            cta_small_frames<RS>(C, s1, s1r, n, s2, s2r, m, go, ge, bufA, bufB, X, ca, ident, match, ncell);
    }
    cta_small_frames<RS>(C, s1, s1r, n, s2, s2r, m, go, ge, bufA, bufB, X, ca, ident, match, ncell);
    if (lane == 0) {
        C.ident[warp] = ident;
        C.match[warp] = match;
        C.dcells[warp] = ncell;
    }
    __syncthreads();
    n_ident = n_match = 0;
    cells = 0;
    for (int w = 0; w < nw; ++w) {
        n_ident += C.ident[w];
        n_match += C.match[w];
        cells += C.dcells[w];
    }
    mm_score = C.mm;
    __syncthreads();
}

// FullPairwiseAlign.cpp:112-183 for pair q by the whole CTA.
template <int RS>
__device__ void cta_pair(const cwgpu::PairArgs& g, long long q, CtaCtl& C, const cwgpu::Env& X, int2* bufs,
                         size_t stride, int nw, const CtaArgs& ca, unsigned long long& epoch,
                         unsigned long long (&acc)[3]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int si = g.pairs[2 * q], sj = g.pairs[2 * q + 1];
    const int n = g.lens[si], m = g.lens[sj];
    const int8_t* s1 = g.codes + g.offs[si];
    const int8_t* s2 = g.codes + g.offs[sj];
    const int8_t* s1r = cwgpu::rev_of(s1, n);
    const int8_t* s2r = cwgpu::rev_of(s2, m);
    const int go = g.go_table[min(n, m)], ge = g.ge;
    cwgpu_pair_stats st = cwgpu_pair_stats{0, 0, 0, 0, 0, 0, 0, 0};
    float dist = 1.0f;
    if (n > 0 && m > 0) {
        cwgpu::MwSync mw;
        mw.prog = C.prog;
        mw.abort = &C.abort;
        mw.err = g.err;
        mw.limit_ns = ca.limit_ns;
        // forwardPass
        cwgpu::Task t;
        t.rseq = s1;
        t.cseq = s2;
        t.rows = n;
        t.cols = m;
        t.ht0 = 0;
        t.hts = 0;
        t.eo = go;
        t.hl0 = 0;
        t.hls = 0;
        t.fo = go;
        t.buf = nullptr;
        mw.epoch = (++epoch) << 32;
        cwgpu::Best b;
        cwgpu::sweep_mw<RS, cwgpu::MODE_LOCAL_FWD>(t, go, ge, 0, X, b, bufs, stride, 0, warp, nw, mw, &C.stop);
        if (lane == 0) {
            C.bval[warp] = b.val;
            C.bkey[warp] = b.key;
        }
        __syncthreads();
        const cwgpu::Best fb = cta_reduce(C, nw);
        const int max_score = fb.val;
        const int se1 = max_score > 0 ? (int)(fb.key >> 16) + 1 : 0;
        const int se2 = max_score > 0 ? (int)(fb.key & 0xffffu) : 0;
        __syncthreads();
        if (threadIdx.x == 0) C.stop = INT_MAX;
        __syncthreads();
        // reversePass
        int sb1 = 1, sb2 = 1;
        if (se1 > 0) {
            cwgpu::Task r;
            r.rseq = s1r + (n - se1);
            r.cseq = s2r + (m - se2);
            r.rows = se1;
            r.cols = se2;
            r.ht0 = -1;
            r.hts = 0;
            r.eo = 0;
            r.hl0 = -1;
            r.hls = 0;
            r.fo = 0;
            r.buf = nullptr;
            mw.epoch = (++epoch) << 32;
            cwgpu::sweep_mw<RS, cwgpu::MODE_LOCAL_REV>(r, go, ge, max_score, X, b, bufs, stride, 0, warp, nw, mw,
                                                       &C.stop);
            if (lane == 0) {
                C.bval[warp] = b.val;
                C.bkey[warp] = b.key;
            }
            __syncthreads();
            const cwgpu::Best rb = cta_reduce(C, nw);
            __syncthreads();
            if (rb.val > 0) {
                sb1 = se1 - (int)(rb.key >> 16);
                sb2 = se2 - (int)(rb.key & 0xffffu) + 1;
            }
            if (rb.val >= max_score)
                acc[1] += (unsigned long long)(se1 - sb1) * se2 + (unsigned long long)(se2 - sb2 + 1);
            else
                acc[1] += (unsigned long long)se1 * se2;
        }
        acc[0] += (unsigned long long)n * m;
        // diff + tracePath
        int mm = 0, ident = 0, matches = 0;
        long long dcells = 0;
        cta_diff<RS>(C, s1, s1r, n, s2, s2r, m, sb1 - 1, sb2 - 1, se1 - sb1 + 1, se2 - sb2 + 1, go, ge, bufs, stride,
                     nw, X, mw, epoch, ca, mm, ident, matches, dcells);
        acc[2] += (unsigned long long)dcells;
        // distance (:170-181), float arithmetic with IEEE rounding.
        const int len1 = g.nres[si], len2 = g.nres[sj];
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
    if (threadIdx.x == 0) {
        g.dist[q] = dist;
        if (g.stats) g.stats[q] = st;
    }
}

// Persistent: each CTA takes the next pair of the longest-first queue.
__global__ void __launch_bounds__(kCtaMaxWarps * 32, 1) k_pairwise_cta(cwgpu::PairArgs g, CtaArgs ca) {
    __shared__ int smat[CWGPU_NUMRES * CWGPU_NUMRES];
    __shared__ CtaCtl C;
    extern __shared__ __align__(16) uint16_t region_all[];
    for (int i = threadIdx.x; i < CWGPU_NUMRES * CWGPU_NUMRES; i += blockDim.x) smat[i] = g.matrix[i];
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5;
    if (threadIdx.x < kCtaMaxWarps) C.prog[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        C.abort = 0;
        C.stop = INT_MAX;
    }
    cwgpu::Env X;
    X.smat = smat;
    X.region = region_all + (size_t)warp * (cwgpu::warp_region_bytes(g.K) / sizeof(uint16_t));
    X.K = g.K;
    X.gp1 = g.gp1;
    X.gp2 = g.gp2;
    X.tiny_m = g.tiny_m;
    X.tiny_n = g.tiny_n;
    X.err = g.err;
    const size_t stride = 2 * (size_t)(g.lmax + 1);  // a warp's two rows
    int2* bufs = g.scratch + (size_t)blockIdx.x * nw * stride;
    __syncthreads();
    unsigned long long epoch = 0;
    unsigned long long acc[3] = {0, 0, 0};
    for (;;) {
        if (threadIdx.x == 0) C.q = (long long)atomicAdd(g.counter, 1ULL);
        __syncthreads();
        const long long k = C.q;
        __syncthreads();
        if (k >= g.npairs) break;
        cta_pair<cwgpu::kR>(g, (long long)g.order[k], C, X, bufs, stride, nw, ca, epoch, acc);
    }
    if (threadIdx.x == 0 && g.cells && (acc[0] | acc[1] | acc[2])) {
        atomicAdd(g.cells + 0, acc[0]);
        atomicAdd(g.cells + 1, acc[1]);
        atomicAdd(g.cells + 2, acc[2]);
    }
}

// A wait of the shared sweeps on a progress word that nothing raises: warp 1
// waits for warp 0, which publishes nothing. It must end at its limit with
// the timeout status.
__global__ void k_cta_wait_probe(int* err, unsigned long long limit_ns) {
    __shared__ unsigned long long prog[2];
    __shared__ int abort_flag;
    if (threadIdx.x < 2) prog[threadIdx.x] = 0;
    if (threadIdx.x == 0) abort_flag = 0;
    __syncthreads();
    cwgpu::MwSync mw;
    mw.prog = prog;
    mw.abort = &abort_flag;
    mw.err = err;
    mw.epoch = 1ULL << 32;
    mw.limit_ns = limit_ns;
    if ((threadIdx.x >> 5) == 1) cwgpu::mw_wait(mw, 0, cwgpu::mw_word(mw, 0, 1));
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
    bool ctas = false;  // the long pairs run one CTA per pair
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

cudaError_t pinned_grow(unsigned char*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMallocHost(&p, std::max<size_t>(need, 4096));
    if (e == cudaSuccess) cap = std::max<size_t>(need, 4096);
    return e;
}

// Everything the pair kernels and the quick path read, in one arena: the code
// layout, both offset arrays and the lengths; with params, the residue counts
// (len1/len2 of FullPairwiseAlign.cpp:100-127) and the gap-open table by
// min(n, m) (:129-146); with the matrix, the matrix over the dense codes.
// One copy from one pinned buffer, on the context's stream, so later work on
// that stream sees it; the staging buffer is reused only after that copy.
int stage_inputs(cwgpu_context* ctx) {
    if (!ctx->in_dirty) return CWGPU_OK;
    if (!ctx->has_seqs) return fail(ctx, CWGPU_ERR_STATE, "sequences not uploaded");
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    const int ns = ctx->nseqs;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_codes = 0;
    const size_t o_poffs = o_codes + up(ctx->host_layout.size());
    const size_t o_offs = o_poffs + up(8 * (size_t)ns);
    const size_t o_lens = o_offs + up(8 * (size_t)ns);
    const size_t o_nres = o_lens + up(4 * (size_t)ns);
    const size_t o_go = o_nres + up(4 * (size_t)ns);
    const size_t o_mat = o_go + up(4 * (size_t)(ctx->lmax + 1));
    const size_t total = o_mat + 4 * CWGPU_NUMRES * CWGPU_NUMRES;
    if (total > ctx->cap_in) {
        dfree(ctx->d_in);
        ctx->cap_in = 0;
        CW_CUDA(ctx, cudaMalloc(&ctx->d_in, total));
        ctx->cap_in = total;
    }
    if (!ctx->ev_in) CW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming));
    CW_CUDA(ctx, cudaEventSynchronize(ctx->ev_in));  // the previous staging copy is done
    CW_CUDA(ctx, pinned_grow(ctx->h_in, ctx->cap_h_in, total));
    unsigned char* h = ctx->h_in;
    memcpy(h + o_codes, ctx->host_layout.data(), ctx->host_layout.size());
    memcpy(h + o_poffs, ctx->host_poffs.data(), 8 * (size_t)ns);
    memcpy(h + o_offs, ctx->offs.data(), 8 * (size_t)ns);
    memcpy(h + o_lens, ctx->lens.data(), 4 * (size_t)ns);
    if (ctx->has_params) {
        int32_t* nres = reinterpret_cast<int32_t*>(h + o_nres);
        const int gp1 = ctx->params.gap_pos1, gp2 = ctx->params.gap_pos2;
        auto occurs = [&](int c) { return c >= 0 && c < CWGPU_NUMRES && ((ctx->codes_present >> c) & 1u); };
        if (!occurs(gp1) && !occurs(gp2)) {
            memcpy(nres, ctx->lens.data(), 4 * (size_t)ns);  // no gap codes: every position is a residue
        } else {
            for (int s = 0; s < ns; ++s) {
                int c = 0;
                const int8_t* p = ctx->host_codes.data() + ctx->offs[s];
                for (int i = 0; i < ctx->lens[s]; ++i)
                    if (p[i] != gp1 && p[i] != gp2) ++c;
                nres[s] = c;
            }
        }
        // Gap open by length depends only on the params: kept between calls.
        std::vector<int32_t>& go = ctx->host_go;
        if (go.empty() || memcmp(&ctx->go_params, &ctx->params, sizeof(cwgpu_params)) != 0) {
            go.assign(1, 0);  // L = 0 pairs never reach the penalties (:113-118)
            ctx->go_params = ctx->params;
        }
        for (int L = (int)go.size(); L <= ctx->lmax; ++L) {
            int32_t g = 0, e = 0;
            cwgpu_gap_penalties(&ctx->params, L, L, &g, &e);
            go.push_back(g);
        }
        memcpy(h + o_go, go.data(), 4 * (size_t)(ctx->lmax + 1));
    }
    if (ctx->has_matrix) {  // over the dense codes, row stride 32 (entries past K unused)
        int32_t* dm = reinterpret_cast<int32_t*>(h + o_mat);
        memset(dm, 0, 4 * CWGPU_NUMRES * CWGPU_NUMRES);
        for (int a = 0; a < ctx->K; ++a)
            for (int b = 0; b < ctx->K; ++b)
                dm[a * CWGPU_NUMRES + b] = ctx->matrix[ctx->code_of[a] * CWGPU_NUMRES + ctx->code_of[b]];
    }
    CW_CUDA(ctx, cudaMemcpyAsync(ctx->d_in, h, total, cudaMemcpyHostToDevice, ctx->stream));
    CW_CUDA(ctx, cudaEventRecord(ctx->ev_in, ctx->stream));
    unsigned char* d = ctx->d_in;
    ctx->d_codes = reinterpret_cast<int8_t*>(d + o_codes);
    ctx->d_poffs = reinterpret_cast<int64_t*>(d + o_poffs);
    ctx->d_offs = reinterpret_cast<int64_t*>(d + o_offs);
    ctx->d_lens = reinterpret_cast<int32_t*>(d + o_lens);
    ctx->d_nres = ctx->has_params ? reinterpret_cast<int32_t*>(d + o_nres) : nullptr;
    ctx->d_go = ctx->has_params ? reinterpret_cast<int32_t*>(d + o_go) : nullptr;
    ctx->go_len = ctx->lmax + 1;
    ctx->d_matrix = ctx->has_matrix ? reinterpret_cast<int32_t*>(d + o_mat) : nullptr;
    ctx->in_dirty = false;
    ctx->generation++;
    return CWGPU_OK;
}

// The pair path needs params, matrix and sequences on the device.
int refresh_derived(cwgpu_context* ctx) {
    if (!ctx->has_params || !ctx->has_seqs) return fail(ctx, CWGPU_ERR_STATE, "params or sequences not set");
    return stage_inputs(ctx);
}

int gap_extend_of(const cwgpu_params& p) {
    int32_t g = 0, e = 0;
    cwgpu_gap_penalties(&p, 1, 1, &g, &e);
    return e;
}

size_t block_smem(int K, int warps) { return (size_t)cwgpu::warp_region_bytes(K) * warps; }

// CTAs of k_pairwise<RS> that fit on all SMs at once for an alphabet of K codes.
template <int RS>
cudaError_t pair_grid(int K, int sm_count, int* grid) {
    int per_sm = 0;
    cudaError_t e = cudaFuncSetAttribute(k_pairwise<RS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)block_smem(CWGPU_NUMRES, kWarpsPerBlock));
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairwise<RS>, kWarpsPerBlock * 32,
                                                          block_smem(K, kWarpsPerBlock));
    *grid = (per_sm < 1 ? 1 : per_sm) * sm_count;
    return e;
}

template <int RS>
int persistent_grid(cwgpu_context* ctx, int* grid) {
    CW_CUDA(ctx, pair_grid<RS>(ctx->K, ctx->sm_count, grid));
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
size_t cta_smem(int K, int warps) { return block_smem(K, warps); }

// CTAs of k_pairwise_cta that fit at once, capped so that their warps use no
// more scratch slots than the long-pair kernel's grid (the short-pair kernel's
// slots follow those, and it may run beside either).
// 0 when the CTA's shared memory (a score-profile region per warp) does not
// fit; launches then keep one warp per pair.
int cta_grid(cwgpu_context* ctx, int warps, int* grid) {
    int per_sm = 0, optin = 0;
    const size_t smem = cta_smem(ctx->K, warps);
    cudaFuncAttributes fa;
    CW_CUDA(ctx, cudaFuncGetAttributes(&fa, k_pairwise_cta));
    CW_CUDA(ctx, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    *grid = 0;
    if (smem + fa.sharedSizeBytes > (size_t)optin) return CWGPU_OK;
    CW_CUDA(ctx, cudaFuncSetAttribute(k_pairwise_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      std::max(fa.maxDynamicSharedSizeBytes, (int)smem)));
    CW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairwise_cta, warps * 32, smem));
    if (per_sm < 1) return CWGPU_OK;
    *grid = std::min(per_sm * ctx->sm_count, ctx->grid * kWarpsPerBlock / warps);
    return CWGPU_OK;
}

int ensure_scratch(cwgpu_context* ctx) {
    if (ctx->grid == 0 || ctx->grid_K != ctx->K) {
        int rc = persistent_grid<cwgpu::kR>(ctx, &ctx->grid);
        if (!rc) rc = persistent_grid<cwgpu::kRShort>(ctx, &ctx->grid_short);
        for (int l = 1; l <= 4 && !rc; ++l) rc = cta_grid(ctx, 1 << l, &ctx->grid_cta[l]);
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

// The order the persistent kernels take the pairs in (cwgpu_order.h).
void work_order(const cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, int32_t* order, int64_t* nlong) {
    cwgpu::work_order(ctx->lens.data(), ctx->len_key.data(), ctx->short_rows, pairs, npairs, order, nlong);
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

// Warps per CTA for a launch of nlong long pairs: the knob, or, when it is 0,
// 16 for at most half a pair per SM, 8 up to 2.5 pairs per SM, else 4
// (measured on 3000- and 1523-residue families: 15 pairs 21.4 / 18.6 / 14.3
// GCUPS with 16 / 8 / 4 warps; 190 pairs 137 / 171 / 151; 1,770 pairs 117 /
// 187 / 248).
int cta_warps_for(const cwgpu_context* ctx, int64_t nlong) {
    if (ctx->cta_warps) return ctx->cta_warps;
    if (2 * nlong <= ctx->sm_count) return 16;
    if (2 * nlong <= 5 * (int64_t)ctx->sm_count) return 8;
    return 4;
}

int log2_warps(int w) { return w >= 16 ? 4 : w >= 8 ? 3 : w >= 4 ? 2 : 1; }

// One persistent launch of k_pairwise_cta over g's queue (one CTA per pair).
cudaError_t launch_cta(const cwgpu_context* ctx, const cwgpu::PairArgs& g, int priority, cudaStream_t s) {
    const int warps = cta_warps_for(ctx, g.npairs);
    const int grid = (int)std::min<int64_t>(ctx->grid_cta[log2_warps(warps)], g.npairs);
    CtaArgs ca;
    ca.large_rows = ctx->cta_large_rows;
    ca.limit_ns = 4000000000ULL;  // no legitimate hand-over waits this long
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(warps * 32);
    cfg.dynamicSmemBytes = cta_smem(ctx->K, warps);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = priority;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_pairwise_cta, g, ca);
}

// Long pairs of a launch run one CTA per pair when there are few of them: at
// most cta_pairs, or, by default, a quarter of the long-pair kernel's warps
// (below that one warp per pair leaves most SMs idle; measured crossover on
// 1523-residue families between 190 and 1,770 pairs).
bool use_cta(const cwgpu_context* ctx, int64_t nlong) {
    const int64_t limit = ctx->cta_pairs >= 0 ? ctx->cta_pairs : (int64_t)ctx->grid * kWarpsPerBlock / 4;
    return nlong > 0 && nlong <= limit && ctx->grid_cta[log2_warps(cta_warps_for(ctx, nlong))] > 0;
}

// The queue-counter reset and one persistent launch per kernel: long pairs
// on s, short pairs on s2 forked from s when both kinds are present (joined
// back into s), else on s. The short-pair kernel runs at lower priority so
// that its CTAs take the SM slots long-pair CTAs leave as the long queue
// drains. Long pairs run one CTA per pair when there are at most cta_pairs of
// them, else one warp per pair. Works the same under stream capture.
cudaError_t enqueue_pairs(cwgpu_context* ctx, const cwgpu::PairArgs& gl, const cwgpu::PairArgs& gs, cudaStream_t s,
                          cudaStream_t s2, cudaEvent_t fork, cudaEvent_t join, bool counters_zeroed = false) {
    const size_t smem = block_smem(ctx->K, kWarpsPerBlock);
    const bool both = gl.npairs > 0 && gs.npairs > 0;
    cudaError_t e = counters_zeroed
                        ? cudaSuccess
                        : cudaMemsetAsync(gl.counter, 0, kCounterWords * sizeof(unsigned long long), s);
    cudaStream_t short_stream = s;
    if (e == cudaSuccess && both) {
        e = cudaEventRecord(fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, fork, 0);
        short_stream = s2;
    }
    if (e == cudaSuccess && gl.npairs > 0)
        e = use_cta(ctx, gl.npairs) ? launch_cta(ctx, gl, ctx->prio_high, s)
                                    : launch_persistent<cwgpu::kR>(gl, ctx->grid, smem, ctx->prio_high, s);
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

int status_error(cwgpu_context* ctx, int err) {
    if (err == cwgpu::kStatusTimeout)
        return fail(ctx, CWGPU_ERR_TIMEOUT, "a hand-over wait between the warps of a pair's CTA timed out");
    return fail(ctx, CWGPU_ERR_DEVICE, "kernel reported an internal limit (Myers-Miller stack depth)");
}

int check_kernel_error(cwgpu_context* ctx) {
    int err = 0;
    CW_CUDA(ctx, cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        CW_CUDA(ctx, cudaMemset(ctx->d_err, 0, sizeof(int)));
        if (err == cwgpu::kStatusTimeout)
            return fail(ctx, CWGPU_ERR_TIMEOUT, "a hand-over wait between the warps of a pair's CTA timed out");
        return fail(ctx, CWGPU_ERR_DEVICE, "kernel reported an internal limit (Myers-Miller stack depth)");
    }
    return CWGPU_OK;
}

}  // namespace

int cwgpu_stage_inputs(cwgpu_context* ctx) { return stage_inputs(ctx); }

cudaError_t cwgpu_pair_kernel_grids(int K, int sm_count, int* grid, int* grid_short) {
    cudaError_t e = pair_grid<cwgpu::kR>(K, sm_count, grid);
    if (e == cudaSuccess) e = pair_grid<cwgpu::kRShort>(K, sm_count, grid_short);
    return e;
}

int cwgpu_pair_kernel_warps_per_cta() { return kWarpsPerBlock; }

cudaError_t cwgpu_enqueue_pair_kernels(const cwgpu::PairArgs& gl, const cwgpu::PairArgs& gs, int grid,
                                       int grid_short, int prio_high, int prio_low, cudaStream_t s, cudaStream_t s2,
                                       cudaEvent_t fork, cudaEvent_t join) {
    const size_t smem = block_smem(gl.K, kWarpsPerBlock);
    const bool both = gl.npairs > 0 && gs.npairs > 0;
    cudaError_t e = cudaMemsetAsync(gl.counter, 0, kCounterWords * sizeof(unsigned long long), s);
    cudaStream_t short_stream = s;
    if (e == cudaSuccess && both) {
        e = cudaEventRecord(fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, fork, 0);
        short_stream = s2;
    }
    if (e == cudaSuccess && gl.npairs > 0) e = launch_persistent<cwgpu::kR>(gl, grid, smem, prio_high, s);
    if (e == cudaSuccess && gs.npairs > 0)
        e = launch_persistent<cwgpu::kRShort>(gs, grid_short, smem, prio_low, short_stream);
    if (e == cudaSuccess && both) {
        e = cudaEventRecord(join, s2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    }
    return e;
}

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
    dfree(ctx->d_in);
    if (ctx->h_in) cudaFreeHost(ctx->h_in);
    if (ctx->h_io) cudaFreeHost(ctx->h_io);
    if (ctx->ev_in) cudaEventDestroy(ctx->ev_in);
    dfree(ctx->d_scratch);
    dfree(ctx->d_counter);
    dfree(ctx->d_err);
    dfree(ctx->d_call);
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
    ctx->in_dirty = true;  // the device copy is remapped to the dense codes
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_set_params(cwgpu_context* ctx, const cwgpu_params* params) {
    if (!ctx || !params) return CWGPU_ERR_ARG;
    ctx->params = *params;
    ctx->has_params = true;
    ctx->in_dirty = true;
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_upload_seqs(cwgpu_context* ctx, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                      const int32_t* lens) {
    if (!ctx || nseqs < 0 || (nseqs > 0 && (!offsets || !lens))) return CWGPU_ERR_ARG;
    std::vector<int64_t> doffs(nseqs);
    int64_t total = 0;
    int lmax = 0;
    // One pass over the residues: the range check (a code outside [0, 31], read
    // as a byte, has a bit above bit 4) and the set of codes that occur.
    unsigned char seen[256] = {0};
    for (int s = 0; s < nseqs; ++s) {
        if (lens[s] < 0 || lens[s] > CWGPU_MAX_SEQ_LEN)
            return fail(ctx, CWGPU_ERR_ARG, "sequence length outside [0, CWGPU_MAX_SEQ_LEN]");
        if (lens[s] > 0 && (!codes || offsets[s] < 0)) return fail(ctx, CWGPU_ERR_ARG, "bad sequence offset");
        const uint8_t* p = lens[s] > 0 ? reinterpret_cast<const uint8_t*>(codes + offsets[s]) : nullptr;
        unsigned bits = 0;
        for (int i = 0; i < lens[s]; ++i) {
            bits |= p[i];
            seen[p[i]] = 1;
        }
        if (bits & ~(unsigned)(CWGPU_NUMRES - 1)) return fail(ctx, CWGPU_ERR_ARG, "residue code outside [0, 31]");
        doffs[s] = total;
        total += (lens[s] + 15) & ~15;
        lmax = std::max(lmax, (int)lens[s]);
    }
    std::vector<int8_t> packed((size_t)std::max<int64_t>(total, 16), 0);
    for (int s = 0; s < nseqs; ++s)
        if (lens[s] > 0) memcpy(packed.data() + doffs[s], codes + offsets[s], lens[s]);
    // Remap residue codes to the dense alphabet of the codes that occur, so the
    // per-stripe score profile holds K rows instead of 32.
    int K = 0, dense_of[CWGPU_NUMRES], code_of[CWGPU_NUMRES];
    uint32_t codes_present = 0;
    for (int c = 0; c < CWGPU_NUMRES; ++c) {
        dense_of[c] = seen[c] ? K : -1;
        if (seen[c]) {
            code_of[K++] = c;
            codes_present |= 1u << c;
        }
    }
    if (K == 0) {  // no residues at all: keep one code so launches stay well-formed
        dense_of[0] = 0;
        code_of[0] = 0;
        K = 1;
    }
    int8_t remap[CWGPU_NUMRES];
    for (int c = 0; c < CWGPU_NUMRES; ++c) remap[c] = (int8_t)dense_of[c];
    std::vector<int8_t> dense;
    std::vector<int64_t> poffs;
    cwgpu::build_layout(
        nseqs, lens, [&](int s) { return lens[s] > 0 ? codes + offsets[s] : nullptr; }, remap, dense, poffs);
    // The device copy is made by the next call that needs it (stage_inputs),
    // in one copy together with the tables derived from params and matrix.
    ctx->host_layout.swap(dense);
    ctx->host_poffs.swap(poffs);
    ctx->nseqs = nseqs;
    ctx->lmax = lmax;
    ctx->lens.assign(lens, lens + nseqs);
    ctx->len_key.resize((size_t)nseqs);
    for (int s = 0; s < nseqs; ++s) ctx->len_key[(size_t)s] = (uint16_t)cwgpu::len_key(lens[s]);
    ctx->offs.swap(doffs);
    ctx->host_codes.swap(packed);
    ctx->codes_present = codes_present;
    ctx->K = K;
    memcpy(ctx->dense_of, dense_of, sizeof(dense_of));
    memcpy(ctx->code_of, code_of, sizeof(code_of));
    ctx->has_seqs = true;
    ctx->in_dirty = true;
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
        std::vector<int32_t> order((size_t)npairs);
        work_order(ctx, pairs, npairs, order.data(), &p->nlong);
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
    p->ctas = use_cta(ctx, p->nlong);
    *out = p;
    return CWGPU_OK;
}

int cwgpu_plan_launch(cwgpu_plan* p, void* stream) {
    if (!p) return CWGPU_ERR_ARG;
    cwgpu_context* ctx = p->ctx;
    if (p->generation != ctx->generation || ctx->in_dirty)
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

int cwgpu_plan_pair_ctas(const cwgpu_plan* p) { return p && p->ctas ? 1 : 0; }

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
    // Created on first use; each handle on its own, so a call after a failed
    // creation retries what is missing.
    if (!ctx->stream_short) CW_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream_short, cudaStreamNonBlocking));
    if (!ctx->ev_fork) CW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    if (!ctx->ev_join) CW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    // One buffer per call, filled and read back in one copy each way:
    //   in:  pair list, work order, zeroed queue counters, zeroed status word
    //   out: status word and distances (the statistics, if asked for, after them)
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t n = (size_t)npairs;
    const size_t o_order = up(8 * n), o_ctr = o_order + up(4 * n), o_err = o_ctr + 256;
    const size_t o_dist = o_err + 16, o_stats = up(o_dist + 4 * n);
    const size_t bytes_in = o_err + 16, bytes_out = 16 + 4 * n;
    const size_t total = o_stats + sizeof(cwgpu_pair_stats) * n;
    if (total > ctx->cap_call) {
        dfree(ctx->d_call);
        ctx->cap_call = 0;
        CW_CUDA(ctx, cudaMalloc(&ctx->d_call, total));
        ctx->cap_call = total;
    }
    CW_CUDA(ctx, pinned_grow(ctx->h_io, ctx->cap_h_io, total));
    int64_t nlong = 0;
    unsigned char* h = ctx->h_io;
    work_order(ctx, pairs, npairs, reinterpret_cast<int32_t*>(h + o_order), &nlong);
    memcpy(h, pairs, 8 * n);
    memset(h + o_ctr, 0, o_err + 16 - o_ctr);
    unsigned char* d = ctx->d_call;
    cudaStream_t s = ctx->stream;
    CW_CUDA(ctx, cudaMemcpyAsync(d, h, bytes_in, cudaMemcpyHostToDevice, s));
    cwgpu::PairArgs gl, gs;
    split_args(ctx, reinterpret_cast<const int32_t*>(d), reinterpret_cast<const int32_t*>(d + o_order), npairs, nlong,
               reinterpret_cast<float*>(d + o_dist),
               stats_out ? reinterpret_cast<cwgpu_pair_stats*>(d + o_stats) : nullptr, &gl, &gs);
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(d + o_ctr);
    int* err = reinterpret_cast<int*>(d + o_err);
    gl.counter = ctr;
    gl.cells = ctr + 1;
    gl.err = err;
    gs.counter = ctr + 4;
    gs.cells = ctr + 1;
    gs.err = err;
    CW_CUDA(ctx, enqueue_pairs(ctx, gl, gs, s, ctx->stream_short, ctx->ev_fork, ctx->ev_join, true));
    CW_CUDA(ctx, cudaMemcpyAsync(h + o_err, d + o_err, bytes_out, cudaMemcpyDeviceToHost, s));
    if (stats_out)
        CW_CUDA(ctx, cudaMemcpyAsync(h + o_stats, d + o_stats, sizeof(cwgpu_pair_stats) * n, cudaMemcpyDeviceToHost, s));
    CW_CUDA(ctx, cudaStreamSynchronize(s));
    int status = 0;
    memcpy(&status, h + o_err, 4);
    if (status) return status_error(ctx, status);
    memcpy(dist_out, h + o_dist, 4 * n);
    if (stats_out) memcpy(stats_out, h + o_stats, sizeof(cwgpu_pair_stats) * n);
    return CWGPU_OK;
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

int cwgpu_set_cta_tuning(cwgpu_context* ctx, const cwgpu_cta_tuning* t) {
    if (!ctx || !t) return CWGPU_ERR_ARG;
    const int w = t->warps;
    if (t->max_pairs < -1 || !(w == 0 || w == 2 || w == 4 || w == 8 || w == 16) ||
        (t->large_rows != 0 && t->large_rows < 2) || t->large_rows > CWGPU_MAX_SEQ_LEN)
        return fail(ctx, CWGPU_ERR_ARG,
                    "max_pairs must be >= -1, warps 0, 2, 4, 8 or 16, large_rows 0 or in [2, 65535]");
    ctx->cta_pairs = t->max_pairs;
    ctx->cta_warps = w;
    ctx->cta_large_rows = t->large_rows;
    ctx->generation++;
    return CWGPU_OK;
}

int cwgpu_get_cta_tuning(const cwgpu_context* ctx, cwgpu_cta_tuning* t) {
    if (!ctx || !t) return CWGPU_ERR_ARG;
    t->max_pairs = ctx->cta_pairs;
    t->warps = ctx->cta_warps;
    t->large_rows = ctx->cta_large_rows;
    return CWGPU_OK;
}

int cwgpu_cta_wait_probe(cwgpu_context* ctx, int64_t timeout_ns, int32_t* timed_out) {
    if (!ctx || !timed_out || timeout_ns < 1 || timeout_ns > 4000000000LL) return CWGPU_ERR_ARG;
    *timed_out = 0;
    CW_CUDA(ctx, cudaSetDevice(ctx->device));
    CW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int err = 0;
    CW_CUDA(ctx, cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return check_kernel_error(ctx);  // an earlier call's status first
    k_cta_wait_probe<<<1, 64, 0, ctx->stream>>>(ctx->d_err, (unsigned long long)timeout_ns);
    CW_CUDA(ctx, cudaGetLastError());
    CW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    CW_CUDA(ctx, cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    CW_CUDA(ctx, cudaMemset(ctx->d_err, 0, sizeof(int)));
    *timed_out = err == cwgpu::kStatusTimeout ? 1 : 0;
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
