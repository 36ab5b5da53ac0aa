// Device code of the full-pairwise distance stage for sm_103a.
//
// One warp aligns one sequence pair end to end, the way
// FullPairwiseAlign::pairwiseAlign does it per (si, sj)
// (CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.cpp:112-183):
//   1. forwardPass  (:280-341)  local Gotoh sweep, max score, first max cell
//   2. reversePass  (:343-416)  reverse sweep from the end cell, start cell
//   3. diff         (:418-612)  Myers-Miller recursion on the [sb..se] box
//   4. tracePath    (:231-278)  identity count, folded into diff's M==1 leaves
//   5. distance     (:172-181)  float arithmetic identical to the reference
//
// All dynamic-programming sweeps of steps 1-3 run on one primitive, `sweep`:
// a row-striped anti-diagonal wavefront. Lane l of a W-lane segment owns R
// consecutive rows of the current stripe and processes column c = t - l + 1 at
// step t. H and E of the row above arrive from lane l-1 by __shfl_up_sync; the
// segment's first lane takes them from the previous stripe's last row, which
// the segment reads W columns at a time with one coalesced load and hands to
// that lane by shuffle, or from the closed-form boundary of the first stripe.
//
// E and F are carried shifted by gapOpen+gapExtend (E' = E + goe, F' = F + goe)
// so each cell costs five integer operations, three of them DPX:
//   E'(r,c) = max(E'(r-1,c) - ge, H(r-1,c))                __viaddmax_s32
//   F'(r,c) = max(F'(r,c-1) - ge, H(r,c-1))                __viaddmax_s32
//   H(r,c)  = max(H(r-1,c-1) + s, max(E', F') - goe [, 0]) max + add + __viaddmax_s32[_relu]
// which is the reference's recurrence written with fewer operations.
//
// Scores come from a per-stripe int16 profile in shared memory,
// prof[code][lane][row], one conflict-free 16-byte load per step and lane
// (8 bytes in the short-pair kernel, whose lanes hold 4 rows).
// Residues are remapped on the host to the K codes that occur (K <= 32), so
// the profile holds K rows of codes.
//
// Myers-Miller frames small enough (M <= tiny_m, N <= tiny_n) are not swept
// by the warp: they are queued, and 32 of them at a time are solved one per
// lane with the reference's sequential loops, rows kept in the lane's column
// of the warp's shared scratch.
#pragma once

#include <climits>
#include <stdint.h>

#include "cwgpu.h"
#include "cwgpu_layout.h"

namespace cwgpu {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kR = 8;              // rows per lane in every sweep of long pairs
constexpr int kRShort = 4;         // rows per lane in the short-pair kernel
constexpr int kTinyMaxN = 16;      // tiny frames: N <= kTinyMaxN (shared-memory rows)
constexpr int kTinyStride = kTinyMaxN + 1;
constexpr int kTinyWords = 4 * kTinyStride * 32;  // HH, DD, RR, SS for 32 lanes
constexpr int kTinyStack = 16;

// Bytes of the per-warp shared region: the stripe profile or the tiny-frame rows.
__host__ __device__ constexpr int warp_region_bytes(int K) {
    return (K * 32 * kR * 2 > kTinyWords * 4) ? K * 32 * kR * 2 : kTinyWords * 4;
}

// One rectangular sweep. Row r (0-based) uses residue rseq[r]; column c
// (1-based) uses residue cseq[c - 1]. Sweeps that run backwards over a
// sequence read its reversed copy, so every sweep reads its residues in
// ascending address order. cseq[-kGuard .. cols + kGuard) must be readable.
// Closed-form boundaries, which is what every sweep of the reference uses:
//   H(-1, c) = ht0 - c*hts        E(-1, c) = H(-1, c) - eo      (c >= 1)
//   H(r, 0)  = hl0 - (r+1)*hls    F(r, 0)  = H(r, 0) - fo
//   H(-1, 0) = 0
// buf[c] (c = 1..cols) carries (H, E') of the last row of a stripe to the next
// stripe, and in MODE_GLOBAL holds the final row on return.
struct Task {
    const int8_t* rseq;
    const int8_t* cseq;
    int2* buf;
    int rows, cols;
    int ht0, hts, eo;
    int hl0, hls, fo;
};

enum { MODE_LOCAL_FWD = 0, MODE_LOCAL_REV = 1, MODE_GLOBAL = 2 };

struct Best {
    int val;
    unsigned key;  // (row << 16) | col of the winning cell
};

// Per-block constants the device functions read.
struct Env {
    const int* smat;     // shared 32x32 matrix over remapped codes
    uint16_t* region;    // this warp's shared region (profile or tiny rows)
    int K;               // number of remapped codes
    int gp1, gp2;        // remapped gapPos1 / gapPos2 (-1 if absent)
    int tiny_m, tiny_n;  // tiny-frame thresholds
    int* err;
};

template <int R>
struct SweepState {
    int hl[R];  // H(r, c-1)
    int fp[R];  // F'(r, c-1)
    int rm[R];  // tracked maximum per row
    int rc[R];  // its first column
    int diag;   // H of the row above the lane's first row, column c-1
    int hout, eout, thr;
    int ch, ce, nh, ne;  // boundary chunks: current and next W columns
};

// Residue load. NC: through the read-only data path (codes written before the
// kernel started); otherwise a plain load (codes the kernel itself wrote).
template <bool NC>
__device__ __forceinline__ int ldres(const int8_t* p) {
    if constexpr (NC)
        return (int)__ldg(p);
    else
        return (int)*p;
}

__device__ __forceinline__ void unpack2(unsigned w, int& lo, int& hi) {
    lo = (int)(int16_t)(w & 0xffffu);
    hi = ((int)w) >> 16;
}

// The R int16 scores of one (code, lane) profile entry: one 16-byte (R == 8)
// or 8-byte (R == 4) shared load.
template <int R>
__device__ __forceinline__ void load_scores(const uint16_t* p, int (&s)[R]) {
    static_assert(R == 8 || R == 4, "profile entries hold 4 or 8 rows");
    if constexpr (R == 8) {
        const uint4 w = *reinterpret_cast<const uint4*>(p);
        unpack2(w.x, s[0], s[1]);
        unpack2(w.y, s[2], s[3]);
        unpack2(w.z, s[4], s[5]);
        unpack2(w.w, s[6], s[7]);
    } else {
        const uint2 w = *reinterpret_cast<const uint2*>(p);
        unpack2(w.x, s[0], s[1]);
        unpack2(w.y, s[2], s[3]);
    }
}

__device__ __forceinline__ unsigned pack2(int lo, int hi) {
    return ((unsigned)lo & 0xffffu) | ((unsigned)hi << 16);
}

// prof[(b*32 + lane)*R + k] = matrix[a[k]][b] for the K codes b. Lane l starts
// at code l % K so that its shared-matrix reads spread over the banks.
template <int R>
__device__ __forceinline__ void build_profile(uint16_t* prof, const int* smat, const int (&a)[R], int lane,
                                              int K) {
    int b = lane % K;
    for (int i = 0; i < K; ++i) {
        if constexpr (R == 8) {
            uint4 w;
            w.x = pack2(smat[a[0] * 32 + b], smat[a[1] * 32 + b]);
            w.y = pack2(smat[a[2] * 32 + b], smat[a[3] * 32 + b]);
            w.z = pack2(smat[a[4] * 32 + b], smat[a[5] * 32 + b]);
            w.w = pack2(smat[a[6] * 32 + b], smat[a[7] * 32 + b]);
            *reinterpret_cast<uint4*>(prof + (b * 32 + lane) * 8) = w;
        } else {
            uint2 w;
            w.x = pack2(smat[a[0] * 32 + b], smat[a[1] * 32 + b]);
            w.y = pack2(smat[a[2] * 32 + b], smat[a[3] * 32 + b]);
            *reinterpret_cast<uint2*>(prof + (b * 32 + lane) * 4) = w;
        }
        b = (b + 1 == K) ? 0 : b + 1;
    }
}

// ---------------------------------------------------- warps sharing one sweep

// Device-side status values of the pair kernels' status word (nonzero = error).
enum { kStatusStackLimit = 1, kStatusTimeout = 2 };

// Hand-over of stripe boundary rows between the warps of a CTA that sweep one
// task together (stripes dealt round-robin). Warp w writes the last row of
// each of its stripes into its own row buffer and publishes how far it got in
// its progress word: epoch | stripe << 17 | columns written, which only grows
// (columns <= 65535, stripes <= 511, epochs count the CTA's sweeps). The warp
// with the next stripe waits for that word before it loads a chunk of the
// row. Every wait is bounded: past `limit_ns` it records kStatusTimeout, sets
// `abort`, and every later wait of the CTA returns at once, so the kernel
// ends (with wrong values that the host does not return).
struct MwSync {
    volatile unsigned long long* prog;  // shared: one progress word per warp of the CTA
    volatile int* abort;                // shared
    int* err;                           // global status word
    unsigned long long epoch;           // the sweep's epoch, shifted left by 32
    unsigned long long limit_ns;        // bound of one wait
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long mw_word(const MwSync& m, int stripe, int cols) {
    return m.epoch | ((unsigned long long)stripe << 17) | (unsigned)cols;
}

// Warp-uniform: lane 0 waits until progress word `slot` reaches `target`.
__device__ __forceinline__ void mw_wait(const MwSync& m, int slot, unsigned long long target) {
    if ((threadIdx.x & 31) == 0 && m.prog[slot] < target && !*m.abort) {
        const unsigned long long t0 = global_ns();
        for (unsigned polls = 1;; ++polls) {
            if (m.prog[slot] >= target || *m.abort) break;
            if ((polls & 63) == 0 && global_ns() - t0 > m.limit_ns) {
                *m.abort = 1;
                atomicExch(m.err, kStatusTimeout);
                break;
            }
        }
    }
    __threadfence_block();  // the row entries published before the word are read after it
    __syncwarp();
}

// One lane: the row entries it wrote are visible to the CTA before the word.
__device__ __forceinline__ void mw_publish(const MwSync& m, int slot, int stripe, int cols) {
    __threadfence_block();
    m.prog[slot] = mw_word(m, stripe, cols);
}

// Where a stripe's boundary rows come from and go to. Single-warp sweeps read
// and write one buffer; in a shared sweep the row above comes from the
// predecessor warp's buffer and the stripe's last row goes to the own one.
struct StripeIO {
    const int2* rbuf;
    int2* wbuf;
    int stripe;     // index of the stripe in the task
    int pred_slot;  // progress word of the warp with the previous stripe
    int own_slot;   // progress word of this warp
};

// The steps of one stripe. Lane sl processes column c = t - sl + 1 at step t.
// Lane 0 of the segment takes the row above from the chunk registers (W columns
// per lane-wide load: the previous stripe's last row, or the closed-form top
// boundary for the first stripe). PARTIAL: some rows of the stripe are past the
// task's last row; they pass the row above through so the segment's last used
// lane still emits the last real row. One loop body per (MODE, PARTIAL) keeps
// the hot code small enough for the instruction cache (unrolling the step loop
// made it slower for that reason); lanes outside their column range skip the
// body. The next step's residue is loaded one step ahead from the lane's own
// pointer, without clamping (the layout's guard bytes make the reads of fill
// and drain steps safe; those residues are never used).
// MW: the stripe is one of a sweep shared by several warps (MwSync): before a
// chunk of the row above is loaded the predecessor's progress is awaited, and
// the writer publishes its progress every W columns and at the last one.
template <int R, int W, int MODE, bool PARTIAL, bool NC, bool MW = false>
__device__ __forceinline__ void run_stripe(int nsteps, bool first, const Task& T, SweepState<R>& S, int sl,
                                           int nvalid, bool writer, int ge, int goe, int thresh,
                                           const uint16_t* prof_lane, const StripeIO& io = StripeIO{},
                                           const MwSync* mw = nullptr) {
    const unsigned ucols = (unsigned)T.cols;
    const int8_t* cp = T.cseq - sl;                 // residue of step t: cp[t]
    int2* wp = (MW ? io.wbuf : T.buf) + 1 - sl;     // boundary-row entry of step t: wp[t]
    const int2* rb = MW ? io.rbuf : T.buf;
    int bnext = ldres<NC>(cp);
    for (int t = 0; t < nsteps; ++t) {
        int hin = __shfl_up_sync(kFull, S.hout, 1, W);
        int ein = __shfl_up_sync(kFull, S.eout, 1, W);
        const int idx = t & (W - 1);
        const int bh = __shfl_sync(kFull, S.ch, idx, W);
        const int be = __shfl_sync(kFull, S.ce, idx, W);
        if (sl == 0) {
            hin = bh;
            ein = be;
        }
        if (idx == W - 1) {
            S.ch = S.nh;
            S.ce = S.ne;
            const int col = (t / W + 2) * W + 1 + sl;
            if (first) {
                S.nh = T.ht0 - col * T.hts;
                S.ne = S.nh - T.eo + goe;
            } else {
                if constexpr (MW) {
                    const int cfirst = (t / W + 2) * W + 1;
                    if (cfirst <= T.cols)
                        mw_wait(*mw, io.pred_slot, mw_word(*mw, io.stripe - 1, min(T.cols, cfirst + W - 1)));
                }
                if (col <= T.cols) {
                    const int2 v = rb[col];
                    S.nh = v.x;
                    S.ne = v.y;
                }
            }
        }
        const int b = bnext;
        bnext = ldres<NC>(cp + t + 1);
        if ((unsigned)(t - sl) < ucols) {
            int sc[R];
            load_scores<R>(prof_lane + b * (32 * R), sc);
            int hup = hin, eup = ein, d = S.diag;
            int hs[R];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                int e = __viaddmax_s32(eup, -ge, hup);
                const int f = __viaddmax_s32(S.fp[k], -ge, S.hl[k]);
                const int mx = max(e, f);
                int h;
                if (MODE == MODE_LOCAL_FWD)
                    h = __viaddmax_s32_relu(mx, -goe, d + sc[k]);
                else
                    h = __viaddmax_s32(mx, -goe, d + sc[k]);
                if (PARTIAL) {
                    const bool v = k < nvalid;
                    h = v ? h : hup;
                    e = v ? e : eup;
                }
                d = S.hl[k];
                S.hl[k] = h;
                S.fp[k] = f;
                hup = h;
                eup = e;
                hs[k] = h;
            }
            S.hout = hup;
            S.eout = eup;
            S.diag = hin;
            if (MODE != MODE_GLOBAL) {
                int sm = hs[0];
#pragma unroll
                for (int k = 1; k + 1 < R; k += 2) sm = __vimax3_s32(sm, hs[k], hs[k + 1]);
                if ((R & 1) == 0) sm = max(sm, hs[R - 1]);
                if (MODE == MODE_LOCAL_REV) sm = min(sm, thresh);
                if (sm >= S.thr) {
                    const int c = t - sl + 1;
#pragma unroll
                    for (int k = 0; k < R; ++k) {
                        const int hv = (MODE == MODE_LOCAL_REV) ? min(hs[k], thresh) : hs[k];
                        if (hv > S.rm[k]) {
                            S.rm[k] = hv;
                            S.rc[k] = c;
                        }
                    }
                    S.thr = sm;
                }
            }
            if (writer) {
                wp[t] = make_int2(hup, eup);
                if constexpr (MW) {
                    const int c = t - sl + 1;
                    if ((c & (W - 1)) == 0 || c == T.cols) mw_publish(*mw, io.own_slot, io.stripe, c);
                }
            }
        }
    }
}

// The wavefront sweep. W = lanes per segment (32: one task per warp, 16: two
// tasks, one per half-warp; the two tasks have the same column count).
// MODE_LOCAL_FWD tracks the first maximum in row-major order (forwardPass's
// strict `hh > maxScore`); MODE_LOCAL_REV tracks the first cell, in the sweep's
// row-major order, of the maximum of min(H, thresh) (reversePass's strict
// `hh > cost` and its break at cost >= maxScore) and stops after the first
// stripe that reached thresh. Tracking runs on the per-step maximum of the
// lane's rows; only when it reaches the lane's running maximum are the rows
// examined one by one.
template <int R, int W, int MODE, bool NC = true>
__device__ void sweep(const Task& T, int go, int ge, int thresh, const Env& X, Best& best) {
    const int lane = threadIdx.x & 31;
    const int sl = lane & (W - 1);
    const int goe = go + ge;
    constexpr int RPS = W * R;
    const int nstr = T.rows > 0 ? (T.rows + RPS - 1) / RPS : 0;
    const int nstr_max = __reduce_max_sync(kFull, nstr);
    const uint16_t* prof_lane = X.region + lane * R;
    best.val = 0;
    best.key = 0xffffffffu;
    SweepState<R> S;

    for (int s = 0; s < nstr_max; ++s) {
        const int srow0 = s * RPS;
        const int seg_rows = min(T.rows - srow0, RPS);
        const int lrow0 = srow0 + sl * R;
        const int nvalid = max(0, min(R, T.rows - lrow0));
        const int lused = seg_rows > 0 ? (seg_rows + R - 1) / R : 0;
        const int nsteps = (seg_rows > 0 && T.cols > 0) ? T.cols + lused - 1 : 0;
        const int nsteps_max = __reduce_max_sync(kFull, nsteps);
        const bool last = (s == nstr - 1);
        const bool writer = (sl == lused - 1) && (MODE == MODE_GLOBAL || !last);
        const bool full = __all_sync(kFull, seg_rows == RPS);

        int a[R];
#pragma unroll
        for (int k = 0; k < R; ++k) a[k] = (k < nvalid) ? ldres<NC>(T.rseq + lrow0 + k) : 0;
        __syncwarp();  // previous users of the shared region are done
        build_profile<R>(X.region, X.smat, a, lane, X.K);
        __syncwarp();  // previous stripe's buf writes visible to the whole segment

        const int gbest = best.val;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            S.hl[k] = T.hl0 - (lrow0 + k + 1) * T.hls;
            S.fp[k] = S.hl[k] - T.fo + goe;
            S.rm[k] = gbest;
            S.rc[k] = 0;
        }
        S.diag = (lrow0 == 0) ? 0 : T.hl0 - lrow0 * T.hls;
        S.hout = 0;
        S.eout = 0;
        S.thr = gbest + 1;
        const bool first = (s == 0);
        if (first) {
            S.ch = T.ht0 - (1 + sl) * T.hts;
            S.ce = S.ch - T.eo + goe;
            S.nh = T.ht0 - (W + 1 + sl) * T.hts;
            S.ne = S.nh - T.eo + goe;
        } else {
            S.ch = S.ce = S.nh = S.ne = 0;
            if (1 + sl <= T.cols) {
                const int2 v = T.buf[1 + sl];
                S.ch = v.x;
                S.ce = v.y;
            }
            if (W + 1 + sl <= T.cols) {
                const int2 v = T.buf[W + 1 + sl];
                S.nh = v.x;
                S.ne = v.y;
            }
        }
        if (full)
            run_stripe<R, W, MODE, false, NC>(nsteps_max, first, T, S, sl, nvalid, writer, ge, goe, thresh, prof_lane);
        else
            run_stripe<R, W, MODE, true, NC>(nsteps_max, first, T, S, sl, nvalid, writer, ge, goe, thresh, prof_lane);

        if (MODE != MODE_GLOBAL) {
            // Earliest row of this lane holding the lane's maximum (rows ascend with k).
            int lv = gbest;
            unsigned lk = 0xffffffffu;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                if (k < nvalid && S.rm[k] > lv) {
                    lv = S.rm[k];
                    lk = ((unsigned)(lrow0 + k) << 16) | (unsigned)S.rc[k];
                }
            }
            const int wv = __reduce_max_sync(kFull, lv);
            const unsigned wk = __reduce_min_sync(kFull, lv == wv ? lk : 0xffffffffu);
            if (wv > best.val) {  // later stripes hold later rows: strict keeps the first
                best.val = wv;
                best.key = wk;
            }
            if (MODE == MODE_LOCAL_REV && best.val >= thresh) break;
        }
    }
    __syncwarp();
}

// A sweep shared by the nw warps of a group (ranks 0..nw-1, CTA warps
// slot0 + rank): stripes of 32 x R rows are dealt round-robin, stripe s to rank
// s % nw, and each stripe's last row goes to the buffer of its warp,
// bufs + (slot0 + rank) * stride, from which the warp with the next stripe
// reads it (MwSync). Every warp tracks the best of its own stripes the way
// sweep() does (strict, so the first in row-major order); the caller reduces
// the ranks' results: maximum value, then lowest key. MODE_LOCAL_REV: *stop
// (shared, INT_MAX at the start) is lowered to every stripe that reached
// thresh; stripes above it are skipped (their progress is published as
// complete so no successor waits), which leaves the result of the lowest
// such stripe, reversePass's break cell. MODE_GLOBAL: the final row is in the
// buffer of rank (stripes - 1) % nw (see mw_last_rank).
__host__ __device__ inline int mw_stripes(int rows, int R) { return rows > 0 ? (rows + 32 * R - 1) / (32 * R) : 0; }

template <int R, int MODE, bool NC = true>
__device__ void sweep_mw(const Task& T, int go, int ge, int thresh, const Env& X, Best& best, int2* bufs,
                         size_t stride, int slot0, int rank, int nw, const MwSync& mw, volatile int* stop) {
    constexpr int W = 32;
    const int lane = threadIdx.x & 31;
    const int sl = lane;
    const int goe = go + ge;
    constexpr int RPS = W * R;
    const int nstr = mw_stripes(T.rows, R);
    const uint16_t* prof_lane = X.region + lane * R;
    best.val = 0;
    best.key = 0xffffffffu;
    if (T.cols <= 0) return;  // no column: nothing to hand over (callers give columns)
    SweepState<R> S;
    StripeIO io;
    io.wbuf = bufs + (size_t)(slot0 + rank) * stride;
    io.own_slot = slot0 + rank;

    for (int s = rank; s < nstr; s += nw) {
        io.stripe = s;
        io.pred_slot = slot0 + (s + nw - 1) % nw;
        io.rbuf = bufs + (size_t)io.pred_slot * stride;
        if (MODE == MODE_LOCAL_REV && __shfl_sync(kFull, *stop, 0) < s) {  // one decision per warp
            if (lane == 0) mw_publish(mw, io.own_slot, s, T.cols);
            continue;
        }
        const int srow0 = s * RPS;
        const int seg_rows = min(T.rows - srow0, RPS);
        const int lrow0 = srow0 + sl * R;
        const int nvalid = max(0, min(R, T.rows - lrow0));
        const int lused = (seg_rows + R - 1) / R;
        const int nsteps = T.cols > 0 ? T.cols + lused - 1 : 0;
        const bool last = (s == nstr - 1);
        const bool writer = (sl == lused - 1) && (MODE == MODE_GLOBAL || !last);
        const bool full = seg_rows == RPS;

        int a[R];
#pragma unroll
        for (int k = 0; k < R; ++k) a[k] = (k < nvalid) ? ldres<NC>(T.rseq + lrow0 + k) : 0;
        __syncwarp();
        build_profile<R>(X.region, X.smat, a, lane, X.K);
        __syncwarp();

        const int gbest = best.val;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            S.hl[k] = T.hl0 - (lrow0 + k + 1) * T.hls;
            S.fp[k] = S.hl[k] - T.fo + goe;
            S.rm[k] = gbest;
            S.rc[k] = 0;
        }
        S.diag = (lrow0 == 0) ? 0 : T.hl0 - lrow0 * T.hls;
        S.hout = 0;
        S.eout = 0;
        S.thr = gbest + 1;
        const bool first = (s == 0);
        if (first) {
            S.ch = T.ht0 - (1 + sl) * T.hts;
            S.ce = S.ch - T.eo + goe;
            S.nh = T.ht0 - (W + 1 + sl) * T.hts;
            S.ne = S.nh - T.eo + goe;
        } else {
            mw_wait(mw, io.pred_slot, mw_word(mw, s - 1, min(T.cols, 2 * W)));
            S.ch = S.ce = S.nh = S.ne = 0;
            if (1 + sl <= T.cols) {
                const int2 v = io.rbuf[1 + sl];
                S.ch = v.x;
                S.ce = v.y;
            }
            if (W + 1 + sl <= T.cols) {
                const int2 v = io.rbuf[W + 1 + sl];
                S.nh = v.x;
                S.ne = v.y;
            }
        }
        if (full)
            run_stripe<R, W, MODE, false, NC, true>(nsteps, first, T, S, sl, nvalid, writer, ge, goe, thresh,
                                                    prof_lane, io, &mw);
        else
            run_stripe<R, W, MODE, true, NC, true>(nsteps, first, T, S, sl, nvalid, writer, ge, goe, thresh,
                                                   prof_lane, io, &mw);

        if (MODE != MODE_GLOBAL) {
            int lv = gbest;
            unsigned lk = 0xffffffffu;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                if (k < nvalid && S.rm[k] > lv) {
                    lv = S.rm[k];
                    lk = ((unsigned)(lrow0 + k) << 16) | (unsigned)S.rc[k];
                }
            }
            const int wv = __reduce_max_sync(kFull, lv);
            const unsigned wk = __reduce_min_sync(kFull, lv == wv ? lk : 0xffffffffu);
            if (wv > best.val) {
                best.val = wv;
                best.key = wk;
            }
            if (MODE == MODE_LOCAL_REV && wv >= thresh && lane == 0) atomicMin((int*)stop, s);
        }
    }
    __syncwarp();
}

__host__ __device__ inline int mw_last_rank(int rows, int R, int nw) { return (mw_stripes(rows, R) - 1) % nw; }

// ---------------------------------------------------------------- tiny frames

// Sequential Myers-Miller (FullPairwiseAlign.cpp:418-612) on one lane for one
// frame and its whole subtree. Rows live in this lane's column of the warp's
// shared scratch (word j*32 + lane, conflict-free), the frame stack in local
// memory. Returns the frame's score; adds identities, matches and diff()
// inner-loop iterations.
template <bool NC>
static __device__ int lane_mm(const int8_t* s1, const int8_t* s2, int A0, int B0, int M0, int N0, int tbf0, int tef0, int go,
                       int ge, const Env& X, int* scratch, int& ident, int& matches, long long& cells) {
    const int lane = threadIdx.x & 31;
    int* HH = scratch + lane;
    int* DD = HH + kTinyStride * 32;
    int* RR = DD + kTinyStride * 32;
    int* SS = RR + kTinyStride * 32;
#define TI(arr, j) arr[(j) * 32]
    int4 stk[kTinyStack];
    int sp = 0;
    stk[sp++] = make_int4(A0, B0, M0, N0 | (tbf0 << 29) | (tef0 << 30));
    int root_score = 0;
    bool root = true;
    while (sp > 0) {
        const int4 fr = stk[--sp];
        const int A = fr.x, B = fr.y, M = fr.z;
        const int N = fr.w & ((1 << 29) - 1);
        const int tbf = (fr.w >> 29) & 1, tef = (fr.w >> 30) & 1;
        const int tb = tbf ? go : 0, te = tef ? go : 0;
        int midh;
        if (N <= 0) {
            midh = -(M > 0 ? tb + ge * M : 0);
        } else if (M <= 1) {
            if (M <= 0) {
                midh = -(tb + ge * N);
            } else {
                cells += N;
                midh = -(tb + ge) - (te + ge * N);
                const int hh0 = -(te + ge) - (tb + ge * N);
                if (hh0 > midh) midh = hh0;
                int midj = 0;
                const int* row = X.smat + 32 * ldres<NC>(s1 + A);
                for (int j = 1; j <= N; ++j) {
                    const int hh = row[ldres<NC>(s2 + B + j - 1)] - (N - j > 0 ? te + ge * (N - j) : 0) -
                                   (j - 1 > 0 ? tb + ge * (j - 1) : 0);
                    if (hh > midh) {
                        midh = hh;
                        midj = j;
                    }
                }
                if (midj > 0) {
                    ++matches;
                    const int ra = ldres<NC>(s1 + A), rb = ldres<NC>(s2 + B + midj - 1);
                    if (ra != X.gp1 && rb != X.gp2 && ra == rb) ++ident;
                }
            }
        } else {
            cells += (long long)M * N;
            const int midi = M / 2;
            int t = -tb;
            TI(HH, 0) = 0;
            for (int j = 1; j <= N; ++j) {
                t -= ge;
                TI(HH, j) = t;
                TI(DD, j) = t - go;
            }
            t = -tb;
            for (int i = 1; i <= midi; ++i) {
                const int* row = X.smat + 32 * ldres<NC>(s1 + A + i - 1);
                int s = TI(HH, 0);
                int hh = t = t - ge;
                TI(HH, 0) = hh;
                int f = t - go;
                for (int j = 1; j <= N; ++j) {
                    f = max(f - ge, hh - go - ge);
                    const int e = max(TI(DD, j) - ge, TI(HH, j) - go - ge);
                    hh = max(max(s + row[ldres<NC>(s2 + B + j - 1)], f), e);
                    s = TI(HH, j);
                    TI(HH, j) = hh;
                    TI(DD, j) = e;
                }
            }
            TI(DD, 0) = TI(HH, 0);
            TI(RR, N) = 0;
            t = -te;
            for (int j = N - 1; j >= 0; --j) {
                t -= ge;
                TI(RR, j) = t;
                TI(SS, j) = t - go;
            }
            t = -te;
            for (int i = M - 1; i >= midi; --i) {
                const int* row = X.smat + 32 * ldres<NC>(s1 + A + i);
                int s = TI(RR, N);
                int hh = t = t - ge;
                TI(RR, N) = hh;
                int f = t - go;
                for (int j = N - 1; j >= 0; --j) {
                    f = max(f - ge, hh - go - ge);
                    const int e = max(TI(SS, j) - ge, TI(RR, j) - go - ge);
                    hh = max(max(s + row[ldres<NC>(s2 + B + j)], f), e);
                    s = TI(RR, j);
                    TI(RR, j) = hh;
                    TI(SS, j) = e;
                }
            }
            TI(SS, N) = TI(RR, N);
            midh = TI(HH, 0) + TI(RR, 0);
            int midj = 0;
            bool type2 = false;
            for (int j = 0; j <= N; ++j) {
                const int hh = TI(HH, j) + TI(RR, j);
                if (hh >= midh)
                    if (hh > midh || (TI(HH, j) != TI(DD, j) && TI(RR, j) == TI(SS, j))) {
                        midh = hh;
                        midj = j;
                    }
            }
            for (int j = N; j >= 0; --j) {
                const int hh = TI(DD, j) + TI(SS, j) + go;
                if (hh > midh) {
                    midh = hh;
                    midj = j;
                    type2 = true;
                }
            }
            if (sp + 2 > kTinyStack) {
                atomicExch(X.err, 1);
                break;
            }
            if (!type2) {
                stk[sp++] = make_int4(A + midi, B + midj, M - midi, (N - midj) | (1 << 29) | (tef << 30));
                stk[sp++] = make_int4(A, B, midi, midj | (tbf << 29) | (1 << 30));
            } else {
                stk[sp++] = make_int4(A + midi + 1, B + midj, M - midi - 1, (N - midj) | (tef << 30));
                stk[sp++] = make_int4(A, B, midi - 1, midj | (tbf << 29));
            }
        }
        if (root) root_score = midh;
        root = false;
    }
#undef TI
    return root_score;
}

// ---------------------------------------------------------------- diff()

// A CTA's shared stack of Myers-Miller frames (used by the one-CTA-per-pair
// kernel): frames (A, B, M, N | tb << 29 | te << 30) that any warp of the CTA
// may take; count and lock live in shared memory, the lock taken by one lane.
struct FrameShare {
    int4* frames;
    volatile int* count;
    int* lock;
    int cap;
    int min_rows;  // frames with fewer rows stay with the warp that made them
};

// Lane 0: pushes f if the stack has room and its lock is free within a few
// tries; returns whether it did (else the caller keeps the frame).
__device__ __forceinline__ bool share_push(const FrameShare& fs, int4 f) {
    for (int tries = 0; tries < 64; ++tries) {
        if (atomicCAS(fs.lock, 0, 1) == 0) {
            __threadfence_block();
            bool ok = false;
            const int c = *fs.count;
            if (c < fs.cap) {
                fs.frames[c] = f;
                __threadfence_block();
                *fs.count = c + 1;
                ok = true;
            }
            __threadfence_block();
            atomicExch(fs.lock, 0);
            return ok;
        }
    }
    return false;
}

// Midpoint scans of a Myers-Miller frame (FullPairwiseAlign.cpp:570-593), by
// one warp. fwd[j] holds (HH, DD + goe) of row midi from the forward half,
// rev[N - j] holds (RR, SS + goe) of the same row from the reverse half (j =
// 1..N and 0..N-1; the other ends are closed-form). Scan 1 keeps the first j
// reaching the maximum of HH+RR, replaced by the last tied j with HH!=DD &&
// RR==SS; scan 2 switches to a type-2 midpoint at the largest j whose
// DD+SS+gapOpen is strictly above that maximum.
__device__ __forceinline__ void midpoint_scan(const int2* fwd, const int2* rev, int M, int N, int midi, int tb, int te,
                                              int go, int ge, int& midh, int& midj, bool& type2) {
    const int lane = threadIdx.x & 31;
    const int goe = go + ge;
    const int HH0 = -tb - midi * ge;        // HH[0] = DD[0]
    const int RRN = -te - (M - midi) * ge;  // RR[N] = SS[N]
    int b1 = INT_MIN, j1 = 0x7fffffff, jc = -1, b2 = INT_MIN, j2 = -1;
    for (int j = lane; j <= N; j += 32) {
        int hh, dd, rr, ss;
        if (j == 0) {
            hh = dd = HH0;
        } else {
            const int2 v = fwd[j];
            hh = v.x;
            dd = v.y - goe;
        }
        if (j == N) {
            rr = ss = RRN;
        } else {
            const int2 v = rev[N - j];
            rr = v.x;
            ss = v.y - goe;
        }
        const int v1 = hh + rr;
        const bool cond = (hh != dd) && (rr == ss);
        if (v1 > b1) {
            b1 = v1;
            j1 = j;
            jc = cond ? j : -1;
        } else if (v1 == b1 && cond) {
            jc = j;
        }
        const int v2 = dd + ss + go;
        if (v2 >= b2) {
            b2 = v2;
            j2 = j;
        }
    }
    const int V = __reduce_max_sync(kFull, b1);
    const int J1 = (int)__reduce_min_sync(kFull, b1 == V ? (unsigned)j1 : 0x7fffffffu);
    const int JC = __reduce_max_sync(kFull, b1 == V ? jc : -1);
    const int W2 = __reduce_max_sync(kFull, b2);
    const int J2 = __reduce_max_sync(kFull, b2 == W2 ? j2 : -1);
    midh = V;
    midj = max(J1, JC);
    type2 = false;
    if (W2 > midh) {
        midh = W2;
        midj = J2;
        type2 = true;
    }
}

// Myers-Miller recursion (FullPairwiseAlign.cpp:418-612) for one pair. Large
// frames are divided by the warp: forward half on lanes 0-15 and reverse half
// on lanes 16-31, then the midpoint scans as warp reductions. Frames go on an
// explicit stack held in registers (lane k holds frame k); tiny frames go on a
// queue (lane k holds entry k) that is solved 32 at a time by lane_mm. Frames
// are independent once (A, B, M, N, tb, te) are known, and the identity and
// match counts are sums over the M == 1 leaves, so the traversal order is
// free; the top frame's score is diff()'s return value. tb/te are always 0 or
// gapOpen, kept as flags. s1/s2 are 0-based: the reference's 1-based residue
// seq1[A + i] is s1[A + i - 1]. s1r/s2r are the reversed copies of the n- and
// m-residue sequences (s1r[i] = s1[n - 1 - i]), which the reverse halves read.
// N0 carries the top frame's flags: tb = gapOpen if bit 29, te if bit 30 (a
// whole pair's frame has neither). SHARE: after each division the right child,
// if it has at least fs->min_rows rows, goes to the CTA's shared stack (when
// it has room) for any warp of the CTA to take, instead of this warp's own.
template <int RS, bool NC = true, bool SHARE = false>
static __device__ void mm_align(const int8_t* s1, const int8_t* s1r, int n, const int8_t* s2, const int8_t* s2r, int m,
                                int A0, int B0, int M0, int N0, int go, int ge, int2* bufA, int2* bufB, const Env& X,
                                int& mm_score, int& n_ident, int& n_match, long long& cells,
                                const FrameShare* fs = nullptr) {
    const int lane = threadIdx.x & 31;
    constexpr int NMASK = (1 << 29) - 1;
    int stA = 0, stB = 0, stM = 0, stN = 0;  // stack entry `lane`
    int qA = 0, qB = 0, qM = 0, qN = 0;      // tiny-queue entry `lane`
    if (lane == 0) {
        stA = A0;
        stB = B0;
        stM = M0;
        stN = N0;
    }
    int sp = 1, nq = 0;
    bool top = true;
    int ident = 0, matches = 0, mm = 0;
    long long ncell = 0;
    bool q_has_top = false;  // queue entry 0 is the top frame

    while (sp > 0 || nq > 0) {
        if (sp == 0 || nq == 32) {
            // Solve the queued tiny frames, one per lane.
            __syncwarp();
            int li = 0, lm = 0, score = 0;
            long long lc = 0;
            if (lane < nq) {
                score = lane_mm<NC>(s1, s2, qA, qB, qM, qN & NMASK, (qN >> 29) & 1, (qN >> 30) & 1, go, ge, X,
                                reinterpret_cast<int*>(X.region), li, lm, lc);
            }
            __syncwarp();
            ident += __reduce_add_sync(kFull, li);
            matches += __reduce_add_sync(kFull, lm);
            ncell += (long long)__reduce_add_sync(kFull, (unsigned)lc);
            if (q_has_top) mm = __shfl_sync(kFull, score, 0);
            q_has_top = false;
            nq = 0;
            continue;
        }
        --sp;
        const int A = __shfl_sync(kFull, stA, sp);
        const int B = __shfl_sync(kFull, stB, sp);
        const int M = __shfl_sync(kFull, stM, sp);
        const int NN = __shfl_sync(kFull, stN, sp);
        const int N = NN & NMASK;
        const int tbf = (NN >> 29) & 1, tef = (NN >> 30) & 1;
        const int tb = tbf ? go : 0, te = tef ? go : 0;

        if (M <= X.tiny_m && N <= X.tiny_n) {
            if (lane == nq) {
                qA = A;
                qB = B;
                qM = M;
                qN = NN;
            }
            if (top) q_has_top = true;  // only possible as entry 0
            top = false;
            ++nq;
            continue;
        }
        if (N <= 0) {  // del(M); return -tbgap(M, tb)
            if (top) mm = -(M > 0 ? tb + ge * M : 0);
            top = false;
            continue;
        }
        if (M <= 1) {
            if (M <= 0) {  // add(N); return -tbgap(N, tb)
                if (top) mm = -(tb + ge * N);
                top = false;
                continue;
            }
            // M == 1 with a long row (:443-477): best single column, first max.
            ncell += N;
            int midh = -(tb + ge) - (te + ge * N);
            const int hh0 = -(te + ge) - (tb + ge * N);
            if (hh0 > midh) midh = hh0;
            const int ra = ldres<NC>(s1 + A);
            int bv = INT_MIN, bj = 0x7fffffff;
            for (int j = lane + 1; j <= N; j += 32) {
                const int rb = ldres<NC>(s2 + B + j - 1);
                const int v = X.smat[ra * 32 + rb] - (N - j > 0 ? te + ge * (N - j) : 0) -
                              (j - 1 > 0 ? tb + ge * (j - 1) : 0);
                if (v > bv) {
                    bv = v;
                    bj = j;
                }
            }
            const int wv = __reduce_max_sync(kFull, bv);
            const int wj = (int)__reduce_min_sync(kFull, bv == wv ? (unsigned)bj : 0x7fffffffu);
            if (wv > midh) {
                midh = wv;
                const int rb = ldres<NC>(s2 + B + wj - 1);
                ++matches;
                if (ra != X.gp1 && rb != X.gp2 && ra == rb) ++ident;
            }
            if (top) mm = midh;
            top = false;
            continue;
        }

        // Divide (:480-593): forward half on lanes 0-15, reverse half on 16-31.
        const int midi = M / 2;
        ncell += (long long)M * N;
        Task t;
        if (lane < 16) {
            t.rseq = s1 + A;
            t.cseq = s2 + B;
            t.rows = midi;
            t.ht0 = -tb;
            t.hl0 = -tb;
            t.buf = bufA;
        } else {
            // rows A+M-1 down to A+midi and columns B+N-1 down to B, read in
            // ascending order from the reversed copies
            t.rseq = s1r + (n - A - M);
            t.cseq = s2r + (m - B - N);
            t.rows = M - midi;
            t.ht0 = -te;
            t.hl0 = -te;
            t.buf = bufB;
        }
        t.cols = N;
        t.hts = ge;
        t.eo = go;
        t.hls = ge;
        t.fo = go;
        Best unused;
        sweep<RS, 16, MODE_GLOBAL, NC>(t, go, ge, 0, X, unused);

        int midh, midj;
        bool type2;
        midpoint_scan(bufA, bufB, M, N, midi, tb, te, go, ge, midh, midj, type2);
        if (top) mm = midh;
        top = false;
        __syncwarp();  // scan reads of bufA/bufB finish before the next sweep writes

        // Push right then left so the left frame is processed first (:598-609).
        if (sp + 2 > 32) {
            if (lane == 0) atomicExch(X.err, 1);
            break;
        }
        if constexpr (SHARE) {
            const int4 right = !type2 ? make_int4(A + midi, B + midj, M - midi, (N - midj) | (1 << 29) | (tef << 30))
                                      : make_int4(A + midi + 1, B + midj, M - midi - 1, (N - midj) | (tef << 30));
            int shared = 0;
            if (lane == 0 && right.z >= fs->min_rows) shared = share_push(*fs, right) ? 1 : 0;
            if (__shfl_sync(kFull, shared, 0)) {
                if (lane == sp) {
                    stA = A;
                    stB = B;
                    stM = !type2 ? midi : midi - 1;
                    stN = !type2 ? (midj | (tbf << 29) | (1 << 30)) : (midj | (tbf << 29));
                }
                sp += 1;
                continue;
            }
        }
        if (!type2) {
            if (lane == sp) {
                stA = A + midi;
                stB = B + midj;
                stM = M - midi;
                stN = (N - midj) | (1 << 29) | (tef << 30);
            }
            if (lane == sp + 1) {
                stA = A;
                stB = B;
                stM = midi;
                stN = midj | (tbf << 29) | (1 << 30);
            }
        } else {
            if (lane == sp) {
                stA = A + midi + 1;
                stB = B + midj;
                stM = M - midi - 1;
                stN = (N - midj) | (tef << 30);
            }
            if (lane == sp + 1) {
                stA = A;
                stB = B;
                stM = midi - 1;
                stN = midj | (tbf << 29);
            }
        }
        sp += 2;
    }
    mm_score = mm;
    n_ident = ident;
    n_match = matches;
    cells = ncell;
}

struct PairArgs {
    const int8_t* codes;
    const int64_t* offs;
    const int32_t* lens;
    const int32_t* nres;
    const int32_t* pairs;
    const int32_t* order;
    const int32_t* go_table;
    const int32_t* matrix;
    float* dist;
    cwgpu_pair_stats* stats;
    int2* scratch;
    unsigned long long* counter;
    int* err;
    unsigned long long* cells;  // [3]: forward, reverse (up to its break), diff
    long long npairs;
    int lmax;
    int ge;
    int gp1, gp2;  // remapped gap codes
    int K;         // remapped alphabet size
    int tiny_m, tiny_n;
};

// forwardPass + reversePass + diff + distance for one pair, given its 0-based
// code pointers, lengths, non-gap residue counts and gap penalties. Returns
// the distance and fills `st`; adds the algorithmic cell counts (the
// inner-loop iterations the reference executes) to acc[0..2]. RS = rows per
// lane in every sweep: any RS gives the same results; kRShort needs fewer
// warp steps when n <= 128 (one stripe, lanes of 4 rows instead of
// half-empty lanes of 8). Each sequence's reversed copy follows it at the
// next 16-byte boundary (cwgpu_layout.h), and kGuard readable bytes surround both.
__device__ __forceinline__ const int8_t* rev_of(const int8_t* s, int len) { return s + rev_offset(len); }

template <int RS = kR, bool NC = true>
static __device__ float align_one(const int8_t* s1, int n, const int8_t* s2, int m, int len1, int len2, int go, int ge,
                           int2* bufA, int2* bufB, const Env& X, cwgpu_pair_stats& st, unsigned long long (&acc)[3]) {
    const int8_t* s1r = rev_of(s1, n);
    const int8_t* s2r = rev_of(s2, m);
    st = cwgpu_pair_stats{0, 0, 0, 0, 0, 0, 0, 0};
    if (n <= 0 || m <= 0) return 1.0f;
    // forwardPass
    Task t;
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
    t.buf = bufA;
    Best fb;
    sweep<RS, 32, MODE_LOCAL_FWD, NC>(t, go, ge, 0, X, fb);
    const int max_score = fb.val;
    const int se1 = max_score > 0 ? (int)(fb.key >> 16) + 1 : 0;
    const int se2 = max_score > 0 ? (int)(fb.key & 0xffffu) : 0;

    // reversePass
    int sb1 = 1, sb2 = 1;
    if (se1 > 0) {
        Task r;
        r.rseq = s1r + (n - se1);  // rows se1-1 .. 0 of s1
        r.cseq = s2r + (m - se2);  // columns se2 .. 1
        r.rows = se1;
        r.cols = se2;
        r.ht0 = -1;
        r.hts = 0;
        r.eo = 0;
        r.hl0 = -1;
        r.hls = 0;
        r.fo = 0;
        r.buf = bufA;
        Best rb;
        sweep<RS, 32, MODE_LOCAL_REV, NC>(r, go, ge, max_score, X, rb);
        if (rb.val > 0) {
            sb1 = se1 - (int)(rb.key >> 16);
            sb2 = se2 - (int)(rb.key & 0xffffu) + 1;
        }
        // reversePass stops at the first cell reaching maxScore (:404-413).
        if (rb.val >= max_score)
            acc[1] += (unsigned long long)(se1 - sb1) * se2 + (unsigned long long)(se2 - sb2 + 1);
        else
            acc[1] += (unsigned long long)se1 * se2;
    }
    acc[0] += (unsigned long long)n * m;

    // diff + tracePath
    int mm = 0, ident = 0, matches = 0;
    long long dcells = 0;
    mm_align<RS, NC>(s1, s1r, n, s2, s2r, m, sb1 - 1, sb2 - 1, se1 - sb1 + 1, se2 - sb2 + 1, go, ge, bufA, bufB, X, mm,
                 ident, matches, dcells);
    acc[2] += (unsigned long long)dcells;

    // distance (:170-181), float arithmetic with IEEE rounding.
    float mmv = (float)(100 * ident);
    if (len1 == 0 || len2 == 0)
        mmv = 0.0f;
    else
        mmv = __fdiv_rn(mmv, (float)min(len1, len2));
    st.fwd_score = max_score;
    st.se1 = se1;
    st.se2 = se2;
    st.sb1 = sb1;
    st.sb2 = sb2;
    st.mm_score = mm;
    st.n_ident = ident;
    st.n_match = matches;
    return __fdiv_rn(__fsub_rn(100.0f, mmv), 100.0f);
}

// Aligns pair q: FullPairwiseAlign.cpp:112-183 for one (si, sj).
template <int RS = kR>
static __device__ void align_pair(const PairArgs& g, long long q, const Env& X, int2* bufA, int2* bufB,
                           unsigned long long (&acc)[3]) {
    const int lane = threadIdx.x & 31;
    const int si = g.pairs[2 * q], sj = g.pairs[2 * q + 1];
    const int n = g.lens[si], m = g.lens[sj];
    cwgpu_pair_stats st;
    const float dist = align_one<RS>(g.codes + g.offs[si], n, g.codes + g.offs[sj], m, g.nres[si], g.nres[sj],
                                 g.go_table[min(n, m)], g.ge, bufA, bufB, X, st, acc);
    if (lane == 0) {
        g.dist[q] = dist;
        if (g.stats) g.stats[q] = st;
    }
}

}  // namespace cwgpu
