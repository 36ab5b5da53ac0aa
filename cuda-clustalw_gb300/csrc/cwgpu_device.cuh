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
// All three dynamic-programming sweeps run on one primitive, `sweep`: a
// row-striped anti-diagonal wavefront. Lane l of a W-lane segment owns R
// consecutive rows of the current stripe and processes column c = t - l + 1
// at step t; the H and E values of the row above arrive from lane l-1 by
// __shfl_up_sync, the first lane reads them from the previous stripe's last
// row (a global buffer, L2-resident) or from a closed-form boundary. Integer
// recurrences use the DPX instructions (__viaddmax_s32, __vimax3_s32[_relu]).
// Scores come from a per-stripe int16 profile in shared memory
// (prof[code][lane][row]) so each step needs one conflict-free 8-byte load.
#pragma once

#include <climits>
#include <stdint.h>

#include "cwgpu.h"

namespace cwgpu {

constexpr unsigned kFull = 0xffffffffu;

// One rectangular sweep. Row r (0-based) uses residue rseq[r * rdir]; column c
// (1-based) uses residue cseq[(c - 1) * cdir]. Boundaries (closed form, which
// is what every sweep of the reference uses):
//   H(-1, c) = ht0 - c*hts        E(-1, c) = H(-1, c) - eo      (c >= 1)
//   H(r, 0)  = hl0 - (r+1)*hls    F(r, 0)  = H(r, 0) - fo
//   H(-1, 0) = 0
// For stripes after the first, H/E of the row above come from buf[c]. In
// MODE_GLOBAL the last row's H/E are left in buf[1..cols].
struct Task {
    const int8_t* rseq;
    const int8_t* cseq;
    int2* buf;
    int rdir, cdir;
    int rows, cols;
    int ht0, hts, eo;
    int hl0, hls, fo;
};

enum { MODE_LOCAL_FWD = 0, MODE_LOCAL_REV = 1, MODE_GLOBAL = 2 };

struct Best {
    int val;
    unsigned key;  // (row << 16) | col of the winning cell
};

template <int R>
__device__ __forceinline__ void unpack_scores(uint2 w, int (&s)[R]);

template <>
__device__ __forceinline__ void unpack_scores<4>(uint2 w, int (&s)[4]) {
    s[0] = (int)(int16_t)(w.x & 0xffffu);
    s[1] = ((int)w.x) >> 16;
    s[2] = (int)(int16_t)(w.y & 0xffffu);
    s[3] = ((int)w.y) >> 16;
}

// Fills this lane's slice of the stripe profile: prof[(b*32 + lane)*R + k] =
// matrix[a[k]][b] for all 32 codes b. Lane l starts at code l so the reads of
// the shared matrix hit 32 different banks.
template <int R>
__device__ __forceinline__ void build_profile(uint16_t* prof, const int* smat, const int (&a)[R],
                                              int lane) {
    static_assert(R == 4, "profile packing written for R == 4");
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
        const int b = (i + lane) & 31;
        const unsigned v0 = (unsigned)smat[a[0] * 32 + b] & 0xffffu;
        const unsigned v1 = (unsigned)smat[a[1] * 32 + b] & 0xffffu;
        const unsigned v2 = (unsigned)smat[a[2] * 32 + b] & 0xffffu;
        const unsigned v3 = (unsigned)smat[a[3] * 32 + b] & 0xffffu;
        *reinterpret_cast<uint2*>(prof + (b * 32 + lane) * R) = make_uint2(v0 | (v1 << 16), v2 | (v3 << 16));
    }
}

// The wavefront sweep. W = lanes per segment (32: one task per warp, 16: two
// tasks, one per half-warp). MODE_LOCAL_FWD tracks the first maximum in
// row-major order (forwardPass's strict `hh > maxScore`); MODE_LOCAL_REV
// tracks the first cell, in the sweep's own order, of the running maximum of
// min(H, thresh) (reversePass's strict `hh > cost` with its break at
// cost >= maxScore) and stops after the first stripe that reached thresh.
template <int R, int W, int MODE>
__device__ void sweep(const Task& T, int go, int ge, int thresh, uint16_t* prof, const int* smat,
                      Best& best) {
    const int lane = threadIdx.x & 31;
    const int sl = lane & (W - 1);
    const int goe = go + ge;
    constexpr int RPS = W * R;
    const int nstr = T.rows > 0 ? (T.rows + RPS - 1) / RPS : 0;
    const int nstr_max = __reduce_max_sync(kFull, nstr);
    const bool use_prof = T.cols >= 24;
    const bool use_prof_w = __all_sync(kFull, use_prof);
    best.val = 0;
    best.key = 0xffffffffu;

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

        int a[R];
#pragma unroll
        for (int k = 0; k < R; ++k) a[k] = (k < nvalid) ? (int)__ldg(T.rseq + (lrow0 + k) * T.rdir) : 0;
        if (use_prof_w) build_profile<R>(prof, smat, a, lane);
        __syncwarp();  // previous stripe's buf writes are visible to the first lane

        int hl[R], f[R], rm[R], rc[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            hl[k] = T.hl0 - (lrow0 + k + 1) * T.hls;
            f[k] = hl[k] - T.fo;
            rm[k] = 0;
            rc[k] = 0;
        }
        int diag = (lrow0 == 0) ? 0 : T.hl0 - lrow0 * T.hls;
        int hout = 0, eout = 0;

        for (int t = 0; t < nsteps_max; ++t) {
            const int c = t - sl + 1;
            int hin = __shfl_up_sync(kFull, hout, 1, W);
            int ein = __shfl_up_sync(kFull, eout, 1, W);
            if (c >= 1 && c <= T.cols && nvalid > 0) {
                if (sl == 0) {
                    if (s == 0) {
                        hin = T.ht0 - c * T.hts;
                        ein = hin - T.eo;
                    } else {
                        const int2 v = T.buf[c];
                        hin = v.x;
                        ein = v.y;
                    }
                }
                const int b = (int)__ldg(T.cseq + (c - 1) * T.cdir);
                int sc[R];
                if (use_prof_w) {
                    const uint2 w = *reinterpret_cast<const uint2*>(prof + (b * 32 + lane) * R);
                    unpack_scores<R>(w, sc);
                } else {
#pragma unroll
                    for (int k = 0; k < R; ++k) sc[k] = smat[a[k] * 32 + b];
                }
                int hup = hin, eup = ein, d = diag;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    if (k < nvalid) {
                        const int e = __viaddmax_s32(eup, -ge, hup - goe);
                        f[k] = __viaddmax_s32(f[k], -ge, hl[k] - goe);
                        int h;
                        if (MODE == MODE_LOCAL_FWD)
                            h = __vimax3_s32_relu(d + sc[k], e, f[k]);
                        else
                            h = __vimax3_s32(d + sc[k], e, f[k]);
                        d = hl[k];
                        hl[k] = h;
                        hup = h;
                        eup = e;
                        if (MODE == MODE_LOCAL_FWD) {
                            if (h > rm[k]) {
                                rm[k] = h;
                                rc[k] = c;
                            }
                        } else if (MODE == MODE_LOCAL_REV) {
                            const int hc = min(h, thresh);
                            if (hc > rm[k]) {
                                rm[k] = hc;
                                rc[k] = c;
                            }
                        }
                    }
                }
                hout = hup;
                eout = eup;
                diag = hin;
                if (writer) T.buf[c] = make_int2(hout, eout);
            }
        }

        if (MODE != MODE_GLOBAL) {
            // Earliest row of this lane with the lane's maximum (rows ascend with k).
            int lv = 0;
            unsigned lk = 0xffffffffu;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                if (k < nvalid && rm[k] > lv) {
                    lv = rm[k];
                    lk = ((unsigned)(lrow0 + k) << 16) | (unsigned)rc[k];
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
        __syncwarp();
    }
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
    int gp1, gp2;
};

// Myers-Miller recursion (FullPairwiseAlign.cpp:418-612) on an explicit stack
// held in registers (lane k holds frame k). Frames are independent once their
// (A, B, M, N, tb, te) are known, and the identity count and match count are
// sums over the M == 1 leaves, so the traversal order is free; the top frame's
// score is diff()'s return value. tb/te are always 0 or gapOpen, kept as flags.
// s1/s2 are 0-based code pointers: the reference's 1-based residue seq1[A + i]
// is s1[A + i - 1].
template <int R>
__device__ void mm_align(const int8_t* s1, const int8_t* s2, int A0, int B0, int M0, int N0, int go,
                         int ge, int gp1, int gp2, int2* bufA, int2* bufB, uint16_t* prof,
                         const int* smat, int* err, int& mm_score, int& n_ident, int& n_match,
                         long long& cells) {
    const int lane = threadIdx.x & 31;
    constexpr int NMASK = (1 << 29) - 1;
    int stA = 0, stB = 0, stM = 0, stN = 0;
    int sp = 0;
    if (lane == 0) {
        stA = A0;
        stB = B0;
        stM = M0;
        stN = N0 & NMASK;
    }
    sp = 1;
    bool top = true;
    int ident = 0, matches = 0, mm = 0;
    long long ncell = 0;  // diff() inner-loop iterations, counted as the reference runs them

    while (sp > 0) {
        --sp;
        const int A = __shfl_sync(kFull, stA, sp);
        const int B = __shfl_sync(kFull, stB, sp);
        const int M = __shfl_sync(kFull, stM, sp);
        const int NN = __shfl_sync(kFull, stN, sp);
        const int N = NN & NMASK;
        const int tbf = (NN >> 29) & 1, tef = (NN >> 30) & 1;
        const int tb = tbf ? go : 0, te = tef ? go : 0;

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
            // M == 1 (:443-477): best single column for residue A+1, first max.
            ncell += N;
            int midh = -(tb + ge) - (te + ge * N);
            const int hh0 = -(te + ge) - (tb + ge * N);
            if (hh0 > midh) midh = hh0;
            const int ra = (int)__ldg(s1 + A);
            int bv = INT_MIN, bj = 0x7fffffff;
            for (int j = lane + 1; j <= N; j += 32) {
                const int rb = (int)__ldg(s2 + B + j - 1);
                const int v = smat[ra * 32 + rb] - (N - j > 0 ? te + ge * (N - j) : 0) -
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
                const int rb = (int)__ldg(s2 + B + wj - 1);
                ++matches;
                if (ra != gp1 && rb != gp2 && ra == rb) ++ident;
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
            t.rdir = 1;
            t.cseq = s2 + B;
            t.cdir = 1;
            t.rows = midi;
            t.ht0 = -tb;
            t.hl0 = -tb;
            t.buf = bufA;
        } else {
            t.rseq = s1 + A + M - 1;
            t.rdir = -1;
            t.cseq = s2 + B + N - 1;
            t.cdir = -1;
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
        sweep<R, 16, MODE_GLOBAL>(t, go, ge, 0, prof, smat, unused);
        __syncwarp();

        // Midpoint scans (:570-593). Scan 1 keeps the first j reaching the
        // maximum of HH+RR, replaced by the last tied j with HH!=DD && RR==SS;
        // scan 2 switches to a type-2 midpoint at the largest j whose
        // DD+SS+gapOpen is strictly above that maximum.
        const int HH0 = -tb - midi * ge;       // HH[0] = DD[0]
        const int RRN = -te - (M - midi) * ge; // RR[N] = SS[N]
        int b1 = INT_MIN, j1 = 0x7fffffff, jc = -1, b2 = INT_MIN, j2 = -1;
        for (int j = lane; j <= N; j += 32) {
            int hh, dd, rr, ss;
            if (j == 0) {
                hh = dd = HH0;
            } else {
                const int2 v = bufA[j];
                hh = v.x;
                dd = v.y;
            }
            if (j == N) {
                rr = ss = RRN;
            } else {
                const int2 v = bufB[N - j];
                rr = v.x;
                ss = v.y;
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
        int midh = V, midj = max(J1, JC);
        bool type2 = false;
        if (W2 > midh) {
            midh = W2;
            midj = J2;
            type2 = true;
        }
        if (top) mm = midh;
        top = false;
        __syncwarp();  // scan reads of bufA/bufB finish before the next sweep writes

        // Push right then left so the left frame is processed first (:598-609).
        if (sp + 2 > 32) {
            if (lane == 0) atomicExch(err, 1);
            break;
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
                stN = (N - midj) | (0 << 29) | (tef << 30);
            }
            if (lane == sp + 1) {
                stA = A;
                stB = B;
                stM = midi - 1;
                stN = midj | (tbf << 29) | (0 << 30);
            }
        }
        sp += 2;
    }
    mm_score = mm;
    n_ident = ident;
    n_match = matches;
    cells = ncell;
}

// Aligns pair q: FullPairwiseAlign.cpp:112-183 for one (si, sj).
// Adds the pair's algorithmic cell counts (the inner-loop iterations the
// reference executes) to acc[0..2].
template <int R>
__device__ void align_pair(const PairArgs& g, long long q, uint16_t* prof, const int* smat, int2* bufA,
                           int2* bufB, unsigned long long (&acc)[3]) {
    const int lane = threadIdx.x & 31;
    const int si = g.pairs[2 * q], sj = g.pairs[2 * q + 1];
    const int n = g.lens[si], m = g.lens[sj];
    const int8_t* s1 = g.codes + g.offs[si];
    const int8_t* s2 = g.codes + g.offs[sj];
    const int go = g.go_table[min(n, m)];
    const int ge = g.ge;
    cwgpu_pair_stats st = {0, 0, 0, 0, 0, 0, 0, 0};
    float dist = 1.0f;
    if (n > 0 && m > 0) {
        // forwardPass
        Task t;
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
        Best fb;
        sweep<R, 32, MODE_LOCAL_FWD>(t, go, ge, 0, prof, smat, fb);
        const int max_score = fb.val;
        const int se1 = max_score > 0 ? (int)(fb.key >> 16) + 1 : 0;
        const int se2 = max_score > 0 ? (int)(fb.key & 0xffffu) : 0;
        __syncwarp();

        // reversePass
        int sb1 = 1, sb2 = 1;
        if (se1 > 0) {
            Task r;
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
            Best rb;
            sweep<R, 32, MODE_LOCAL_REV>(r, go, ge, max_score, prof, smat, rb);
            if (rb.val > 0) {
                sb1 = se1 - (int)(rb.key >> 16);
                sb2 = se2 - (int)(rb.key & 0xffffu) + 1;
            }
            // reversePass stops at the first cell reaching maxScore (:404-413).
            if (rb.val >= max_score)
                acc[1] += (unsigned long long)(se1 - sb1) * se2 + (unsigned long long)(se2 - sb2 + 1);
            else
                acc[1] += (unsigned long long)se1 * se2;
            __syncwarp();
        }
        acc[0] += (unsigned long long)n * m;

        // diff + tracePath
        int mm = 0, ident = 0, matches = 0;
        long long dcells = 0;
        mm_align<R>(s1, s2, sb1 - 1, sb2 - 1, se1 - sb1 + 1, se2 - sb2 + 1, go, ge, g.gp1, g.gp2, bufA,
                    bufB, prof, smat, g.err, mm, ident, matches, dcells);
        acc[2] += (unsigned long long)dcells;

        // distance (:170-181), float arithmetic with IEEE rounding.
        float mmv = (float)(100 * ident);
        const int len1 = g.nres[si], len2 = g.nres[sj];
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
        g.dist[q] = dist;
        if (g.stats) g.stats[q] = st;
    }
}

}  // namespace cwgpu
