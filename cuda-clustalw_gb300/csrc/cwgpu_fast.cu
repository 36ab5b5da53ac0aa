// cwgpu_fast.cu - quick k-tuple distances (ClustalW's FastPairwiseAlign) on sm_103a.
//
// Computes what clustalw::FastPairwiseAlign::pairwiseAlign computes
// (CPU/clustalw-2.0.11/src/pairwise/FastPairwiseAlign.cpp:20-400) for every
// pair, bit-identically: the Wilbur-Lipman k-tuple diagonal method. Per pair:
//   count    k-tuple hits per diagonal (vn1 - vn2 + l2)               :198-219
//   select   the top `signif` diagonals after the reference's quicksort :221-241
//   flag     diagonals within `window` of a selected one
//   chain    for every k-tuple of seq 1 (ascending) and every match in
//            seq 2 (descending position) on a flagged diagonal, the A-loop
//            that extends or opens a fragment, fragments kept in a list
//            sorted by score (putFrag)                                  :246-398
//   score    the best fragment's score, as percent of the shorter length
//
// GB300 form: one warp per pair (a CTA of 32 threads), pairs taken longest
// first from an atomic queue. The lanes count hits with shared-memory
// atomics (16-bit counts, two per word) over per-sequence k-tuple position
// lists (built once per sequence set by k_fast_prep), select the top
// diagonals in parallel, and enumerate the flagged matches of each k-tuple in
// the reference's order. The fragment list is walked and updated by the whole
// warp: its top 32 entries in registers, the next ones as records in shared
// memory, the low-score tail in a per-warp global array. The chain is a
// dependent sequence of short steps, so throughput comes from pairs in
// flight: about 7 KB of shared memory per pair at 1,500 residues lets 28
// pairs share an SM.
//
// Selection: the reference sorts the diagonal counts of positions
// 1..tl1-1 ascending with its own quicksort and flags around the diagonals that
// land in positions tl1-signif+1..tl1 (position tl1 itself is never sorted).
// Only which diagonals land there matters. When the boundary value of the top
// positions is not shared by more diagonals than fit, that set is every
// diagonal above (or at) the boundary and no sort is needed; otherwise lane 0
// replays the reference's quicksort, restricted to the sub-ranges that contain
// top positions (the other sub-ranges cannot change them).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "cwgpu.h"
#include "cwgpu_context.h"
#include "cwgpu_ranges.h"

namespace cwfast {

constexpr int kMaxLimit = 4096;  // k-tuple codes (25^2 protein, 4^6 DNA)
constexpr int kMaxLen = 8191;    // longest sequence (16-bit fields, fs <= ktup * L < 2^15)

struct Params {
    int dna, ktup, window, window_gap, signif, percent, max_aa, max_aln;
    int limit;  // number of k-tuple codes
    int pot[8];
};

// DNA residue codes of the reference's mask (FastPairwiseAlign.cpp:163-164):
// A C G T U -> 0 1 2 3 3, anything else invalid.
__device__ __forceinline__ int aa2dna(int c) {
    return c == 0 ? 0 : c == 2 ? 1 : c == 6 ? 2 : (c == 18 || c == 19) ? 3 : -1;
}

// Per sequence: kcode[p] = 1 + k-tuple code of the k-tuple starting at
// 0-based position p (0 if it has an invalid residue or runs off the end),
// and the 1-based positions of every code, grouped by code (CSR): positions of
// code c are pos[start[c] .. start[c+1]) in sequence-local indices.
__global__ void k_fast_prep(const int8_t* orig, const int64_t* offs, const int32_t* lens, Params P,
                            int16_t* kcode, uint16_t* pos, int32_t* start) {
    extern __shared__ int hist[];  // limit + 2
    const int s = blockIdx.x;
    const int L = lens[s];
    const int64_t off = offs[s];
    int32_t* st = start + (size_t)s * (P.limit + 2);
    for (int c = threadIdx.x; c < P.limit + 2; c += blockDim.x) hist[c] = 0;
    __syncthreads();
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
        int code = 0;
        if (p + P.ktup <= L) {
            code = 1;
            for (int j = 0; j < P.ktup; ++j) {
                int r = orig[off + p + j];
                if (P.dna) r = aa2dna(r);
                if (r < 0 || r > (P.dna ? 3 : P.max_aa)) {
                    code = 0;
                    break;
                }
                code += r * P.pot[j];
            }
        }
        kcode[off + p] = (int16_t)code;
        if (code) atomicAdd(&hist[code], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int c = 0; c <= P.limit; ++c) {
            const int h = hist[c];
            st[c] = acc;
            hist[c] = acc;  // cursor
            acc += h;
        }
        st[P.limit + 1] = acc;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
        const int code = kcode[off + p];
        if (code) {
            const int k = atomicAdd(&hist[code], 1);
            pos[off + k] = (uint16_t)(p + 1);
        }
    }
}

struct Args {
    const int16_t* kcode;
    const uint16_t* pos;
    const int32_t* start;
    const int64_t* offs;
    const int32_t* lens;
    const int32_t* pairs;  // [npairs][2] 0-based (si, sj)
    const int32_t* order;  // processing order (longest first)
    long long npairs;
    double* dist;
    cwgpu_fast_stats* stats;
    unsigned long long* counter;
    Params P;
    int lmax;  // longest sequence of the set (sizes the shared regions)
    uint2* overflow;       // per warp: list records below the shared ones
    long long ovf_stride;  // records per warp (2 * max_aln + 2)
    uint16_t* sortbuf;     // per warp: counts and diagonals for the reference's sort
    long long sort_stride; // entries per array (2 * lmax + 4)
};

// Shared memory of one pair (one CTA), sizes from lmax:
//   U       union: counts uint16[T] (count/select), then the list records of
//           the chain (uint2: v1 | v2 << 16, score), CAP of them, the part of
//           the score-sorted list below its top 32
//   flag    one bit per diagonal (T bits), flagged uint16[NF], last uint32[NF]
// with T = 2*lmax + 2 diagonals and NF the most diagonals that can be
// flagged, signif * (2*window + 1) (at most T). `last` holds the newest
// fragment on each flagged diagonal as v1 | score << 16 (0: none) and is
// indexed like `flagged`. List records below the CAP that fit shared memory
// live in a per-warp global overflow array (the list's low-score tail, which
// the chain rarely visits). The reference's sort of the counts, needed for
// about one pair in ten, runs on a per-warp global copy (counts, diagonals).
struct Smem {
    unsigned* cntw;   // 16-bit counts, two per word (atomics on the word)
    uint16_t* cnt;    // the same counts as an array
    uint2* sl;        // list records in shared memory
    int cap;          // their capacity (a multiple of 32)
    unsigned* flagw;
    uint16_t* flagged;
    unsigned* last;
};

__host__ __device__ inline size_t max_flagged(int lmax, int signif, int window) {
    const size_t T = 2 * (size_t)lmax + 2, nf = (size_t)signif * (2 * (size_t)window + 1);
    return nf < T ? nf : T;
}

constexpr int kMinListCap = 256;  // list records in shared memory, at least

// Layout of Smem; returns the bytes. offs_out: flagw, flagged, last.
__host__ __device__ inline size_t smem_bytes(int lmax, size_t NF, size_t* offs_out = nullptr, int* cap_out = nullptr) {
    const size_t T = 2 * (size_t)lmax + 2;
    const size_t Tp = (T + 2 + 1) & ~(size_t)1;  // even: whole words of counts
    size_t u = 2 * Tp;                            // cnt
    if (u < 8 * (size_t)kMinListCap) u = 8 * (size_t)kMinListCap;
    u = (u + 255) & ~(size_t)255;  // 32 records of 8 bytes
    size_t off = u;
    const size_t o_flag = off;
    off += ((T + 2 + 31) / 32) * 4;
    off = (off + 15) & ~(size_t)15;
    const size_t o_flagged = off;
    off += (2 * NF + 15) & ~(size_t)15;
    const size_t o_last = off;
    off += (4 * NF + 15) & ~(size_t)15;
    if (offs_out) {
        offs_out[0] = o_flag;
        offs_out[1] = o_flagged;
        offs_out[2] = o_last;
    }
    if (cap_out) *cap_out = (int)(u / 8);
    return off;
}

__device__ Smem carve(int lmax, size_t NF) {
    extern __shared__ __align__(16) unsigned char smem[];
    size_t o[3];
    int cap = 0;
    smem_bytes(lmax, NF, o, &cap);
    Smem S;
    S.cntw = reinterpret_cast<unsigned*>(smem);
    S.cnt = reinterpret_cast<uint16_t*>(smem);
    S.sl = reinterpret_cast<uint2*>(smem);
    S.cap = cap;
    S.flagw = reinterpret_cast<unsigned*>(smem + o[0]);
    S.flagged = reinterpret_cast<uint16_t*>(smem + o[1]);
    S.last = reinterpret_cast<unsigned*>(smem + o[2]);
    return S;
}

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int warp_max(int v) {
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
__device__ __forceinline__ int warp_sum(int v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// The reference's quicksort (desQuickSort, FastPairwiseAlign.cpp:585-658) of
// a[1..size-1] ascending with b permuted alongside, run only on sub-ranges
// that overlap [want_lo, size-1]: a partition permutes only inside its own
// range, so the other sub-ranges cannot change positions want_lo and up.
// Lane 0 only. The explicit stack holds at most log2(size) + 1 ranges, as the
// reference's (it always continues with the smaller part).
__device__ void top_quick_sort(uint16_t* a, uint16_t* b, int size, int want_lo) {
    int lst[50], ust[50], p = 1;
    lst[1] = 1;
    ust[1] = size - 1;
    while (p > 0) {
        if (lst[p] >= ust[p] || ust[p] < want_lo) {
            p--;
            continue;
        }
        int i = lst[p] - 1, j = ust[p];
        const int piv = a[j];
        while (i < j) {
            for (i = i + 1; a[i] < piv; i++)
                ;
            for (j = j - 1; j > i; j--)
                if (a[j] <= piv) break;
            if (i < j) {
                uint16_t t = a[i]; a[i] = a[j]; a[j] = t;
                t = b[i]; b[i] = b[j]; b[j] = t;
            }
        }
        j = ust[p];
        uint16_t t = a[i]; a[i] = a[j]; a[j] = t;
        t = b[i]; b[i] = b[j]; b[j] = t;
        if (i - lst[p] < ust[p] - i) {
            lst[p + 1] = lst[p];
            ust[p + 1] = i - 1;
            lst[p] = i + 1;
        } else {
            lst[p + 1] = i + 1;
            ust[p + 1] = ust[p];
            ust[p] = i - 1;
        }
        p = p + 1;
        if (p >= 49) {  // cannot happen (depth <= log2(size) + 1); keep the stack in bounds
            p = 48;
        }
    }
}

__device__ __forceinline__ bool frag_rel_pos(int a1, int b1, int a2, int b2, int ktup) {
    if (a1 - b1 == a2 - b2) return a2 < a1;
    return a2 + ktup - 1 < a1 && b2 + ktup - 1 < b1;
}

// Sets the flag bits of diagonals lo..hi.
__device__ __forceinline__ void set_flags(unsigned* flagw, int lo, int hi) {
    for (int l = lo; l <= hi; ++l) atomicOr(&flagw[l >> 5], 1u << (l & 31));
}

// Hits per diagonal (:198-219) into 16-bit counts (at most min(l1, l2)),
// cnt[0 .. tl1+1].
__device__ __forceinline__ void count_hits(const Smem& S, const int16_t* kc1, const uint16_t* pos2,
                                           const int32_t* st2, int l1, int l2, int ktup) {
    const int lane = threadIdx.x & 31;
    const int tl1 = l1 + l2 - 1;
    const int ncw = (tl1 + 3) / 2;  // words holding counts 0..tl1+1
    for (int w = lane; w < ncw; w += 32) S.cntw[w] = 0;
    __syncwarp();
    for (int p1 = 1 + lane; p1 <= l1 - ktup + 1; p1 += 32) {
        const int c = kc1[p1 - 1];
        if (!c) continue;
        const int b = __ldg(st2 + c), e = __ldg(st2 + c + 1);
#pragma unroll 4
        for (int k = b; k < e; ++k) {
            const int d = p1 - __ldg(pos2 + k) + l2;
            atomicAdd(&S.cntw[d >> 1], 1u << ((d & 1) << 4));
        }
    }
    __syncwarp();

}

// The top diagonals (:221-241), the diagonals within `window` of them flagged,
// and the flagged diagonals in ascending order in S.flagged; returns how many.
__device__ __forceinline__ int flag_top_diagonals(const Args& A, const Smem& S, int tl1) {
    const Params& P = A.P;
    const int lane = threadIdx.x & 31;
    const int jlo = max(1, tl1 - P.signif + 1);  // first top position
    const int kk = tl1 - jlo;                    // sorted top positions jlo..tl1-1
    int mode = 0;                                 // 0: none, 1: count > T, 2: count >= T, 3: sorted
    int T = 0;
    if (kk > 0) {
        int cur = 0x7fffffff, got = 0, eq = 0;
        for (;;) {  // k-th largest of cnt[1..tl1-1], with multiplicity: one scan per distinct value
            int lv = -1, lc = 0;  // this lane's largest count below cur and how often it occurs
            for (int d = 1 + lane; d <= tl1 - 1; d += 32) {
                const int x = S.cnt[d];
                if (x < cur) {
                    if (x > lv) {
                        lv = x;
                        lc = 1;
                    } else if (x == lv) {
                        ++lc;
                    }
                }
            }
            const int v = warp_max(lv);
            if (v < 0) break;  // fewer than kk values below cur (cannot happen: kk <= tl1 - 1)
            const int c = warp_sum(lv == v ? lc : 0);
            got += c;
            cur = v;
            if (got >= kk) {
                eq = c;
                break;
            }
        }
        T = cur;
        const int gt = got - eq;
        if (T <= 0) mode = 1;                // every positive count is in the top positions
        else if (eq == kk - gt) mode = 2;    // all diagonals at the boundary fit
        else mode = 3;                       // ties straddle the boundary: the reference's sort decides
    }
    const int nfw = (tl1 + 2 + 31) / 32;
    for (int w = lane; w < nfw; w += 32) S.flagw[w] = 0;
    __syncwarp();
    if (mode == 3) {
        uint16_t* const ga = A.sortbuf + (size_t)blockIdx.x * 2 * (size_t)A.sort_stride;
        uint16_t* const gd = ga + A.sort_stride;
        for (int d = lane; d <= tl1; d += 32) {
            ga[d] = S.cnt[d];
            gd[d] = (uint16_t)d;
        }
        __syncwarp();
        if (lane == 0) {
            top_quick_sort(ga, gd, tl1, jlo);
            for (int i = tl1 - 1; i >= jlo; --i)
                if (ga[i] > 0) {
                    const int c = gd[i];
                    set_flags(S.flagw, max(1, c - P.window), min(tl1, c + P.window));
                }
        }
    } else if (mode != 0) {
        for (int d = 1 + lane; d <= tl1 - 1; d += 32) {
            const int x = S.cnt[d];
            if (x > 0 && (x > T || (mode == 2 && x == T)))
                set_flags(S.flagw, max(1, d - P.window), min(tl1, d + P.window));
        }
    }
    if (lane == 0 && tl1 >= 1 && S.cnt[tl1] > 0)  // position tl1 keeps its own diagonal
        set_flags(S.flagw, max(1, tl1 - P.window), tl1);
    __syncwarp();
    // Flagged diagonals in ascending order. At most signif centres with
    // 2*window+1 diagonals each can be flagged, which sizes the list (the
    // bound check never fails).
    const int nf_cap = (int)max_flagged(A.lmax, P.signif, P.window);
    int nf = 0;
    for (int base = 1; base <= tl1; base += 32) {
        const int d = base + lane;
        const bool f = d <= tl1 && ((S.flagw[d >> 5] >> (d & 31)) & 1u);
        const unsigned m = __ballot_sync(kFull, f);
        const int at = nf + __popc(m & ((1u << lane) - 1));
        if (f && at < nf_cap) S.flagged[at] = (uint16_t)d;
        nf += __popc(m);
    }
    nf = min(nf, nf_cap);
    for (int f = lane; f < nf; f += 32) S.last[f] = 0;
    __syncwarp();

    return nf;
}

struct ChainResult {
    int nfr;         // fragments in the list
    int frags;       // currFrag, the fragment count the reference reports
    bool partial;    // the reference's "(Partial alignment)" cut-off was reached
    int head_score;  // score of the best fragment (maxSoFar)
};

// Fragment chaining (:246-398), the whole warp together, over the nf flagged
// diagonals in S.flagged.
// The reference keeps every fragment in a list sorted by score (putFrag)
// and, for each match on a flagged diagonal, walks the list from the best
// fragment to the first one the match can follow (the A-loop). Here list
// entries are records (v1 | v2 << 16, score); the index of the entry at
// distance d from the head (maxSoFar) is nfr-1-d. The top 32 entries live
// in registers, lane d holding distance d (wf = 1, positions wv, score
// ws); indices [base, nfr-32) are the shared records sl[0 .. nsl) and
// indices below base the warp's global overflow array G. A walk from the
// head is a register test and then 32-wide scans down the rest. putFrag
// inserts close to the head: within the top 32 it is a register shift
// whose last entry joins the shared records; deeper it shifts the records
// above it. When the shared records are full, their lower half moves to G.
__device__ __forceinline__ ChainResult chain_fragments(const Args& A, const Smem& S, const int16_t* kc1,
                                                       const int16_t* kc2, int l1, int l2, int nf) {
    const Params& P = A.P;
    const int lane = threadIdx.x & 31;
    const int ktup = P.ktup;
    uint2* const G = A.overflow + (size_t)blockIdx.x * (size_t)A.ovf_stride;
    const int cap = S.cap;
    int nfr = 0, currFrag = 0, base = 0, nsl = 0;
    bool partial = false;
    int wf = 0, ws = 0;
    unsigned wv = 0;
    const int fl0 = lane < nf ? (int)S.flagged[lane] : 0;
    const int fl1 = 32 + lane < nf ? (int)S.flagged[32 + lane] : 0;
    for (int i = 1; i <= l1 - ktup + 1 && !partial; ++i) {
        const int c1 = kc1[i - 1];
        if (!c1) continue;
        for (int fb = 0; fb < nf && !partial; fb += 32) {
            const int k = fb + lane;
            int fd = 0;
            bool hit = false;
            if (k < nf) {
                fd = fb == 0 ? fl0 : (fb == 32 ? fl1 : (int)S.flagged[k]);
                const int vn2 = i - fd + l2;  // osptr = i - vn2 + l2 = flagged[k]
                hit = vn2 >= 1 && vn2 <= l2 - ktup + 1 && __ldg(kc2 + vn2 - 1) == c1;
            }
            unsigned m = __ballot_sync(kFull, hit);
            // ascending diagonal = descending vn2: the order of the reference's list
            while (m && !partial) {
                const int t = __ffs(m) - 1;
                m &= m - 1;
                const int fi = fb + t;  // position of the diagonal in `flagged`
                const int osptr = __shfl_sync(kFull, fd, t);
                const int v2 = i - osptr + l2;
                // the A-loop: first fragment from the head this match can follow
                bool found = false;
                int tfs = 0;
                unsigned fvv = 0;
                unsigned mm = __ballot_sync(kFull, wf != 0 && frag_rel_pos(i, v2, (int)(wv & 0xffffu), (int)(wv >> 16), ktup));
                if (mm) {
                    const int src = __ffs(mm) - 1;
                    found = true;
                    fvv = __shfl_sync(kFull, wv, src);
                    tfs = __shfl_sync(kFull, ws, src);
                } else {
                    for (int kb = 32; kb < nfr; kb += 32) {
                        const int d = kb + lane;
                        uint2 r = make_uint2(0u, 0u);
                        bool ok = false;
                        if (d < nfr) {
                            const int j = nfr - 1 - d;
                            r = j >= base ? S.sl[j - base] : G[j];
                            ok = frag_rel_pos(i, v2, (int)(r.x & 0xffffu), (int)(r.x >> 16), ktup);
                        }
                        mm = __ballot_sync(kFull, ok);
                        if (mm) {
                            const int src = __ffs(mm) - 1;
                            found = true;
                            fvv = __shfl_sync(kFull, r.x, src);
                            tfs = (int)__shfl_sync(kFull, r.y, src);
                            break;
                        }
                    }
                }
                int fs = ktup;
                if (found) {
                    const int tv1 = (int)(fvv & 0xffffu), tv2 = (int)(fvv >> 16);
                    if (i - v2 == tv1 - tv2) {
                        fs = tfs + (i > tv1 + (ktup - 1) ? ktup : i - tv1);
                    } else {
                        const unsigned lf = S.last[fi];
                        int subt1 = ktup;
                        if (lf) {
                            const int lv1 = (int)(lf & 0xffffu);
                            subt1 = (int)(int16_t)(lf >> 16) + (i > lv1 + (ktup - 1) ? ktup : i - lv1);
                        }
                        const int subt2 = tfs - P.window_gap + ktup;
                        fs = subt2 > subt1 ? subt2 : subt1;
                    }
                }
                fs = (int16_t)fs;  // the stored score type (never truncates: fs <= ktup * l1 < 2^15)
                currFrag = nfr + 1;
                if (currFrag >= 2 * P.max_aln) {
                    partial = true;
                    break;
                }
                // putFrag: before the first fragment from the head whose score
                // is not above fs (the tail if none)
                int kins = nfr;
                mm = __ballot_sync(kFull, wf != 0 && ws <= fs);
                if (mm) {
                    kins = __ffs(mm) - 1;
                } else {
                    for (int kb = 32; kb < nfr; kb += 32) {
                        const int d = kb + lane;
                        bool le = false;
                        if (d < nfr) {
                            const int j = nfr - 1 - d;
                            le = (int)(j >= base ? S.sl[j - base].y : G[j].y) <= fs;
                        }
                        mm = __ballot_sync(kFull, le);
                        if (mm) {
                            kins = kb + __ffs(mm) - 1;
                            break;
                        }
                    }
                }
                if (nfr >= 32 && nsl == cap) {  // make room: the lower half of the records to G
                    const int h = cap / 2;
                    for (int e = lane; e < h; e += 32) G[base + e] = S.sl[e];
                    __syncwarp();
                    for (int e = lane; e < cap - h; e += 32) {
                        const uint2 v = S.sl[h + e];
                        S.sl[e] = v;
                    }
                    __syncwarp();
                    base += h;
                    nsl -= h;
                }
                const unsigned nv = (unsigned)i | ((unsigned)v2 << 16);
                if (kins < 32) {
                    // Into the registers: distance 31 (if any) becomes index nfr - 32.
                    if (nfr >= 32) {
                        if (lane == 31) S.sl[nsl] = make_uint2(wv, (unsigned)ws);
                        ++nsl;
                    }
                    const int uf = __shfl_up_sync(kFull, wf, 1);
                    const unsigned uv = __shfl_up_sync(kFull, wv, 1);
                    const int us = __shfl_up_sync(kFull, ws, 1);
                    if (lane > kins) {
                        wf = uf;
                        wv = uv;
                        ws = us;
                    } else if (lane == kins) {
                        wf = 1;
                        wv = nv;
                        ws = fs;
                    }
                } else {
                    const int pnew = nfr - kins;  // the new record's index (<= nfr - 32)
                    const uint2 nrec = make_uint2(nv, (unsigned)fs);
                    const int lo = pnew >= base ? pnew - base : 0;
                    for (int top = nsl - 1; top >= lo; top -= 32) {  // sl[lo .. nsl) up one, top chunk first
                        const int x = top - lane;
                        uint2 v = make_uint2(0u, 0u);
                        if (x >= lo) v = S.sl[x];
                        __syncwarp();
                        if (x >= lo) S.sl[x + 1] = v;
                        __syncwarp();
                    }
                    if (pnew >= base) {
                        if (lane == 0) S.sl[lo] = nrec;
                    } else {  // G[base-1] moves up into sl[0]; G[pnew .. base-1) up one
                        if (lane == 0) S.sl[0] = G[base - 1];
                        __syncwarp();
                        for (int top = base - 2; top >= pnew; top -= 32) {
                            const int x = top - lane;
                            uint2 v = make_uint2(0u, 0u);
                            if (x >= pnew) v = G[x];
                            __syncwarp();
                            if (x >= pnew) G[x + 1] = v;
                            __syncwarp();
                        }
                        if (lane == 0) G[pnew] = nrec;
                    }
                    ++nsl;
                }
                if (lane == 0) S.last[fi] = (unsigned)(uint16_t)i | ((unsigned)(uint16_t)fs << 16);
                __syncwarp();
                nfr = currFrag;
            }
        }
    }
    return ChainResult{nfr, currFrag, partial, __shfl_sync(kFull, ws, 0)};
}

// One pair on one warp.
__device__ void fast_pair(const Args& A, const Smem& S, long long q) {
    const Params& P = A.P;
    const int lane = threadIdx.x & 31;
    const int si = A.pairs[2 * q], sj = A.pairs[2 * q + 1];
    const int l1 = A.lens[si], l2 = A.lens[sj];
    const int64_t o1 = A.offs[si], o2 = A.offs[sj];
    const int tl1 = l1 + l2 - 1;
    const int16_t* kc1 = A.kcode + o1;
    const int16_t* kc2 = A.kcode + o2;  // kc2[p - 1]: code of the k-tuple at 1-based p of seq 2
    const uint16_t* pos2 = A.pos + o2;
    const int32_t* st2 = A.start + (size_t)sj * (P.limit + 2);

    count_hits(S, kc1, pos2, st2, l1, l2, P.ktup);
    const int nf = flag_top_diagonals(A, S, tl1);
    const ChainResult ch = chain_fragments(A, S, kc1, kc2, l1, l2, nf);
    const int nfr = ch.nfr, currFrag = ch.frags, head_score = ch.head_score;
    const bool partial = ch.partial;

    // ---- distance (:88-103), in double as the reference
    if (lane == 0) {
        const int score = nfr ? head_score : 0;
        double calc = 0.0;
        if (nfr) {
            calc = (double)score;
            if (P.percent) calc = __dmul_rn(__ddiv_rn(calc, (double)min(l1, l2)), 100.0);
        }
        A.dist[q] = __ddiv_rn(__dsub_rn(100.0, calc), 100.0);
        if (A.stats) {
            cwgpu_fast_stats st;
            st.score = score;
            st.frags = currFrag;
            st.partial = partial ? 1 : 0;
            st.pad = 0;
            A.stats[q] = st;
        }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32) k_fast(Args A) {
    const Smem S = carve(A.lmax, max_flagged(A.lmax, A.P.signif, A.P.window));
    const int lane = threadIdx.x;
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(A.counter, 1ULL);
        k = __shfl_sync(kFull, k, 0);
        if (k >= (unsigned long long)A.npairs) break;
        fast_pair(A, S, A.order ? A.order[k] : (long long)k);
    }
}

}  // namespace cwfast

using namespace cwfast;

// Per-context tables of the quick path, rebuilt when the sequences or the
// k-tuple parameters change.
struct cwgpu_fast_state {
    unsigned generation = ~0u;
    int key_dna = -1, key_ktup = -1, key_max_aa = -1;
    int8_t* d_orig = nullptr;
    int16_t* d_kcode = nullptr;
    uint16_t* d_pos = nullptr;
    int32_t* d_start = nullptr;
    int limit = 0;
    unsigned long long* d_counter = nullptr;
    size_t smem_set = 0;
    uint2* d_ovf = nullptr;  // list overflow, ovf_records per warp of the grid
    size_t ovf_bytes = 0;
    uint16_t* d_sort = nullptr;  // sort copies, 2 * sort_stride per warp of the grid
    size_t sort_bytes = 0;
    // cwgpu_fast_align_pairs: grow-only pair, order and output arrays
    int32_t* d_pairs = nullptr;
    int32_t* d_order = nullptr;
    double* d_dist = nullptr;
    cwgpu_fast_stats* d_stats = nullptr;
    int64_t cap_pairs = 0;
};

void cwgpu_fast_release(cwgpu_context* ctx) {
    if (!ctx || !ctx->fast) return;
    cwgpu_fast_state* F = ctx->fast;
    void* ptrs[] = {F->d_orig, F->d_kcode, F->d_pos, F->d_start, F->d_counter, F->d_ovf, F->d_sort,
                    F->d_pairs, F->d_order, F->d_dist, F->d_stats};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete F;
    ctx->fast = nullptr;
}

namespace {

int ffail(cwgpu_context* ctx, int code, const std::string& msg) {
    ctx->last_error = msg;
    return code;
}

#define FAST_CUDA(ctx, call)                                                                               \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return ffail(ctx, e_ == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA,          \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                              \
    } while (0)

int make_params(cwgpu_context* ctx, const cwgpu_fast_params* p, Params* P) {
    if (!p) return CWGPU_ERR_ARG;
    const int base = p->dna ? 4 : p->max_aa + 1;
    if (p->ktup < 1 || p->ktup > 6 || base < 1 || p->max_aa < 0 || p->max_aa > 31 || p->window < 0 ||
        p->window_gap < 0 || p->signif < 1)
        return ffail(ctx, CWGPU_ERR_ARG, "k-tuple parameters out of range");
    long long limit = 1;
    for (int i = 0; i < p->ktup; ++i) limit *= base;
    if (limit > kMaxLimit) return ffail(ctx, CWGPU_ERR_ARG, "too many k-tuple codes (ktup too large)");
    memset(P, 0, sizeof(*P));
    P->dna = p->dna ? 1 : 0;
    P->ktup = p->ktup;
    P->window = p->window;
    P->window_gap = p->window_gap;
    P->signif = p->signif;
    P->percent = p->percent ? 1 : 0;
    P->max_aa = p->max_aa;
    P->max_aln = p->max_aln_length > 0 ? p->max_aln_length : 2 * ctx->lmax;
    P->limit = (int)limit;
    int v = 1;
    for (int i = 0; i < p->ktup; ++i) {
        P->pot[i] = v;
        v *= base;
    }
    if (ctx->lmax > kMaxLen || (long long)P->ktup * ctx->lmax > 32767 || 2LL * P->max_aln + 2 > 65535)
        return ffail(ctx, CWGPU_ERR_ARG, "sequences too long for the quick k-tuple path (8191 residues)");
    return CWGPU_OK;
}

int ensure_tables(cwgpu_context* ctx, const Params& P) {
    const int rc = cwgpu_stage_inputs(ctx);  // offsets and lengths on the device
    if (rc) return rc;
    if (!ctx->fast) ctx->fast = new cwgpu_fast_state();
    cwgpu_fast_state* F = ctx->fast;
    if (F->generation == ctx->generation && F->key_dna == P.dna && F->key_ktup == P.ktup &&
        F->key_max_aa == P.max_aa)
        return CWGPU_OK;
    FAST_CUDA(ctx, cudaSetDevice(ctx->device));
    void* ptrs[] = {F->d_orig, F->d_kcode, F->d_pos, F->d_start};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    F->d_orig = nullptr;
    F->d_kcode = nullptr;
    F->d_pos = nullptr;
    F->d_start = nullptr;
    const size_t total = std::max<size_t>(ctx->host_codes.size(), 16);
    const int ns = std::max(1, ctx->nseqs);
    FAST_CUDA(ctx, cudaMalloc(&F->d_orig, total));
    FAST_CUDA(ctx, cudaMalloc(&F->d_kcode, total * sizeof(int16_t)));
    FAST_CUDA(ctx, cudaMalloc(&F->d_pos, total * sizeof(uint16_t)));
    FAST_CUDA(ctx, cudaMalloc(&F->d_start, (size_t)ns * (P.limit + 2) * sizeof(int32_t)));
    if (!F->d_counter) FAST_CUDA(ctx, cudaMalloc(&F->d_counter, sizeof(unsigned long long)));
    FAST_CUDA(ctx, cudaMemcpy(F->d_orig, ctx->host_codes.data(), ctx->host_codes.size(), cudaMemcpyHostToDevice));
    if (ctx->nseqs > 0) {
        k_fast_prep<<<ctx->nseqs, 256, sizeof(int) * (P.limit + 2), ctx->stream>>>(
            F->d_orig, ctx->d_offs, ctx->d_lens, P, F->d_kcode, F->d_pos, F->d_start);
        FAST_CUDA(ctx, cudaGetLastError());
        FAST_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    F->generation = ctx->generation;
    F->key_dna = P.dna;
    F->key_ktup = P.ktup;
    F->key_max_aa = P.max_aa;
    F->limit = P.limit;
    return CWGPU_OK;
}

// Runs the pairs (device pointers) in `d_order` order on `st`; synchronous.
int run_fast(cwgpu_context* ctx, const Params& P, const int32_t* d_pairs, const int32_t* d_order, long long npairs,
             double* d_dist, cwgpu_fast_stats* d_stats, cudaStream_t st) {
    cwgpu_fast_state* F = ctx->fast;
    const size_t sm = smem_bytes(ctx->lmax, max_flagged(ctx->lmax, P.signif, P.window));
    if (sm > 227 * 1024) return ffail(ctx, CWGPU_ERR_ARG, "sequences too long for the quick path's shared memory");
    if (sm > F->smem_set) {
        FAST_CUDA(ctx, cudaFuncSetAttribute(k_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        F->smem_set = sm;
    }
    int per_sm = 0;
    FAST_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fast, 32, sm));
    if (per_sm < 1) return ffail(ctx, CWGPU_ERR_ARG, "quick path does not fit one SM");
    const long long grid = std::min<long long>((long long)per_sm * ctx->sm_count, std::max<long long>(npairs, 1));
    const long long ovf_records = 2LL * P.max_aln + 2;
    const size_t ovf = (size_t)grid * (size_t)ovf_records * sizeof(uint2);
    if (ovf > F->ovf_bytes) {
        if (F->d_ovf) FAST_CUDA(ctx, cudaFree(F->d_ovf));
        F->d_ovf = nullptr;
        F->ovf_bytes = 0;
        FAST_CUDA(ctx, cudaMalloc(&F->d_ovf, ovf));
        F->ovf_bytes = ovf;
    }
    const long long sort_stride = 2LL * ctx->lmax + 4;
    const size_t sortb = (size_t)grid * 2 * (size_t)sort_stride * sizeof(uint16_t);
    if (sortb > F->sort_bytes) {
        if (F->d_sort) FAST_CUDA(ctx, cudaFree(F->d_sort));
        F->d_sort = nullptr;
        F->sort_bytes = 0;
        FAST_CUDA(ctx, cudaMalloc(&F->d_sort, sortb));
        F->sort_bytes = sortb;
    }
    Args A;
    A.kcode = F->d_kcode;
    A.pos = F->d_pos;
    A.start = F->d_start;
    A.offs = ctx->d_offs;
    A.lens = ctx->d_lens;
    A.pairs = d_pairs;
    A.order = d_order;
    A.npairs = npairs;
    A.dist = d_dist;
    A.stats = d_stats;
    A.counter = F->d_counter;
    A.P = P;
    A.lmax = ctx->lmax;
    A.overflow = F->d_ovf;
    A.ovf_stride = ovf_records;
    A.sortbuf = F->d_sort;
    A.sort_stride = sort_stride;
    FAST_CUDA(ctx, cudaMemsetAsync(F->d_counter, 0, sizeof(unsigned long long), st));
    if (npairs > 0) {
        k_fast<<<(unsigned)grid, 32, sm, st>>>(A);
        FAST_CUDA(ctx, cudaGetLastError());
    }
    return CWGPU_OK;
}

}  // namespace

extern "C" {

int cwgpu_fast_align_pairs(cwgpu_context* ctx, const cwgpu_fast_params* p, const int32_t* pairs, int64_t npairs,
                           double* dist_out, cwgpu_fast_stats* stats_out) {
    if (!ctx || npairs < 0 || (npairs > 0 && (!pairs || !dist_out))) return CWGPU_ERR_ARG;
    if (npairs > CWGPU_MAX_PAIRS_PER_CALL)
        return ffail(ctx, CWGPU_ERR_ARG, "more than CWGPU_MAX_PAIRS_PER_CALL pairs in one call");
    if (!ctx->has_seqs) return ffail(ctx, CWGPU_ERR_STATE, "sequences not set");
    Params P;
    int rc = make_params(ctx, p, &P);
    if (rc) return rc;
    for (int64_t q = 0; q < npairs; ++q) {
        const int32_t a = pairs[2 * q], b = pairs[2 * q + 1];
        if (a < 0 || b < 0 || a >= ctx->nseqs || b >= ctx->nseqs)
            return ffail(ctx, CWGPU_ERR_ARG, "pair index outside the sequence set");
    }
    if (npairs == 0) return CWGPU_OK;
    rc = ensure_tables(ctx, P);
    if (rc) return rc;
    // Longest pairs first: the hit count and the chain grow with l1 * l2. The
    // order only balances the load: a stable counting sort on the top 12
    // bits of l1 * l2 as a float.
    constexpr int kKeyBits = 12, kBuckets = 1 << kKeyBits;
    std::vector<uint16_t> key((size_t)npairs);
    std::vector<int64_t> start(kBuckets + 1, 0);
    for (int64_t q = 0; q < npairs; ++q) {
        const float w = (float)((double)ctx->lens[pairs[2 * q]] * (double)ctx->lens[pairs[2 * q + 1]]);
        uint32_t bits;
        memcpy(&bits, &w, sizeof(bits));
        const int k = kBuckets - 1 - (int)(bits >> (31 - kKeyBits));
        key[(size_t)q] = (uint16_t)k;
        ++start[k + 1];
    }
    for (int k = 0; k < kBuckets; ++k) start[k + 1] += start[k];
    std::vector<int32_t> order((size_t)npairs);
    for (int64_t q = 0; q < npairs; ++q) order[(size_t)start[key[(size_t)q]]++] = (int32_t)q;
    cwgpu_fast_state* F = ctx->fast;
    cudaStream_t st = ctx->stream;
    if (npairs > F->cap_pairs) {
        void* old[] = {F->d_pairs, F->d_order, F->d_dist, F->d_stats};
        for (void* ptr : old)
            if (ptr) cudaFree(ptr);
        F->d_pairs = F->d_order = nullptr;
        F->d_dist = nullptr;
        F->d_stats = nullptr;
        F->cap_pairs = 0;
        FAST_CUDA(ctx, cudaMalloc(&F->d_pairs, sizeof(int32_t) * 2 * npairs));
        FAST_CUDA(ctx, cudaMalloc(&F->d_order, sizeof(int32_t) * npairs));
        FAST_CUDA(ctx, cudaMalloc(&F->d_dist, sizeof(double) * npairs));
        FAST_CUDA(ctx, cudaMalloc(&F->d_stats, sizeof(cwgpu_fast_stats) * npairs));
        F->cap_pairs = npairs;
    }
    int32_t* d_pairs = F->d_pairs;
    int32_t* d_order = F->d_order;
    double* d_dist = F->d_dist;
    cwgpu_fast_stats* d_stats = stats_out ? F->d_stats : nullptr;
    FAST_CUDA(ctx, cudaMemcpyAsync(d_pairs, pairs, sizeof(int32_t) * 2 * npairs, cudaMemcpyHostToDevice, st));
    FAST_CUDA(ctx, cudaMemcpyAsync(d_order, order.data(), sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, st));
    rc = run_fast(ctx, P, d_pairs, d_order, npairs, d_dist, d_stats, st);
    if (rc == CWGPU_OK) {
        cudaError_t e = cudaMemcpyAsync(dist_out, d_dist, sizeof(double) * npairs, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && stats_out)
            e = cudaMemcpyAsync(stats_out, d_stats, sizeof(cwgpu_fast_stats) * npairs, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = ffail(ctx, CWGPU_ERR_CUDA, std::string("quick path: ") + cudaGetErrorString(e));
    }
    return rc;
}

int cwgpu_fast_align_pairs_device(cwgpu_context* ctx, const cwgpu_fast_params* p, const int32_t* d_pairs,
                                  const int32_t* d_order, int64_t npairs, double* d_dist,
                                  cwgpu_fast_stats* d_stats, void* stream) {
    if (!ctx || npairs < 0 || (npairs > 0 && (!d_pairs || !d_dist))) return CWGPU_ERR_ARG;
    if (npairs > CWGPU_MAX_PAIRS_PER_CALL)
        return ffail(ctx, CWGPU_ERR_ARG, "more than CWGPU_MAX_PAIRS_PER_CALL pairs in one call");
    if (!ctx->has_seqs) return ffail(ctx, CWGPU_ERR_STATE, "sequences not set");
    Params P;
    int rc = make_params(ctx, p, &P);
    if (rc) return rc;
    rc = ensure_tables(ctx, P);
    if (rc) return rc;
    return run_fast(ctx, P, d_pairs, d_order, npairs, d_dist, d_stats, stream ? (cudaStream_t)stream : ctx->stream);
}

int cwgpu_fast_pairwise_align(cwgpu_context* ctx, const cwgpu_fast_params* p, int32_t i_start, int32_t i_end,
                              int32_t j_start, int32_t j_end, double* elements, int32_t dist_size,
                              cwgpu_fast_stats* stats_out) {
    if (!ctx || !elements) return CWGPU_ERR_ARG;
    if (!ctx->has_seqs) return ffail(ctx, CWGPU_ERR_STATE, "sequences not set");
    const int n = ctx->nseqs;
    if (dist_size != n + 1) return ffail(ctx, CWGPU_ERR_ARG, "The distance matrix is not the right size!");
    if (i_start < 0 || i_end < i_start || j_start < 0 || j_end < j_start)
        return ffail(ctx, CWGPU_ERR_RANGE, "The range for pairwise Alignment is incorrect.");
    // FastPairwiseAlign.cpp:65-84: i = iStart+1..iEnd, j = max(jStart+2, i+1)..jEnd
    // (1-based), i.e. si in [iStart, iEnd), sj in [max(jStart+1, si+1), jEnd),
    // held inside the sequence set; whole rows per call.
    std::vector<double> dist;
    return cwgpu::for_range_blocks(
        n, i_start, i_end, j_start, j_end, cwgpu::kRangeBlockPairs, [&](const int32_t* pairs, int64_t np, int64_t first) {
            dist.resize((size_t)std::max<int64_t>(np, 1));
            const int rc =
                cwgpu_fast_align_pairs(ctx, p, pairs, np, dist.data(), stats_out ? stats_out + first : nullptr);
            if (rc) return rc;
            for (int64_t q = 0; q < np; ++q) {
                const int64_t a = pairs[2 * q + 1], b = pairs[2 * q];  // getIndex(si+1, sj+1), si < sj
                elements[((a * (a + 1)) >> 1) + b] = dist[q];
            }
            return (int)CWGPU_OK;
        });
}

}  // extern "C"
