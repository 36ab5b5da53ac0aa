/*
 * Oracle: a plain-C restatement of ClustalW 2.0.11's full (slow) pairwise
 * distance stage, FullPairwiseAlign::pairwiseAlign
 * (CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.cpp:34-660).
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library, and only to check the GPU results or as
 * the timed CPU baseline. The GPU library never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this restatement
 * against distance matrices written by the unmodified reference
 * (oracle/_ref/refharness) on the reference's own fixtures and on synthetic
 * sets (tests/golden/).
 *
 * Differences from the reference that do not change any output:
 *   - no `static` locals (diff() keeps them at FullPairwiseAlign.cpp:423), so
 *     the batch entry point can run pairs on several threads;
 *   - per-pair statistics (forward max score, end/start cells, identities,
 *     cell counts) are returned instead of being left in members.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NUMRES 32

typedef struct {
    int32_t dna;            /* userParameters->getDNAFlag() */
    float pw_gap_open;      /* getPWGapOpen() */
    float pw_gap_extend;    /* getPWGapExtend() */
    int32_t int_scale;      /* PairScaleValues.intScale */
    float gap_open_scale;   /* PairScaleValues.gapOpenScale */
    float gap_extend_scale; /* PairScaleValues.gapExtendScale */
    int32_t mat_avg;        /* matAvg from getPairwiseMatrix */
    int32_t gap_pos1;       /* getGapPos1() */
    int32_t gap_pos2;       /* getGapPos2() */
} cwo_params;

typedef struct {
    int32_t fwd_score;  /* forwardPass maxScore */
    int32_t se1, se2;   /* forwardPass end cell */
    int32_t sb1, sb2;   /* reversePass start cell */
    int32_t mm_score;   /* diff() return value (FullPairwiseAlign.cpp:165) */
    int32_t n_ident;    /* tracePath count */
    int32_t n_match;    /* number of displ entries equal to 0 */
    int32_t print_ptr;  /* printPtr after diff() */
    int32_t gap_open;   /* per-pair _gapOpen */
    int32_t gap_extend; /* per-pair _gapExtend */
    float dist;         /* value stored with DistMatrix::SetAt */
    int64_t cells_fwd;  /* forwardPass inner-loop iterations */
    int64_t cells_rev;  /* reversePass inner-loop iterations (up to the break) */
    int64_t cells_diff; /* diff() inner-loop iterations (both halves + M==1 scans) */
} cwo_pair_result;

/* Per-pair gap penalties, FullPairwiseAlign.cpp:129-148, with the same C types:
 * the DNA branch and the extension are float expressions, the protein
 * gap-open is a double expression with libm log(). */
void cwo_gap_penalties(const cwo_params* p, int n, int m, int32_t* go, int32_t* ge) {
    if (p->dna) {
        *go = (int)(2 * p->pw_gap_open * p->int_scale * p->gap_open_scale);
        *ge = (int)(p->pw_gap_extend * p->int_scale * p->gap_extend_scale);
    } else {
        int mn = n < m ? n : m;
        if (p->mat_avg <= 0)
            *go = 2 * (int)((p->pw_gap_open + log((double)mn)) * p->int_scale);
        else
            *go = (int)(2 * p->mat_avg * (p->pw_gap_open + log((double)mn)) * p->gap_open_scale);
        *ge = (int)(p->pw_gap_extend * p->int_scale);
    }
}

/* Work state of one pair alignment (the members of FullPairwiseAlign.h:37-59). */
typedef struct {
    const int32_t (*mat)[NUMRES];
    const int8_t* s1; /* 1-based: s1[1..n] */
    const int8_t* s2;
    int go, ge;
    int *HH, *DD, *RR, *SS, *displ;
    int print_ptr, last_print;
    int max_score, se1, se2, sb1, sb2;
    int64_t cells_rev, cells_diff;
    int n_match;
} cwo_ws;

static inline int score_at(const cwo_ws* w, int i, int j) { return w->mat[w->s1[i]][w->s2[j]]; }

/* FullPairwiseAlign.cpp:280-341 */
static void forward_pass(cwo_ws* w, int n, int m) {
    int i, j, f, hh, p, t;
    w->max_score = 0;
    w->se1 = w->se2 = 0;
    for (i = 0; i <= m; i++) {
        w->HH[i] = 0;
        w->DD[i] = -w->go;
    }
    for (i = 1; i <= n; i++) {
        hh = p = 0;
        f = -w->go;
        for (j = 1; j <= m; j++) {
            f -= w->ge;
            t = hh - w->go - w->ge;
            if (f < t) f = t;
            w->DD[j] -= w->ge;
            t = w->HH[j] - w->go - w->ge;
            if (w->DD[j] < t) w->DD[j] = t;
            hh = p + score_at(w, i, j);
            if (hh < f) hh = f;
            if (hh < w->DD[j]) hh = w->DD[j];
            if (hh < 0) hh = 0;
            p = w->HH[j];
            w->HH[j] = hh;
            if (hh > w->max_score) {
                w->max_score = hh;
                w->se1 = i;
                w->se2 = j;
            }
        }
    }
}

/* FullPairwiseAlign.cpp:343-416 */
static void reverse_pass(cwo_ws* w) {
    int i, j, f, hh, p, t, cost = 0;
    w->sb1 = w->sb2 = 1;
    for (i = w->se2; i > 0; i--) {
        w->HH[i] = -1;
        w->DD[i] = -1;
    }
    for (i = w->se1; i > 0; i--) {
        hh = f = -1;
        p = (i == w->se1) ? 0 : -1;
        for (j = w->se2; j > 0; j--) {
            w->cells_rev++;
            f -= w->ge;
            t = hh - w->go - w->ge;
            if (f < t) f = t;
            w->DD[j] -= w->ge;
            t = w->HH[j] - w->go - w->ge;
            if (w->DD[j] < t) w->DD[j] = t;
            hh = p + score_at(w, i, j);
            if (hh < f) hh = f;
            if (hh < w->DD[j]) hh = w->DD[j];
            p = w->HH[j];
            w->HH[j] = hh;
            if (hh > cost) {
                cost = hh;
                w->sb1 = i;
                w->sb2 = j;
                if (cost >= w->max_score) break;
            }
        }
        if (cost >= w->max_score) break;
    }
}

/* add/del: FullPairwiseAlign.cpp:213-224 and :614-624 */
static void op_add(cwo_ws* w, int v) {
    if (w->last_print < 0) {
        w->displ[w->print_ptr - 1] = v;
        w->displ[w->print_ptr++] = w->last_print;
    } else {
        w->last_print = w->displ[w->print_ptr++] = v;
    }
}

static void op_del(cwo_ws* w, int k) {
    if (w->last_print < 0)
        w->last_print = w->displ[w->print_ptr - 1] -= k;
    else
        w->last_print = w->displ[w->print_ptr++] = -k;
}

static inline int tbgap(const cwo_ws* w, int k, int tb) { return k <= 0 ? 0 : tb + w->ge * k; }
static inline int tegap(const cwo_ws* w, int k, int te) { return k <= 0 ? 0 : te + w->ge * k; }

/* Myers-Miller linear-space alignment, FullPairwiseAlign.cpp:418-612. */
static int diff(cwo_ws* w, int A, int B, int M, int N, int tb, int te) {
    int type, midi, midj, i, j, midh;
    int f, hh, e, s, t;
    const int go = w->go, ge = w->ge;
    int *HH = w->HH, *DD = w->DD, *RR = w->RR, *SS = w->SS;

    if (N <= 0) {
        if (M > 0) op_del(w, M);
        return -(int)tbgap(w, M, tb);
    }
    if (M <= 1) {
        if (M <= 0) {
            op_add(w, N);
            return -(int)tbgap(w, N, tb);
        }
        midh = -(tb + ge) - tegap(w, N, te);
        hh = -(te + ge) - tbgap(w, N, tb);
        if (hh > midh) midh = hh;
        midj = 0;
        for (j = 1; j <= N; j++) {
            w->cells_diff++;
            hh = score_at(w, A + 1, B + j) - tegap(w, N - j, te) - tbgap(w, j - 1, tb);
            if (hh > midh) {
                midh = hh;
                midj = j;
            }
        }
        if (midj == 0) {
            op_del(w, 1);
            op_add(w, N);
        } else {
            if (midj > 1) op_add(w, midj - 1);
            w->displ[w->print_ptr++] = w->last_print = 0;
            w->n_match++;
            if (midj < N) op_add(w, N - midj);
        }
        return midh;
    }

    midi = M / 2;
    HH[0] = 0;
    t = -tb;
    for (j = 1; j <= N; j++) {
        HH[j] = t = t - ge;
        DD[j] = t - go;
    }
    t = -tb;
    for (i = 1; i <= midi; i++) {
        s = HH[0];
        HH[0] = hh = t = t - ge;
        f = t - go;
        for (j = 1; j <= N; j++) {
            w->cells_diff++;
            if ((hh = hh - go - ge) > (f = f - ge)) f = hh;
            if ((hh = HH[j] - go - ge) > (e = DD[j] - ge)) e = hh;
            hh = s + score_at(w, A + i, B + j);
            if (f > hh) hh = f;
            if (e > hh) hh = e;
            s = HH[j];
            HH[j] = hh;
            DD[j] = e;
        }
    }
    DD[0] = HH[0];

    RR[N] = 0;
    t = -te;
    for (j = N - 1; j >= 0; j--) {
        RR[j] = t = t - ge;
        SS[j] = t - go;
    }
    t = -te;
    for (i = M - 1; i >= midi; i--) {
        s = RR[N];
        RR[N] = hh = t = t - ge;
        f = t - go;
        for (j = N - 1; j >= 0; j--) {
            w->cells_diff++;
            if ((hh = hh - go - ge) > (f = f - ge)) f = hh;
            if ((hh = RR[j] - go - ge) > (e = SS[j] - ge)) e = hh;
            hh = s + score_at(w, A + i + 1, B + j + 1);
            if (f > hh) hh = f;
            if (e > hh) hh = e;
            s = RR[j];
            RR[j] = hh;
            SS[j] = e;
        }
    }
    SS[N] = RR[N];

    midh = HH[0] + RR[0];
    midj = 0;
    type = 1;
    for (j = 0; j <= N; j++) {
        hh = HH[j] + RR[j];
        if (hh >= midh)
            if (hh > midh || (HH[j] != DD[j] && RR[j] == SS[j])) {
                midh = hh;
                midj = j;
            }
    }
    for (j = N; j >= 0; j--) {
        hh = DD[j] + SS[j] + go;
        if (hh > midh) {
            midh = hh;
            midj = j;
            type = 2;
        }
    }

    if (type == 1) {
        diff(w, A, B, midi, midj, tb, go);
        diff(w, A + midi, B + midj, M - midi, N - midj, go, te);
    } else {
        diff(w, A, B, midi - 1, midj, tb, 0);
        op_del(w, 2);
        diff(w, A + midi + 1, B + midj, M - midi - 1, N - midj, 0, te);
    }
    return midh;
}

/* FullPairwiseAlign.cpp:231-278 */
static int trace_path(const cwo_ws* w, int tsb1, int tsb2, int gap_pos1, int gap_pos2) {
    int i1 = tsb1, i2 = tsb2, count = 0, k, i;
    const int to_do = w->print_ptr - 1;
    for (i = 1; i <= to_do; ++i) {
        if (w->displ[i] == 0) {
            int res1 = w->s1[i1], res2 = w->s2[i2];
            if (res1 != gap_pos1 && res2 != gap_pos2 && res1 == res2) count++;
            ++i1;
            ++i2;
        } else if ((k = w->displ[i]) > 0) {
            i2 += k;
        } else {
            i1 -= k;
        }
    }
    return count;
}

static int count_residues(const int8_t* s, int len, int g1, int g2) {
    int c = 0;
    for (int i = 1; i <= len; i++)
        if (s[i] != g1 && s[i] != g2) c++;
    return c;
}

/* One pair: the body of the sj loop, FullPairwiseAlign.cpp:112-183.
 * s1/s2 are 0-based code arrays of length n/m. `scratch` must hold
 * scratch_ints(maxlen) ints, maxlen >= max(n, m). */
static size_t scratch_ints(int maxlen) { return 4 * (size_t)(2 * maxlen + 1) + 4 * (size_t)maxlen + 8; }

static void align_one(const int32_t (*mat)[NUMRES], const cwo_params* p, const int8_t* s1, int n,
                      const int8_t* s2, int m, int maxlen, int* scratch, cwo_pair_result* r) {
    memset(r, 0, sizeof(*r));
    cwo_gap_penalties(p, n, m, &r->gap_open, &r->gap_extend);
    if (n == 0 || m == 0) {
        r->dist = 1.0f;
        return;
    }
    const int row = 2 * maxlen + 1;
    cwo_ws w;
    memset(&w, 0, sizeof(w));
    w.mat = mat;
    w.s1 = s1 - 1;
    w.s2 = s2 - 1;
    w.go = r->gap_open;
    w.ge = r->gap_extend;
    w.HH = scratch;
    w.DD = scratch + row;
    w.RR = scratch + 2 * row;
    w.SS = scratch + 3 * row;
    w.displ = scratch + 4 * row;

    forward_pass(&w, n, m);
    r->fwd_score = w.max_score;
    r->se1 = w.se1;
    r->se2 = w.se2;
    reverse_pass(&w);
    r->sb1 = w.sb1;
    r->sb2 = w.sb2;
    w.last_print = 0;
    w.print_ptr = 1;
    r->mm_score = diff(&w, w.sb1 - 1, w.sb2 - 1, w.se1 - w.sb1 + 1, w.se2 - w.sb2 + 1, 0, 0);
    int count = trace_path(&w, w.sb1, w.sb2, p->gap_pos1, p->gap_pos2);
    float mm = 100.0 * (float)count;
    int len1 = count_residues(w.s1, n, p->gap_pos1, p->gap_pos2);
    int len2 = count_residues(w.s2, m, p->gap_pos1, p->gap_pos2);
    if (len1 == 0 || len2 == 0)
        mm = 0;
    else
        mm /= (float)(len1 < len2 ? len1 : len2);
    r->dist = ((float)100.0 - mm) / (float)100.0;
    r->n_ident = count;
    r->n_match = w.n_match;
    r->print_ptr = w.print_ptr;
    r->cells_fwd = (int64_t)n * m;
    r->cells_rev = w.cells_rev;
    r->cells_diff = w.cells_diff;
}

/* ---------------------------------------------------------------- batch API */

typedef struct {
    const int8_t* codes;
    const int64_t* offsets;
    const int32_t* lens;
    const int32_t (*mat)[NUMRES];
    const cwo_params* p;
    const int32_t* pairs;
    int64_t npairs;
    cwo_pair_result* out;
    int maxlen;
    int64_t next;
    pthread_mutex_t mu;
} cwo_job;

static void* worker(void* arg) {
    cwo_job* j = (cwo_job*)arg;
    int* scratch = (int*)malloc(sizeof(int) * scratch_ints(j->maxlen));
    if (!scratch) return (void*)1;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int64_t lo = j->next;
        j->next += 16;
        pthread_mutex_unlock(&j->mu);
        if (lo >= j->npairs) break;
        int64_t hi = lo + 16 < j->npairs ? lo + 16 : j->npairs;
        for (int64_t q = lo; q < hi; q++) {
            int a = j->pairs[2 * q], b = j->pairs[2 * q + 1];
            align_one(j->mat, j->p, j->codes + j->offsets[a], j->lens[a], j->codes + j->offsets[b],
                      j->lens[b], j->maxlen, scratch, &j->out[q]);
        }
    }
    free(scratch);
    return 0;
}

/* Aligns the listed pairs (pairs[2q] = row sequence si, pairs[2q+1] = column
 * sequence sj, 0-based) with `nthreads` threads. Returns 0 on success. */
int cwo_align_pairs(const int8_t* codes, const int64_t* offsets, const int32_t* lens, int32_t nseqs,
                    const int32_t* matrix, const cwo_params* p, const int32_t* pairs, int64_t npairs,
                    cwo_pair_result* out, int32_t nthreads) {
    cwo_job j;
    int maxlen = 1;
    for (int s = 0; s < nseqs; s++)
        if (lens[s] > maxlen) maxlen = lens[s];
    for (int64_t q = 0; q < npairs; q++) {
        if (pairs[2 * q] < 0 || pairs[2 * q] >= nseqs || pairs[2 * q + 1] < 0 || pairs[2 * q + 1] >= nseqs)
            return 1;
    }
    j.codes = codes;
    j.offsets = offsets;
    j.lens = lens;
    j.mat = (const int32_t (*)[NUMRES])matrix;
    j.p = p;
    j.pairs = pairs;
    j.npairs = npairs;
    j.out = out;
    j.maxlen = maxlen;
    j.next = 0;
    pthread_mutex_init(&j.mu, 0);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 512) nthreads = 512;
    pthread_t th[512];
    int started = 0, rc = 0;
    for (int t = 1; t < nthreads; t++) {
        if (pthread_create(&th[started], 0, worker, &j) == 0) started++;
    }
    if (worker(&j)) rc = 2;
    for (int t = 0; t < started; t++) {
        void* ret = 0;
        pthread_join(th[t], &ret);
        if (ret) rc = 2;
    }
    pthread_mutex_destroy(&j.mu);
    return rc;
}

/* ------------------------------------------------------------ guide tree */

/* SymMatrix::getIndex (general/SymMatrix.h:166-197) for 1-based i, j. */
static size_t sym_idx(int i, int j) {
    if (i == 0 || j == 0) return 0;
    int a = i - 1, b = j - 1;
    if (a == b) return ((size_t)a * (a + 3)) >> 1;
    if (a < b) {
        int t = a;
        a = b;
        b = t;
    }
    return (((size_t)a * (a + 1)) >> 1) + b;
}

/* Neighbour joining, NJTree::generateTree (tree/NJTree.cpp:161-748) with
 * firstSeq = 1, lastSeq = n, as UnRootedClusterTree::treeFromDistMatrix calls
 * it. d: packed SymMatrix elements of size n+1, updated in place like the
 * reference. left/right: n+2 doubles; desc: (n+1)*(n+1) ints, row-major.
 * Valid nodes are kept in ascending order, which is the order the reference's
 * linked list visits them. joins (may be NULL): 2*(n-3) ints, (mini, minj) of
 * every cycle, as the verbose report names them (NJTree.cpp:413-470).
 * Returns 0, or 1 if n < 2. */
int cwo_nj_tree(int n, double* d, double* left, double* right, int32_t* desc, int32_t* joins) {
    if (n < 2) return 1;
    if (n == 2) return 0; /* :218-229 returns before touching the tree */
    const int W = n + 1;
    double* sumCols = (double*)calloc(n + 1, sizeof(double));
    double* sumRows = (double*)calloc(n + 1, sizeof(double));
    double* join = (double*)calloc(n + 1, sizeof(double));
    double* av = (double*)calloc(n + 1, sizeof(double));
    char* valid = (char*)calloc(n + 2, 1);
    int i, j, ii, jj, nc, mini, minj;
    double fnseqs = (double)n, fnseqs2 = 0, sumd, tmin, total, diq, djq, dij, dio, djo, dmin, bi, bj, da;
    for (i = 0; i < n + 2; i++) left[i] = right[i] = 0.0;
    memset(desc, 0, sizeof(int32_t) * (size_t)W * W);
    for (i = 1; i <= n; i++) {
        d[sym_idx(i, i)] = av[i] = 0.0;
        valid[i] = 1;
    }
    for (j = 1; j <= n; j++) {
        double s = 0.0;
        for (i = 1; i < j; i++) s = s + d[sym_idx(i, j)];
        sumRows[j] = s;
        s = 0.0;
        for (i = j + 1; i <= n; i++) s += d[sym_idx(j, i)];
        sumCols[j] = s;
    }
    for (nc = 1; nc <= n - 3; ++nc) {
        sumd = 0.0;
        for (j = 1; j <= n; j++)
            if (valid[j]) sumd += sumCols[j];
        fnseqs2 = fnseqs - 2.0;
        tmin = 99999.0 * 2.0 * fnseqs2;
        mini = minj = 0;
        for (jj = 2; jj <= n; jj++) {
            if (!valid[jj]) continue;
            for (ii = 1; ii < jj; ii++) {
                if (!valid[ii]) continue;
                diq = sumCols[ii] + sumRows[ii];
                djq = sumCols[jj] + sumRows[jj];
                dij = d[sym_idx(ii, jj)];
                total = fnseqs2 * dij + 2.0 * sumd - diq - djq;
                if (total < tmin) {
                    tmin = total;
                    mini = ii;
                    minj = jj;
                }
            }
        }
        dio = sumCols[mini] + sumRows[mini];
        djo = sumCols[minj] + sumRows[minj];
        dmin = d[sym_idx(mini, minj)];
        dio = (dio - dmin) / fnseqs2;
        djo = (djo - dmin) / fnseqs2;
        bi = (dmin + dio - djo) * 0.5;
        bj = dmin - bi;
        bi = bi - av[mini];
        bj = bj - av[minj];
        const int typei = av[mini] > 0.0 ? 0 : 1, typej = av[minj] > 0.0 ? 0 : 1;
        if (fabs(bi) < 0.0001) bi = 0.0;
        if (fabs(bj) < 0.0001) bj = 0.0;
        left[nc] = bi;
        right[nc] = bj;
        if (joins) {
            joins[2 * (nc - 1)] = mini;
            joins[2 * (nc - 1) + 1] = minj;
        }
        for (i = 1; i <= n; i++) desc[(size_t)nc * W + i] = 0;
        const int who[2] = {mini, minj}, typ[2] = {typei, typej};
        for (int side = 0; side < 2; side++) {
            if (typ[side] == 0) {
                for (i = nc - 1; i >= 1; i--)
                    if (desc[(size_t)i * W + who[side]] == 1) {
                        for (j = 1; j <= n; j++)
                            if (desc[(size_t)i * W + j] == 1) desc[(size_t)nc * W + j] = 1;
                        break;
                    }
            } else {
                desc[(size_t)nc * W + who[side]] = 1;
            }
        }
        if (dmin <= 0.0) dmin = 0.000001;
        av[mini] = dmin * 0.5;
        fnseqs = fnseqs - 1.0;
        valid[minj] = 0;
        for (j = 1; j <= n; j++) {
            if (!valid[j]) continue;
            double tmp_di = 0.0, tmp_dj = 0.0;
            if (j < minj) {
                tmp_dj = d[sym_idx(j, minj)];
                sumCols[j] -= tmp_dj;
            } else if (j > minj) {
                tmp_dj = d[sym_idx(minj, j)];
                sumRows[j] -= tmp_dj;
            }
            if (j < mini) {
                tmp_di = d[sym_idx(j, mini)];
                sumCols[j] -= tmp_di;
            } else if (j > mini) {
                tmp_di = d[sym_idx(mini, j)];
                sumRows[j] -= tmp_di;
            }
            join[j] = (tmp_dj + tmp_di) * 0.5;
        }
        for (j = 1; j <= n; j++) {
            if (!valid[j]) continue;
            if (j < mini) {
                d[sym_idx(j, mini)] = join[j];
                sumCols[j] += join[j];
            } else if (j > mini) {
                d[sym_idx(mini, j)] = join[j];
                sumRows[j] += join[j];
            }
        }
        sumCols[mini] = sumRows[mini] = 0.0;
        da = 0.0;
        for (j = 1; j < mini; j++)
            if (valid[j]) da = da + join[j];
        sumRows[mini] = da;
        da = 0.0;
        for (j = mini + 1; j <= n; j++)
            if (valid[j]) da = da + join[j];
        sumCols[mini] = da;
        sumCols[minj] = sumRows[minj] = 0.0;
        for (j = 1; j <= n; ++j) {
            d[sym_idx(minj, j)] = 0.0;
            d[sym_idx(j, minj)] = 0.0;
            join[j] = 0.0;
        }
    }
    /* last cycle: three nodes left (:646-737) */
    int l[4], nude = 1;
    for (i = 1; i <= n; i++)
        if (valid[i]) l[nude++] = i;
    double b1 = (d[sym_idx(l[1], l[2])] + d[sym_idx(l[1], l[3])] - d[sym_idx(l[2], l[3])]) * 0.5;
    double b2 = d[sym_idx(l[1], l[2])] - b1;
    double b3 = d[sym_idx(l[1], l[3])] - b1;
    double branch[4];
    branch[1] = b1 - av[l[1]];
    branch[2] = b2 - av[l[2]];
    branch[3] = b3 - av[l[3]];
    for (i = 1; i <= 3; i++)
        if (fabs(branch[i]) < 0.0001) branch[i] = 0.0;
    left[n - 2] = branch[1];
    left[n - 1] = branch[2];
    left[n] = branch[3];
    for (i = 1; i <= n; i++) desc[(size_t)(n - 2) * W + i] = 0;
    for (i = 1; i <= 3; ++i) {
        if (av[l[i]] > 0.0) {
            for (int k = n - 3; k >= 1; k--)
                if (desc[(size_t)k * W + l[i]] == 1) {
                    for (j = 1; j <= n; j++)
                        if (desc[(size_t)k * W + j] == 1) desc[(size_t)(n - 2) * W + j] = i;
                    break;
                }
        } else {
            desc[(size_t)(n - 2) * W + l[i]] = i;
        }
    }
    free(sumCols);
    free(sumRows);
    free(join);
    free(av);
    free(valid);
    return 0;
}

/* ------------------------------------------------- k-tuple quick distances */

/* The userParameters values FastPairwiseAlign::pairAlign reads
 * (pairwise/FastPairwiseAlign.cpp:176-183), after setDNAParams/setProtParams. */
typedef struct cwo_fast_params {
    int32_t dna, ktup, window, window_gap, signif, percent, max_aa, max_aln_length;
} cwo_fast_params;

typedef struct cwo_fast_result {
    double dist;       /* (100 - calcScore) / 100, as SetAt stores it */
    int32_t score;     /* accum[0][maxSoFar], 0 if no fragment */
    int32_t frags;     /* fragments made (currFrag) */
    int32_t partial;   /* the "(Partial alignment)" cut-off was hit */
    int32_t pad;
} cwo_fast_result;

typedef struct fast_scratch {
    int *displ, *slopes, *diag, *zza, *zzb, *zzc, *zzd, *acc[5];
} fast_scratch;

/* FastPairwiseAlign.cpp:163-164: A C G T U -> 0 1 2 3 3, anything else -1. */
static int aa2dna(int code) {
    switch (code) {
        case 0: return 0;
        case 2: return 1;
        case 6: return 2;
        case 18: case 19: return 3;
        default: return -1;
    }
}

/* makePPtrs / makeNPtrs (FastPairwiseAlign.cpp:406-510): pl[code] = last
 * position of each k-tuple code, tptr[i] = previous position with the same
 * code (0 ends the chain). seq is 0-based here, positions 1-based. */
static void make_ptrs(const cwo_fast_params* P, int* tptr, int* pl, const int8_t* seq, int length) {
    const int base = P->dna ? 4 : P->max_aa + 1;
    int limit = 1, a[10], i, j;
    a[1] = 1;
    for (i = 2; i <= P->ktup; i++) a[i] = a[i - 1] * base;
    for (i = 1; i <= P->ktup; i++) limit *= base;
    for (i = 1; i <= limit; ++i) pl[i] = 0;
    for (i = 1; i <= length; ++i) tptr[i] = 0;
    for (i = 1; i <= length - P->ktup + 1; ++i) {
        int code = 0, bad = 0;
        for (j = 1; j <= P->ktup; ++j) {
            int r = seq[i + j - 2];
            if (P->dna) {
                r = (r >= 0 && r < 36) ? aa2dna(r) : -1;
                if (r < 0 || r > 3) { bad = 1; break; }
            } else if (r < 0 || r > P->max_aa) {
                bad = 1;
                break;
            }
            code += r * a[j];
        }
        if (bad) continue;
        ++code;
        if (pl[code] != 0) tptr[i] = pl[code];
        pl[code] = i;
    }
}

/* desQuickSort (FastPairwiseAlign.cpp:585-658): the reference's quicksort of
 * array1[1 .. size-1] ascending, array2 permuted alongside. Element `size`
 * itself is not part of the sort. */
static void des_quick_sort(int* array1, int* array2, int size) {
    int lst[50], ust[50], p = 1, i, j, t;
    lst[1] = 1;
    ust[1] = size - 1;
    while (p > 0) {
        if (lst[p] >= ust[p]) {
            p--;
        } else {
            i = lst[p] - 1;
            j = ust[p];
            int piv = array1[j];
            while (i < j) {
                for (i = i + 1; array1[i] < piv; i++)
                    ;
                for (j = j - 1; j > i; j--)
                    if (array1[j] <= piv) break;
                if (i < j) {
                    t = array1[i]; array1[i] = array1[j]; array1[j] = t;
                    t = array2[i]; array2[i] = array2[j]; array2[j] = t;
                }
            }
            j = ust[p];
            t = array1[i]; array1[i] = array1[j]; array1[j] = t;
            t = array2[i]; array2[i] = array2[j]; array2[j] = t;
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
        }
    }
}

/* fragRelPos (FastPairwiseAlign.cpp:563-583). */
static int frag_rel_pos(int a1, int b1, int a2, int b2, int ktup) {
    if (a1 - b1 == a2 - b2) return a2 < a1;
    return a2 + ktup - 1 < a1 && b2 + ktup - 1 < b1;
}

/* putFrag (FastPairwiseAlign.cpp:524-561): fragments kept in a list sorted by
 * score, accum[4] the links, maxSoFar the head. */
static void put_frag(int** acc, int* maxSoFar, int currFrag, int fs, int v1, int v2, int flen) {
    acc[0][currFrag] = fs;
    acc[1][currFrag] = v1;
    acc[2][currFrag] = v2;
    acc[3][currFrag] = flen;
    if (!*maxSoFar) {
        *maxSoFar = 1;
        acc[4][currFrag] = 0;
        return;
    }
    if (fs >= acc[0][*maxSoFar]) {
        acc[4][currFrag] = *maxSoFar;
        *maxSoFar = currFrag;
        return;
    }
    int next = *maxSoFar, end;
    while (1) {
        end = next;
        next = acc[4][next];
        if (fs >= acc[0][next]) break;
    }
    acc[4][currFrag] = next;
    acc[4][end] = currFrag;
}

/* pairAlign (FastPairwiseAlign.cpp:168-400) for sequence 1 (already in
 * zza/zzc) against sequence 2 (zzb/zzd). */
static void pair_align(const cwo_fast_params* P, fast_scratch* S, const int8_t* seq, int l1, int l2,
                       cwo_fast_result* R) {
    const int ktup = P->ktup;
    const int base = P->dna ? 4 : P->max_aa + 1;
    int pot[10], limit = 1, i, j;
    pot[1] = 1;
    for (i = 2; i <= ktup; i++) pot[i] = pot[i - 1] * base;
    for (i = 1; i <= ktup; i++) limit *= base;
    int* displ = S->displ;
    int* slopes = S->slopes;
    int* diag = S->diag;
    int** acc = S->acc;
    const int tl1 = (l1 + l2) - 1;
    for (i = 1; i <= tl1; ++i) {
        slopes[i] = displ[i] = 0;
        diag[i] = i;
    }
    /* diagonal hit counts */
    for (i = 1; i <= limit; ++i) {
        int vn1 = S->zzc[i];
        while (vn1) {
            int vn2 = S->zzd[i];
            while (vn2 != 0) {
                ++displ[vn1 - vn2 + l2];
                vn2 = S->zzb[vn2];
            }
            vn1 = S->zza[vn1];
        }
    }
    des_quick_sort(displ, diag, tl1);
    j = tl1 - P->signif + 1;
    if (j < 1) j = 1;
    for (i = tl1; i >= j; i--)
        if (displ[i] > 0) {
            int pos = diag[i];
            int l = (1 > pos - P->window) ? 1 : pos - P->window;
            int m = (tl1 < pos + P->window) ? tl1 : pos + P->window;
            for (; l <= m; l++) slopes[l] = 1;
        }
    for (i = 1; i <= tl1; i++) displ[i] = 0;
    int currFrag = 0, maxSoFar = 0, next = 0;
    R->partial = 0;
    for (i = 1; i <= (l1 - ktup + 1); ++i) {
        int encrypt = 0, bad = 0;
        for (j = 1; j <= ktup; ++j) {
            int r = seq[i + j - 2];
            if (P->dna) {
                r = (r >= 0 && r < 36) ? aa2dna(r) : -1;
                if (r < 0 || r > 3) { bad = 1; break; }
            } else if (r < 0 || r > P->max_aa) {
                bad = 1;
                break;
            }
            encrypt += r * pot[j];
        }
        if (bad) continue;
        ++encrypt;
        int vn2 = S->zzd[encrypt];
        while (vn2) {
            int osptr = i - vn2 + l2;
            if (slopes[osptr] != 1) {
                vn2 = S->zzb[vn2];
                continue;
            }
            int flen = 0, fs = ktup;
            next = maxSoFar;
            /* the A-loop */
            while (1) {
                if (!next) {
                    ++currFrag;
                    if (currFrag >= 2 * P->max_aln_length) {
                        R->partial = 1;
                        goto done;
                    }
                    displ[osptr] = currFrag;
                    put_frag(acc, &maxSoFar, currFrag, fs, i, vn2, flen);
                } else {
                    int tv1 = acc[1][next], tv2 = acc[2][next];
                    if (frag_rel_pos(i, vn2, tv1, tv2, ktup)) {
                        if (i - vn2 == acc[1][next] - acc[2][next]) {
                            if (i > acc[1][next] + (ktup - 1)) {
                                fs = acc[0][next] + ktup;
                            } else {
                                fs = acc[0][next] + (i - acc[1][next]);
                            }
                            flen = next;
                            next = 0;
                            continue;
                        } else {
                            int subt1, subt2;
                            if (displ[osptr] == 0) {
                                subt1 = ktup;
                            } else if (i > acc[1][displ[osptr]] + (ktup - 1)) {
                                subt1 = acc[0][displ[osptr]] + ktup;
                            } else {
                                subt1 = acc[0][displ[osptr]] + (i - acc[1][displ[osptr]]);
                            }
                            subt2 = acc[0][next] - P->window_gap + ktup;
                            if (subt2 > subt1) {
                                flen = next;
                                fs = subt2;
                            } else {
                                flen = displ[osptr];
                                fs = subt1;
                            }
                            next = 0;
                            continue;
                        }
                    } else {
                        next = acc[4][next];
                        continue;
                    }
                }
                break;
            }
            vn2 = S->zzb[vn2];
        }
    }
done:
    R->frags = currFrag;
    R->score = maxSoFar ? acc[0][maxSoFar] : 0;
    {
        /* FastPairwiseAlign.cpp:88-103, in double */
        double calc = 0.0;
        if (maxSoFar) {
            calc = (double)acc[0][maxSoFar];
            if (P->percent) {
                int dsr = l1 < l2 ? l1 : l2;
                calc = (calc / (double)dsr) * 100.0;
            }
        }
        R->dist = (100.0 - calc) / 100.0;
    }
}

typedef struct fast_job {
    const int8_t* codes;
    const int64_t* offsets;
    const int32_t* lens;
    const cwo_fast_params* P;
    const int32_t* pairs;
    int64_t npairs;
    cwo_fast_result* out;
    int64_t next;
    pthread_mutex_t mu;
    int lmax;
} fast_job;

static void* fast_worker(void* arg) {
    fast_job* J = (fast_job*)arg;
    const cwo_fast_params* P = J->P;
    const int base = P->dna ? 4 : P->max_aa + 1;
    int limit = 1, k;
    for (k = 0; k < P->ktup; k++) limit *= base;
    const int nd = 2 * J->lmax + 2, na = 2 * P->max_aln_length + 2;
    fast_scratch S;
    S.displ = (int*)calloc(nd, sizeof(int));
    S.slopes = (int*)calloc(nd, sizeof(int));
    S.diag = (int*)calloc(nd, sizeof(int));
    S.zza = (int*)calloc(J->lmax + 2, sizeof(int));
    S.zzb = (int*)calloc(J->lmax + 2, sizeof(int));
    S.zzc = (int*)calloc(limit + 2, sizeof(int));
    S.zzd = (int*)calloc(limit + 2, sizeof(int));
    for (k = 0; k < 5; k++) S.acc[k] = (int*)calloc(na, sizeof(int));
    while (1) {
        pthread_mutex_lock(&J->mu);
        int64_t q = J->next;
        J->next += 16;
        pthread_mutex_unlock(&J->mu);
        if (q >= J->npairs) break;
        int64_t qe = q + 16 < J->npairs ? q + 16 : J->npairs;
        for (; q < qe; ++q) {
            const int si = J->pairs[2 * q], sj = J->pairs[2 * q + 1];
            const int8_t* s1 = J->codes + J->offsets[si];
            const int8_t* s2 = J->codes + J->offsets[sj];
            make_ptrs(P, S.zza, S.zzc, s1, J->lens[si]);
            make_ptrs(P, S.zzb, S.zzd, s2, J->lens[sj]);
            pair_align(P, &S, s1, J->lens[si], J->lens[sj], &J->out[q]);
        }
    }
    free(S.displ); free(S.slopes); free(S.diag); free(S.zza); free(S.zzb); free(S.zzc); free(S.zzd);
    for (k = 0; k < 5; k++) free(S.acc[k]);
    return 0;
}

/* FastPairwiseAlign::pairwiseAlign over a pair list (0-based si < sj); each
 * pair's result is independent of the others (the reference resets its
 * per-pair state in makePPtrs/makeNPtrs/pairAlign). */
int cwo_fast_pairs(const int8_t* codes, const int64_t* offsets, const int32_t* lens, int32_t nseqs,
                   const cwo_fast_params* P, const int32_t* pairs, int64_t npairs, cwo_fast_result* out,
                   int32_t nthreads) {
    if (P->ktup < 1 || P->ktup > 8) return 1;
    fast_job J;
    int k;
    J.codes = codes; J.offsets = offsets; J.lens = lens; J.P = P; J.pairs = pairs; J.npairs = npairs;
    J.out = out; J.next = 0; J.lmax = 1;
    for (k = 0; k < nseqs; k++) if (lens[k] > J.lmax) J.lmax = lens[k];
    pthread_mutex_init(&J.mu, 0);
    if (nthreads < 1) nthreads = 1;
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    for (k = 0; k < nthreads; k++) pthread_create(&th[k], 0, fast_worker, &J);
    for (k = 0; k < nthreads; k++) pthread_join(th[k], 0);
    pthread_mutex_destroy(&J.mu);
    return 0;
}
