/*
 * Test double of the GB300 library for running the C++ drop-ins
 * (cuda-clustalw_gb300/host/Gpu*.cpp) on a host without a GPU. It implements
 * the calls of include/cwgpu.h and include/cwgpu_nj.h that the drop-ins make,
 * with the oracle restatement (oracle/oracle.c, compiled into this file).
 *
 * TEST INFRASTRUCTURE ONLY. tests/test_dropin_run.py links the drop-ins
 * against this file and the unmodified reference objects to check the
 * drop-ins' own host code (reading the reference's globals, flattening the
 * SeqArray, ranges, DistMatrix writes, info lines, the tree plugin) against
 * the reference classes. The product library is lib/libcwgpu.so, which has no
 * CPU path; nothing shipped links this file.
 */
#include "../oracle/oracle.c"

#include "cwgpu.h"
#include "cwgpu_nj.h"

struct cwgpu_context {
    int32_t matrix[CWGPU_NUMRES * CWGPU_NUMRES];
    cwo_params params;
    int8_t* codes;
    int64_t* offsets;
    int32_t* lens;
    int32_t nseqs;
};

struct cwgpu_nj {
    int unused;
};

const char* cwgpu_status_string(int status) { return status ? "error (test double)" : "ok"; }
const char* cwgpu_last_error(const cwgpu_context* ctx) { (void)ctx; return ""; }

int cwgpu_create(int device, cwgpu_context** out) {
    (void)device;
    *out = (cwgpu_context*)calloc(1, sizeof(cwgpu_context));
    return *out ? CWGPU_OK : CWGPU_ERR_OOM;
}

void cwgpu_destroy(cwgpu_context* ctx) {
    if (!ctx) return;
    free(ctx->codes);
    free(ctx->offsets);
    free(ctx->lens);
    free(ctx);
}

int cwgpu_set_matrix(cwgpu_context* ctx, const int32_t* matrix) {
    memcpy(ctx->matrix, matrix, sizeof(ctx->matrix));
    return CWGPU_OK;
}

int cwgpu_set_params(cwgpu_context* ctx, const cwgpu_params* p) {
    ctx->params.dna = p->dna;
    ctx->params.pw_gap_open = p->pw_gap_open;
    ctx->params.pw_gap_extend = p->pw_gap_extend;
    ctx->params.int_scale = p->int_scale;
    ctx->params.gap_open_scale = p->gap_open_scale;
    ctx->params.gap_extend_scale = p->gap_extend_scale;
    ctx->params.mat_avg = p->mat_avg;
    ctx->params.gap_pos1 = p->gap_pos1;
    ctx->params.gap_pos2 = p->gap_pos2;
    return CWGPU_OK;
}

int cwgpu_upload_seqs(cwgpu_context* ctx, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                      const int32_t* lens) {
    int64_t total = 0;
    int s;
    for (s = 0; s < nseqs; s++) total += lens[s];
    free(ctx->codes);
    free(ctx->offsets);
    free(ctx->lens);
    ctx->codes = (int8_t*)malloc(total > 0 ? (size_t)total : 1);
    ctx->offsets = (int64_t*)malloc(sizeof(int64_t) * (nseqs > 0 ? nseqs : 1));
    ctx->lens = (int32_t*)malloc(sizeof(int32_t) * (nseqs > 0 ? nseqs : 1));
    total = 0;
    for (s = 0; s < nseqs; s++) {
        if (lens[s] > 0) memcpy(ctx->codes + total, codes + offsets[s], (size_t)lens[s]);
        ctx->offsets[s] = total;
        ctx->lens[s] = lens[s];
        total += lens[s];
    }
    ctx->nseqs = nseqs;
    return CWGPU_OK;
}

int64_t cwgpu_range_pair_count(int32_t nseqs, int32_t i_start, int32_t i_end, int32_t j_start, int32_t j_end) {
    int64_t c = 0;
    int32_t si;
    for (si = i_start < 0 ? 0 : i_start; si < nseqs && si < i_end; si++) {
        int64_t lo = (int64_t)si + 1 > (int64_t)j_start + 1 ? (int64_t)si + 1 : (int64_t)j_start + 1;
        int64_t hi = nseqs < j_end ? nseqs : j_end;
        if (hi > lo) c += hi - lo;
    }
    return c;
}

/* The range loops of the reference, as 0-based (si, sj) pairs. */
static int32_t* range_list(int32_t n, int32_t i0, int32_t i1, int32_t j0, int32_t j1, int64_t* np) {
    int64_t q = 0;
    int32_t si, sj;
    int32_t* pairs;
    *np = cwgpu_range_pair_count(n, i0, i1, j0, j1);
    pairs = (int32_t*)malloc(sizeof(int32_t) * 2 * (size_t)(*np > 0 ? *np : 1));
    for (si = i0 < 0 ? 0 : i0; si < n && si < i1; si++)
        for (sj = (si + 1 > j0 + 1 ? si + 1 : j0 + 1); sj < n && sj < j1; sj++) {
            pairs[2 * q] = si;
            pairs[2 * q + 1] = sj;
            q++;
        }
    return pairs;
}

int cwgpu_pairwise_align(cwgpu_context* ctx, int32_t i_start, int32_t i_end, int32_t j_start, int32_t j_end,
                         double* elements, int32_t dist_size, cwgpu_pair_stats* stats_out) {
    int64_t np, q;
    int32_t* pairs;
    cwo_pair_result* r;
    if (dist_size != ctx->nseqs + 1) return CWGPU_ERR_ARG;
    if (i_start < 0 || i_end < i_start || j_start < 0 || j_end < j_start) return CWGPU_ERR_RANGE;
    pairs = range_list(ctx->nseqs, i_start, i_end, j_start, j_end, &np);
    r = (cwo_pair_result*)calloc((size_t)(np > 0 ? np : 1), sizeof(cwo_pair_result));
    if (np > 0 && cwo_align_pairs(ctx->codes, ctx->offsets, ctx->lens, ctx->nseqs, ctx->matrix, &ctx->params,
                                  pairs, np, r, 1)) {
        free(pairs);
        free(r);
        return CWGPU_ERR_ARG;
    }
    for (q = 0; q < np; q++) {
        int64_t i = pairs[2 * q], j = pairs[2 * q + 1];
        elements[((j * (j + 1)) >> 1) + i] = (double)r[q].dist;
        if (stats_out) {
            stats_out[q].fwd_score = r[q].fwd_score;
            stats_out[q].se1 = r[q].se1;
            stats_out[q].se2 = r[q].se2;
            stats_out[q].sb1 = r[q].sb1;
            stats_out[q].sb2 = r[q].sb2;
            stats_out[q].mm_score = r[q].mm_score;
            stats_out[q].n_ident = r[q].n_ident;
            stats_out[q].n_match = r[q].n_match;
        }
    }
    free(pairs);
    free(r);
    return CWGPU_OK;
}

int cwgpu_fast_pairwise_align(cwgpu_context* ctx, const cwgpu_fast_params* p, int32_t i_start, int32_t i_end,
                              int32_t j_start, int32_t j_end, double* elements, int32_t dist_size,
                              cwgpu_fast_stats* stats_out) {
    int64_t np, q;
    int32_t* pairs;
    cwo_fast_result* r;
    cwo_fast_params P;
    if (dist_size != ctx->nseqs + 1) return CWGPU_ERR_ARG;
    if (i_start < 0 || i_end < i_start || j_start < 0 || j_end < j_start) return CWGPU_ERR_RANGE;
    P.dna = p->dna;
    P.ktup = p->ktup;
    P.window = p->window;
    P.window_gap = p->window_gap;
    P.signif = p->signif;
    P.percent = p->percent;
    P.max_aa = p->max_aa;
    P.max_aln_length = p->max_aln_length;
    pairs = range_list(ctx->nseqs, i_start, i_end, j_start, j_end, &np);
    r = (cwo_fast_result*)calloc((size_t)(np > 0 ? np : 1), sizeof(cwo_fast_result));
    if (np > 0 && cwo_fast_pairs(ctx->codes, ctx->offsets, ctx->lens, ctx->nseqs, &P, pairs, np, r, 1)) {
        free(pairs);
        free(r);
        return CWGPU_ERR_ARG;
    }
    for (q = 0; q < np; q++) {
        int64_t i = pairs[2 * q], j = pairs[2 * q + 1];
        elements[((j * (j + 1)) >> 1) + i] = r[q].dist;
        if (stats_out) {
            stats_out[q].score = r[q].score;
            stats_out[q].frags = r[q].frags;
            stats_out[q].partial = r[q].partial;
            stats_out[q].pad = 0;
        }
    }
    free(pairs);
    free(r);
    return CWGPU_OK;
}

int cwgpu_nj_create(int device, cwgpu_nj** out) {
    (void)device;
    *out = (cwgpu_nj*)calloc(1, sizeof(cwgpu_nj));
    return *out ? CWGPU_OK : CWGPU_ERR_OOM;
}

void cwgpu_nj_destroy(cwgpu_nj* nj) { free(nj); }

const char* cwgpu_nj_last_error(const cwgpu_nj* nj) { (void)nj; return ""; }

int cwgpu_nj_tree(cwgpu_nj* nj, int32_t n, double* elements, double* left_branch, double* right_branch,
                  int32_t* tree_desc, int32_t* joins) {
    (void)nj;
    return cwo_nj_tree(n, elements, left_branch, right_branch, tree_desc, joins) ? CWGPU_ERR_ARG : CWGPU_OK;
}
