/*
 * cwgpu.h - C ABI of the GB300 (sm_103a) full-pairwise distance stage.
 *
 * This library computes what ClustalW 2.0.11's
 * clustalw::FullPairwiseAlign::pairwiseAlign computes
 * (CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.cpp:34-211): for every
 * sequence pair, Gotoh local forward and reverse score sweeps, Myers-Miller
 * linear-space alignment of the local segment, the identity count along that
 * path and the distance (100 - 100*ident/min(len1,len2))/100 in float. Results
 * are bit-identical to the reference on the same inputs.
 *
 * The reference plugin interface this replaces is the pure virtual
 *   PairwiseAlignBase::pairwiseAlign(Alignment*, DistMatrix*, int iStart,
 *                                    int iEnd, int jStart, int jEnd)
 * (CPU/clustalw-2.0.11/src/pairwise/PairwiseAlignBase.h:19-20). The C++ class
 * in cuda-clustalw_gb300/host/GpuFullPairwiseAlign.h implements it on top of
 * these functions.
 *
 * Conventions: plain pointers and sizes only; sequence indices are 0-based
 * (si, sj) like the reference's loop variables, and DistMatrix positions are
 * the reference's 1-based (si+1, sj+1). Every call returns a cwgpu_status; no
 * call exits the process. A context owns one CUDA device and is not
 * thread-safe (like the reference class, which keeps static locals in diff()).
 */
#ifndef CWGPU_H
#define CWGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CWGPU_NUMRES 32       /* clustalw NUMRES (general/clustalw.h:231) */
#define CWGPU_MAX_SEQ_LEN 65535 /* longest sequence a context accepts */
/* Longest pair list one call takes (the work order holds 32-bit positions).
 * The range calls (cwgpu_pairwise_align, cwgpu_fast_pairwise_align) split
 * larger ranges into blocks of whole rows themselves; a served job may have at
 * most this many pairs. */
#define CWGPU_MAX_PAIRS_PER_CALL 2147483647LL

typedef enum cwgpu_status {
    CWGPU_OK = 0,
    CWGPU_ERR_ARG = 1,        /* bad pointer, size, code or range */
    CWGPU_ERR_CUDA = 2,       /* a CUDA runtime call failed (see cwgpu_last_error) */
    CWGPU_ERR_OOM = 3,        /* device allocation failed or over the memory budget */
    CWGPU_ERR_STATE = 4,      /* matrix / params / sequences not set yet */
    CWGPU_ERR_RANGE = 5,      /* iStart..jEnd range rejected (FullPairwiseAlign.cpp:53-58) */
    CWGPU_ERR_TIMEOUT = 6,    /* a bounded device wait ran out */
    CWGPU_ERR_DEVICE = 7,     /* the kernel reported an internal limit (stack depth) */
    CWGPU_ERR_MATRIX = 8,     /* a matrix entry does not fit the int16 score profile */
    CWGPU_ERR_NOT_FOUND = 9   /* unknown job id */
} cwgpu_status;

/* The scalars FullPairwiseAlign::pairwiseAlign reads from userParameters and
 * from SubMatrix::getPairwiseMatrix (FullPairwiseAlign.cpp:69-94). */
typedef struct cwgpu_params {
    int32_t dna;            /* userParameters->getDNAFlag() */
    float pw_gap_open;      /* userParameters->getPWGapOpen() */
    float pw_gap_extend;    /* userParameters->getPWGapExtend() */
    int32_t int_scale;      /* PairScaleValues::intScale */
    float gap_open_scale;   /* PairScaleValues::gapOpenScale */
    float gap_extend_scale; /* PairScaleValues::gapExtendScale */
    int32_t mat_avg;        /* matAvg returned by getPairwiseMatrix */
    int32_t gap_pos1;       /* userParameters->getGapPos1() */
    int32_t gap_pos2;       /* userParameters->getGapPos2() */
} cwgpu_params;

/* Per-pair intermediate results (members of FullPairwiseAlign after the pair). */
typedef struct cwgpu_pair_stats {
    int32_t fwd_score; /* forwardPass maxScore (FullPairwiseAlign.cpp:285-338) */
    int32_t se1, se2;  /* forwardPass end cell */
    int32_t sb1, sb2;  /* reversePass start cell (:350-408) */
    int32_t mm_score;  /* diff() return value (:165) */
    int32_t n_ident;   /* tracePath identity count (:231-278) */
    int32_t n_match;   /* aligned residue pairs on the Myers-Miller path */
} cwgpu_pair_stats;

typedef struct cwgpu_context cwgpu_context;

/* ---- context ------------------------------------------------------------ */

/* Creates a context on CUDA device `device`. No reference counterpart: the
 * reference class allocates its scratch in pairwiseAlign (:74-78). */
int cwgpu_create(int device, cwgpu_context** out);
/* Frees all device memory of the context. Replaces ~FullPairwiseAlign. */
void cwgpu_destroy(cwgpu_context* ctx);
/* Static text for a status code. */
const char* cwgpu_status_string(int status);
/* Detail text of the last failure on this context ("" if none). */
const char* cwgpu_last_error(const cwgpu_context* ctx);

/* ---- inputs ------------------------------------------------------------- */

/* The 32x32 int matrix from SubMatrix::getPairwiseMatrix
 * (substitutionMatrix/SubMatrix.cpp:256-390), row-major matrix[a*32+b].
 * Replaces the `matrix` member filled at FullPairwiseAlign.cpp:81. Entries
 * must lie in [-32768, 32767]. */
int cwgpu_set_matrix(cwgpu_context* ctx, const int32_t* matrix);
/* Scalars of FullPairwiseAlign.cpp:69-94. */
int cwgpu_set_params(cwgpu_context* ctx, const cwgpu_params* params);
/* Uploads `nseqs` encoded sequences (SeqArray rows 1..nseqs without the dummy
 * element 0, Alignment.h:96): sequence s is codes[offsets[s] .. offsets[s] +
 * lens[s]), every code in [0, 31]. Replaces the getSeqArray()/getSeqLength()
 * reads at FullPairwiseAlign.cpp:95-127. */
int cwgpu_upload_seqs(cwgpu_context* ctx, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                      const int32_t* lens);

/* ---- host-side helpers (no device work) ----------------------------------- */

/* Per-pair integer gap penalties exactly as FullPairwiseAlign.cpp:129-148
 * computes them (same float/double expression types). */
int cwgpu_gap_penalties(const cwgpu_params* params, int32_t n, int32_t m, int32_t* gap_open,
                        int32_t* gap_extend);
/* Number of pairs the loops at FullPairwiseAlign.cpp:97 and :110 visit. */
int64_t cwgpu_range_pair_count(int32_t nseqs, int32_t i_start, int32_t i_end, int32_t j_start,
                               int32_t j_end);

/* ---- the pairwise stage --------------------------------------------------- */

/* The drop-in for pairwiseAlign(alignPtr, distMat, iStart, iEnd, jStart, jEnd)
 * (FullPairwiseAlign.cpp:34-211): aligns every pair the reference's loops visit
 * and stores each distance into `elements`, the packed lower-triangular double
 * array of a SymMatrix of size nseqs+1 (SymMatrix::getElements,
 * general/SymMatrix.h:67-71 and :166-197), at getIndex(si+1, sj+1).
 * `dist_size` is the SymMatrix's getSize() and must equal nseqs + 1 (:47-52,
 * else CWGPU_ERR_ARG). Pairs with an empty sequence get 1.0 like :113-118.
 * `stats_out`, if not NULL, receives cwgpu_range_pair_count(...) entries in
 * loop order. Returns CWGPU_ERR_RANGE for the ranges the reference rejects. */
int cwgpu_pairwise_align(cwgpu_context* ctx, int32_t i_start, int32_t i_end, int32_t j_start,
                         int32_t j_end, double* elements, int32_t dist_size, cwgpu_pair_stats* stats_out);

/* Aligns an explicit host pair list: pairs[2q] = si (row sequence, the
 * reference's seq1), pairs[2q+1] = sj. Writes dist_out[q] (the float the
 * reference stores with SetAt) and, if not NULL, stats_out[q]. The same
 * persistent, length-ordered launches as a plan, enqueued directly on the
 * context's streams (no graph is built for a one-shot call). */
int cwgpu_align_pairs(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, float* dist_out,
                      cwgpu_pair_stats* stats_out);

/* The same computation with one kernel launch per pair (the plain GPU form
 * the batched form is measured against). Same outputs. */
int cwgpu_align_pairs_plain(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, float* dist_out,
                            cwgpu_pair_stats* stats_out);

/* ---- plans: the pair list resident on the device, one captured launch -------
 * A plan uploads a pair list and its load-balancing order (longest pairs
 * first) once, owns device output arrays and holds a CUDA graph of the
 * persistent launch, so repeated runs over resident inputs cost one
 * cudaGraphLaunch. Pairs whose first sequence has at most
 * cwgpu_tuning.short_rows residues (128 by default) run in a second
 * persistent kernel (4 rows per lane instead of 8) inside the same graph,
 * beside the long-pair kernel at lower priority. A plan is tied to the sequences, matrix and params that were
 * current when it was made: after cwgpu_upload_seqs/set_params/set_matrix,
 * cwgpu_plan_launch returns CWGPU_ERR_STATE. Plans of one context share its
 * scratch memory and must not run concurrently. No reference counterpart: the
 * reference re-reads its inputs for every call. */
typedef struct cwgpu_plan cwgpu_plan;
int cwgpu_plan_create(cwgpu_context* ctx, const int32_t* pairs, int64_t npairs, cwgpu_plan** out);
/* Enqueues the plan's graph on `stream` (a cudaStream_t; NULL = the context's
 * own stream) and returns without waiting. */
int cwgpu_plan_launch(cwgpu_plan* plan, void* stream);
/* Waits for the device, then copies distances (and stats if not NULL) out. */
int cwgpu_plan_results(cwgpu_plan* plan, float* dist_out, cwgpu_pair_stats* stats_out);
/* Device address of the plan's float distance array (npairs entries). */
void* cwgpu_plan_device_dist(cwgpu_plan* plan);
/* Waits, then returns the algorithmic cell updates of the plan's last run:
 * counts[0] forwardPass (n*m), counts[1] reversePass iterations up to its break
 * (:351-414), counts[2] diff() inner-loop iterations (:450-566). These are the
 * iteration counts the reference itself executes for the same pairs. */
int cwgpu_plan_cell_counts(cwgpu_plan* plan, int64_t* counts);
/* Kernels one cwgpu_plan_launch runs (0, 1 or 2: long-pair and short-pair). */
int cwgpu_plan_kernel_count(const cwgpu_plan* plan);
/* 1 if the plan's long pairs run one CTA per pair (cwgpu_cta_tuning), 0 if
 * one warp per pair. */
int cwgpu_plan_pair_ctas(const cwgpu_plan* plan);
void cwgpu_plan_destroy(cwgpu_plan* plan);

/* ---- allocation-free variant ---------------------------------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc:
 * code inside a host framework that owns all device memory through its own
 * pool, or a process whose device-memory budget is fixed at start-up. The
 * caller passes device buffers it already owns; this call allocates nothing
 * and uses one static device array of CWGPU_NOALLOC_SCRATCH_BYTES (16 MiB,
 * held by every GPU that loads the library until the process exits) for all
 * its working memory. Limit: sequences up to CWGPU_NOALLOC_MAX_LEN residues
 * (longer max_len is rejected with CWGPU_ERR_ARG). All d_* pointers are device
 * memory: codes/offsets/lens as for cwgpu_upload_seqs, d_matrix the 32x32
 * int32 matrix, d_pairs 2*npairs int32, outputs d_dist (npairs floats) and
 * d_stats (nullable). The first call on a device looks up the array's device
 * address. The call waits for its kernel on `stream` (a cudaStream_t, NULL =
 * legacy default) and returns
 * CWGPU_ERR_ARG if the device-side checks rejected an input (pair index,
 * negative sequence offset, length above max_len, residue code outside
 * [0, 31]), CWGPU_ERR_MATRIX if a d_matrix entry is outside int16 (nothing is
 * aligned then), CWGPU_ERR_DEVICE if a pair reached the Myers-Miller stack
 * limit. Calls share the array: calls whose GPU work overlaps race, so callers
 * serialise them (one stream, or calls that do not overlap). */
#define CWGPU_NOALLOC_MAX_LEN 8191
#define CWGPU_NOALLOC_SCRATCH_BYTES (16u << 20)
int cwgpu_align_pairs_noalloc(const int8_t* d_codes, const int64_t* d_offsets, const int32_t* d_lens,
                              int32_t nseqs, int32_t max_len, const int32_t* d_matrix,
                              const cwgpu_params* params, const int32_t* d_pairs, int64_t npairs,
                              float* d_dist, cwgpu_pair_stats* d_stats, void* stream);

/* Tuning knobs of the kernel (no reference counterpart; results do not depend
 * on them). Myers-Miller frames with M <= tiny_m rows and N <= tiny_n columns
 * (tiny_n <= 16, tiny_m <= 256) are solved one frame per lane instead of by a
 * warp-wide sweep. Pairs whose first sequence has at most short_rows residues
 * (0..65535; default 128, 0 = none) run in the short-pair kernel (4 rows per
 * lane) instead of the long-pair one (8 rows per lane). The autotuner in
 * clustalw_gb300/autotune.py picks all three. */
typedef struct cwgpu_tuning {
    int32_t tiny_m;
    int32_t tiny_n;
    int32_t short_rows;
} cwgpu_tuning;
int cwgpu_set_tuning(cwgpu_context* ctx, const cwgpu_tuning* tuning);
int cwgpu_get_tuning(const cwgpu_context* ctx, cwgpu_tuning* tuning);

/* One CTA per pair (no reference counterpart; results do not depend on it).
 * A launch with at most max_pairs long pairs (first sequence longer than
 * short_rows) runs them one CTA of `warps` warps (2, 4, 8 or 16) per pair
 * instead of one warp per pair: the warps share the pair's forwardPass and
 * reversePass stripes and every Myers-Miller frame of at least large_rows
 * rows (two such frames at once on half the CTA each when two are waiting);
 * smaller frames go to a stack in shared memory from which the warps take
 * frames and to which they give back the children they make. Defaults:
 * max_pairs -1 (a quarter of the long-pair kernel's resident warps, 760 on a
 * GB300), warps 0 (16, 8 or 4 as the launch has at most 0.5, 2.5 or more pairs
 * per SM), large_rows 0 (per pair, the larger of 512 and a third of the rows
 * of its diff() box: the top two levels of the recursion); max_pairs 0 turns
 * it off. The reference's own GPU form also
 * runs one CTA per pair (G/cuda/cudaFullPairwiseAlign.cu:369-468), as one
 * 32-thread wavefront. A hand-over wait between the warps that ran out its
 * bound ends the call with CWGPU_ERR_TIMEOUT. */
typedef struct cwgpu_cta_tuning {
    int32_t max_pairs;
    int32_t warps;
    int32_t large_rows;
} cwgpu_cta_tuning;
int cwgpu_set_cta_tuning(cwgpu_context* ctx, const cwgpu_cta_tuning* tuning);
int cwgpu_get_cta_tuning(const cwgpu_context* ctx, cwgpu_cta_tuning* tuning);
/* Diagnostic: runs the CTA form's hand-over wait on a progress word that
 * nothing raises, limited to timeout_ns (1 .. 4e9). *timed_out is 1 when the
 * wait ended at its limit with the timeout status, as every such wait must;
 * the context stays usable. No GPU fault or hang is involved. */
int cwgpu_cta_wait_probe(cwgpu_context* ctx, int64_t timeout_ns, int32_t* timed_out);

/* ---- serving: continuous batching of independent jobs -----------------------
 * No counterpart in the reference (which aligns one sequence set per call).
 * A server owns one device, one scoring scheme (the matrix and params of
 * cwgpu_set_matrix/cwgpu_set_params) and a device-memory budget. Submitted
 * jobs (sequence sets; each job's result is what cwgpu_align_pairs returns
 * for all of its pairs in the reference's loop order) are admitted in arrival
 * order as job slots and budget memory free up; their sequences and distances
 * stay resident until released. A scheduler thread runs rounds: one persistent
 * launch over pairs mixed from every admitted job, two rounds in flight, so
 * jobs that arrive while others run join the next round. */
enum { CWGPU_JOB_QUEUED = 0, CWGPU_JOB_RUNNING = 1, CWGPU_JOB_DONE = 2, CWGPU_JOB_FAILED = 3 };
typedef struct cwgpu_server_opts {
    int64_t memory_budget_bytes; /* arena for resident job data and results */
    int32_t max_jobs;            /* job slots */
    int32_t max_seq_len;         /* longest sequence a job may hold */
    double round_cells;          /* sum of n*m per round (work granularity) */
    int64_t max_items_per_round; /* pairs per round */
    int32_t policy;              /* order jobs fill a round in: CWGPU_SERVE_FIFO or CWGPU_SERVE_SRPT */
    int32_t srpt_age_ms;         /* with CWGPU_SERVE_SRPT: jobs submitted longer ago go first (0: no cap) */
} cwgpu_server_opts;
/* CWGPU_SERVE_FIFO: admission order (the default; best p99 on the mixes
 * measured). CWGPU_SERVE_SRPT: the job with the least remaining work first,
 * except that jobs older than srpt_age_ms come first, in admission order
 * (without the cap: about a third of the p50 and a lower mean, a higher
 * p99; with a cap of a few hundred ms most of the p50 gain at a p99 close
 * to FIFO's). Results never depend on the policy. */
enum { CWGPU_SERVE_FIFO = 0, CWGPU_SERVE_SRPT = 1 };
typedef struct cwgpu_server_stats {
    int64_t jobs_queued, jobs_running, jobs_done;
    int64_t rounds, pairs;
    int64_t bytes_in_use;
    int64_t cells[3]; /* forward, reverse, diff cell updates so far */
} cwgpu_server_stats;
typedef struct cwgpu_server cwgpu_server;
int cwgpu_server_create(int device, const int32_t* matrix, const cwgpu_params* params,
                        const cwgpu_server_opts* opts, cwgpu_server** out);
/* Stops admitting, finishes admitted jobs, frees everything. */
void cwgpu_server_destroy(cwgpu_server* server);
/* Copies the job's sequences (same layout as cwgpu_upload_seqs) and queues
 * it. CWGPU_ERR_OOM if the job can never fit the budget. */
int cwgpu_server_submit(cwgpu_server* server, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                        const int32_t* lens, int32_t want_stats, int64_t* job_id);
int cwgpu_server_poll(cwgpu_server* server, int64_t job_id, int32_t* state);
/* Blocks until the job is done (timeout_ms < 0: no limit; else
 * CWGPU_ERR_TIMEOUT when it runs out). */
int cwgpu_server_wait(cwgpu_server* server, int64_t job_id, int32_t timeout_ms);
/* Distances (N(N-1)/2, loop order), stats (if submitted with want_stats) and
 * times[4] = submit, admit, first round, done (seconds, steady clock). */
int cwgpu_server_result(cwgpu_server* server, int64_t job_id, float* dist_out, cwgpu_pair_stats* stats_out,
                        double* times);
/* Frees the job's device memory and slot. */
int cwgpu_server_release(cwgpu_server* server, int64_t job_id);
int cwgpu_server_query(cwgpu_server* server, cwgpu_server_stats* out);

/* ---- quick k-tuple distances --------------------------------------------- */

/* The userParameters values FastPairwiseAlign::pairAlign reads
 * (FastPairwiseAlign.cpp:176-183), after setProtParams/setDNAParams. Reference
 * defaults (UserParameters.cpp:86-94, 133): protein ktup 1, window 5,
 * window_gap 3, signif 5; DNA ktup 2, window 4, window_gap 5, signif 4;
 * percent 1; max_aa 24. max_aln_length is Alignment::getMaxAlnLength() (0:
 * twice the longest sequence of the context, what the reference computes). */
typedef struct cwgpu_fast_params {
    int32_t dna, ktup, window, window_gap, signif, percent, max_aa;
    int32_t max_aln_length;
} cwgpu_fast_params;

/* Per pair: the best fragment's score, fragments made, and whether the
 * reference's "(Partial alignment)" cut-off was hit (FastPairwiseAlign.cpp:273-278). */
typedef struct cwgpu_fast_stats {
    int32_t score, frags, partial, pad;
} cwgpu_fast_stats;

/* The drop-in for FastPairwiseAlign::pairwiseAlign(alignPtr, distMat, iStart,
 * iEnd, jStart, jEnd) (CPU/clustalw-2.0.11/src/pairwise/FastPairwiseAlign.cpp:20-139)
 * over the sequences of cwgpu_upload_seqs: every pair of its loops
 * (i = iStart+1..iEnd, j = max(jStart+2, i+1)..jEnd, 1-based, held inside the
 * set) gets (100 - calcScore) / 100 in double at getIndex(i, j). The same size
 * and range checks as cwgpu_pairwise_align. Sequences up to 8191 residues. */
int cwgpu_fast_pairwise_align(cwgpu_context* ctx, const cwgpu_fast_params* params, int32_t i_start,
                              int32_t i_end, int32_t j_start, int32_t j_end, double* elements, int32_t dist_size,
                              cwgpu_fast_stats* stats_out);
/* Pair-list form: dist_out[q] for pairs[q] = (si, sj), 0-based. */
int cwgpu_fast_align_pairs(cwgpu_context* ctx, const cwgpu_fast_params* params, const int32_t* pairs,
                           int64_t npairs, double* dist_out, cwgpu_fast_stats* stats_out);
/* Device-resident form: device pair list, optional device processing order
 * (indices into the pair list, e.g. longest first; NULL: list order), device
 * outputs; asynchronous on `stream` (a cudaStream_t; NULL: the context's). */
int cwgpu_fast_align_pairs_device(cwgpu_context* ctx, const cwgpu_fast_params* params, const int32_t* d_pairs,
                                  const int32_t* d_order, int64_t npairs, double* d_dist,
                                  cwgpu_fast_stats* d_stats, void* stream);

/* Waits for all work of the context and reports a kernel-side error flag. */
int cwgpu_synchronize(cwgpu_context* ctx);

#ifdef __cplusplus
}
#endif
#endif /* CWGPU_H */
