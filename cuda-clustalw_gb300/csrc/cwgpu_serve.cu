// Serving engine: continuous batching of independent alignment jobs.
//
// Each job is one call's worth of work in the reference: a sequence set whose
// N(N-1)/2 pairs FullPairwiseAlign::pairwiseAlign would align
// (CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.cpp:97-190). A server
// owns one device, one scoring scheme (matrix + params) and a device-memory
// budget. A scheduler thread:
//   1. admits queued jobs in arrival order while a job slot and budget memory
//      are free, uploading the job's residues, lengths, residue counts and
//      gap-open table into the budget arena, where they stay until the job is
//      released (results stay in the arena until then too);
//   2. forms rounds: a work list of (job, si, sj) items taken from every
//      admitted job in admission order, longest jobs first within the round,
//      up to a cell budget per round;
//   3. runs each round as a plan runs a pair list: the round's pairs, longest
//      first, over a round-local table of the sequences of its jobs, in the
//      same persistent kernels as cwgpu_align_pairs (k_pairwise, 8 rows per
//      lane; pairs whose first sequence has at most 128 residues in the 4-row
//      kernel beside it), then a scatter of the round's distances to the jobs'
//      result arrays; two rounds are in flight on two streams (each with its
//      own buffers and scratch rows), so a round starts filling SMs while the
//      previous one drains, and jobs that arrive while a round runs join the
//      next one;
//   4. credits finished pairs to their jobs; a job whose pairs are all done
//      has its distances copied to host memory and is marked done.
// Results do not depend on the mix: every pair runs the same kernels as
// cwgpu_align_pairs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "cwgpu.h"
#include "cwgpu_context.h"
#include "cwgpu_device.cuh"
#include "cwgpu_layout.h"

namespace {

constexpr int kShortRows = 128;  // pairs whose first sequence is this short: the 4-row kernel

// A job's block in the budget arena.
struct JobDesc {
    const int8_t* codes;  // the job's residues in the pair kernels' layout (cwgpu_layout.h)
    float* dist;
    cwgpu_pair_stats* stats;
};

// Where a round's pair k goes: job slot and pair index q within the job.
struct WorkItem {
    int32_t slot, q;
};

// Round-local results to the jobs' arrays.
__global__ void k_scatter(const WorkItem* items, long long n, const JobDesc* jobs, const float* dist,
                          const cwgpu_pair_stats* stats) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const WorkItem it = items[k];
        const JobDesc J = jobs[it.slot];
        J.dist[it.q] = dist[k];
        if (J.stats && stats) J.stats[it.q] = stats[k];
    }
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over the budget arena (offsets, 256-byte granules).
class Arena {
   public:
    void reset(size_t size) {
        free_.clear();
        free_[0] = size;
        used_ = 0;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

   private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0;
};

struct Job {
    int64_t id = 0;
    int state = CWGPU_JOB_QUEUED;
    int status = CWGPU_OK;
    int nseqs = 0;
    int want_stats = 0;
    int64_t npairs = 0;
    int lmax = 0;
    std::vector<int8_t> codes;  // dense codes in the pair kernels' layout (cwgpu_layout.h)
    std::vector<int64_t> offs;
    std::vector<int32_t> lens, nres;
    int64_t cells_nm = 0;
    // placement
    int slot = -1;
    size_t arena_off = 0, arena_bytes = 0;
    JobDesc desc;
    // progress
    int32_t next_si = 0, next_sj = 1;
    int64_t scheduled = 0, done = 0;
    // results
    std::vector<float> dist;
    std::vector<cwgpu_pair_stats> stats;
    double t_submit = 0, t_admit = 0, t_start = 0, t_done = 0;
};

// One round in flight: its pair list, sequence table and results, built on the
// host in a pinned buffer and copied to the device in one piece.
struct Round {
    std::vector<std::pair<int, int64_t>> credit;  // (slot, pairs)
    cudaEvent_t ev = nullptr, fork = nullptr, join = nullptr;
    cudaStream_t s2 = nullptr;  // the short-pair kernel beside the long-pair one
    bool busy = false;
    int64_t items = 0;
    unsigned char* h = nullptr;  // pinned
    size_t cap_h = 0;
    unsigned char* d = nullptr;
    size_t cap_d = 0;
    int64_t n = 0, nlong = 0, nseq = 0;
    bool stats = false;
    // byte offsets: pairs at 0, then order, items, sequence offsets, lengths,
    // residue counts (copied), then distances and statistics (device only)
    size_t o_order = 0, o_items = 0, o_soffs = 0, o_slens = 0, o_snres = 0, bytes_in = 0, o_dist = 0, o_stats = 0,
           bytes_all = 0;
};

}  // namespace

struct cwgpu_server {
    int device = 0;
    int sm_count = 0;
    cwgpu_server_opts opts;
    cwgpu_params params;
    int32_t matrix[CWGPU_NUMRES * CWGPU_NUMRES];
    int ge = 0;
    // incremental dense alphabet shared by all jobs of the server
    int K = 0;
    int dense_of[CWGPU_NUMRES];
    int code_of[CWGPU_NUMRES];
    bool matrix_dirty = true;
    // device
    unsigned char* arena = nullptr;
    JobDesc* d_jobs = nullptr;
    int32_t* d_matrix = nullptr;
    int* d_err = nullptr;
    cudaStream_t streams[2] = {nullptr, nullptr};
    cudaStream_t upload = nullptr;  // job uploads, waited for before the job's first round
    unsigned long long* d_counter[2] = {nullptr, nullptr};
    int2* d_scratch[2] = {nullptr, nullptr};
    int32_t* d_go = nullptr;  // gap-open penalty by min(n, m), 0..max_seq_len
    int grid = 0, grid_short = 0, grid_K = -1;
    int prio_low = 0, prio_high = 0;
    Round rounds[2];
    int next_round = 0;
    Arena alloc;
    // host state
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job*> pending;
    std::vector<Job*> admitted;  // admission order
    std::map<int64_t, Job*> jobs;
    std::vector<int> free_slots;
    int64_t next_id = 1;
    bool stop = false;
    int fatal = CWGPU_OK;
    std::string error;
    std::thread worker;
    // statistics
    int64_t total_rounds = 0, total_items = 0, jobs_done = 0;
    unsigned long long cells[3] = {0, 0, 0};
};

namespace {

int srv_fail(cwgpu_server* s, int code, const std::string& m) {
    s->error = m;
    return code;
}

// Appends codes that occur in the job to the server alphabet (indices never
// move, so jobs already on the device keep their codes) and remaps the job.
void remap_job(cwgpu_server* s, Job* j, const int8_t* codes, const int64_t* offsets) {
    for (int q = 0; q < j->nseqs; ++q)
        for (int i = 0; i < j->lens[q]; ++i) {
            const int c = codes[offsets[q] + i];
            if (s->dense_of[c] < 0) {
                s->dense_of[c] = s->K;
                s->code_of[s->K++] = c;
                s->matrix_dirty = true;
            }
        }
    int8_t remap[CWGPU_NUMRES];
    for (int c = 0; c < CWGPU_NUMRES; ++c) remap[c] = (int8_t)s->dense_of[c];
    cwgpu::build_layout(
        j->nseqs, j->lens.data(), [&](int q) { return j->lens[q] > 0 ? codes + offsets[q] : nullptr; }, remap,
        j->codes, j->offs);
    j->nres.resize(j->nseqs);
    for (int q = 0; q < j->nseqs; ++q) {
        int r = 0;
        for (int i = 0; i < j->lens[q]; ++i) {
            const int c = codes[offsets[q] + i];
            r += (c != s->params.gap_pos1 && c != s->params.gap_pos2);
        }
        j->nres[q] = r;
    }
}

size_t job_bytes(const Job* j) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t b = up(j->codes.size()) + up(4 * (size_t)std::max<int64_t>(j->npairs, 1));
    if (j->want_stats) b += up(sizeof(cwgpu_pair_stats) * (size_t)std::max<int64_t>(j->npairs, 1));
    return b;
}

// Upload a job into its arena block on the upload stream and wait for it, so
// every round launched afterwards sees the job's data.
int place_job(cwgpu_server* s, Job* j) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    unsigned char* base = s->arena + j->arena_off;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + o;
        o += up(bytes);
        return p;
    };
    int8_t* codes = (int8_t*)take(j->codes.size());
    float* dist = (float*)take(4 * (size_t)std::max<int64_t>(j->npairs, 1));
    cwgpu_pair_stats* stats = j->want_stats ? (cwgpu_pair_stats*)take(sizeof(cwgpu_pair_stats) * j->npairs) : nullptr;
    cudaStream_t st = s->upload;
    cudaError_t e = cudaMemcpyAsync(codes, j->codes.data(), j->codes.size(), cudaMemcpyHostToDevice, st);
    j->desc = JobDesc{codes, dist, stats};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_jobs + j->slot, &j->desc, sizeof(JobDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return srv_fail(s, CWGPU_ERR_CUDA, std::string("job upload: ") + cudaGetErrorString(e));
    return CWGPU_OK;
}

void finish_job(cwgpu_server* s, Job* j) {
    j->dist.resize((size_t)j->npairs);
    cudaError_t e = cudaSuccess;
    if (j->npairs > 0) {
        e = cudaMemcpy(j->dist.data(), j->desc.dist, 4 * (size_t)j->npairs, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && j->want_stats) {
            j->stats.resize((size_t)j->npairs);
            e = cudaMemcpy(j->stats.data(), j->desc.stats, sizeof(cwgpu_pair_stats) * j->npairs,
                           cudaMemcpyDeviceToHost);
        }
    }
    j->status = (e == cudaSuccess) ? CWGPU_OK : CWGPU_ERR_CUDA;
    j->state = (e == cudaSuccess) ? CWGPU_JOB_DONE : CWGPU_JOB_FAILED;
    j->t_done = now_s();
    s->jobs_done++;
}

cudaError_t grow_dev(unsigned char*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMalloc(&p, need);
    if (e == cudaSuccess) cap = need;
    return e;
}

cudaError_t grow_pinned(unsigned char*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMallocHost(&p, need);
    if (e == cudaSuccess) cap = need;
    return e;
}

// The pairs of one round, taken from the admitted jobs in admission order (or
// least remaining work first), up to the round's cell budget: a table of the
// sequences of the round's jobs (offsets into the arena, lengths, residue
// counts), the pairs as indices into it, where each result goes, and the work
// order (long pairs first, then short ones, each longest first by n*m, as a
// plan orders them). Returns the number of pairs, 0 on none, -1 on an error.
int64_t build_round(cwgpu_server* s, Round& r) {
    r.credit.clear();
    std::vector<Job*> order;
    for (Job* j : s->admitted)
        if (j->scheduled < j->npairs) order.push_back(j);
    if (s->opts.policy == CWGPU_SERVE_SRPT) {
        // Least remaining work first; jobs older than the age cap go first, in
        // admission order (the sort is stable).
        const double now = now_s(), cap = s->opts.srpt_age_ms > 0 ? 1e-3 * s->opts.srpt_age_ms : 1e300;
        auto remaining = [](const Job* j) {
            return (double)j->cells_nm * (double)(j->npairs - j->scheduled) / (double)std::max<int64_t>(j->npairs, 1);
        };
        std::stable_sort(order.begin(), order.end(), [&](const Job* a, const Job* b) {
            const bool oa = now - a->t_submit > cap, ob = now - b->t_submit > cap;
            if (oa != ob) return oa;
            return !oa && remaining(a) < remaining(b);
        });
    }
    struct Take {
        Job* j;
        int32_t si0, sj0;
        int64_t q0, count;
    };
    std::vector<Take> taken;
    double budget = s->opts.round_cells;
    int64_t n = 0, nseq = 0;
    bool stats = false;
    for (Job* j : order) {
        if (budget <= 0 || n >= s->opts.max_items_per_round) break;
        Take t{j, j->next_si, j->next_sj, j->scheduled, 0};
        const double per_pair = (double)j->cells_nm / std::max<int64_t>(j->npairs, 1);
        while (j->scheduled < j->npairs && n < s->opts.max_items_per_round && budget > 0) {
            ++n;
            ++t.count;
            ++j->scheduled;
            budget -= per_pair;
            if (++j->next_sj >= j->nseqs) {
                ++j->next_si;
                j->next_sj = j->next_si + 1;
            }
        }
        if (j->t_start == 0) j->t_start = now_s();
        r.credit.push_back({j->slot, t.count});
        taken.push_back(t);
        nseq += j->nseqs;
        stats |= j->want_stats != 0;
    }
    if (n == 0) return 0;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    r.o_order = up(8 * (size_t)n);
    r.o_items = r.o_order + up(4 * (size_t)n);
    r.o_soffs = r.o_items + up(sizeof(WorkItem) * (size_t)n);
    r.o_slens = r.o_soffs + up(8 * (size_t)nseq);
    r.o_snres = r.o_slens + up(4 * (size_t)nseq);
    r.bytes_in = r.o_snres + up(4 * (size_t)nseq);
    r.o_dist = r.bytes_in;
    r.o_stats = r.o_dist + up(4 * (size_t)n);
    r.bytes_all = r.o_stats + (stats ? sizeof(cwgpu_pair_stats) * (size_t)n : 0);
    if (grow_pinned(r.h, r.cap_h, r.bytes_in) != cudaSuccess || grow_dev(r.d, r.cap_d, r.bytes_all) != cudaSuccess)
        return -1;
    int32_t* pairs = reinterpret_cast<int32_t*>(r.h);
    int32_t* ord = reinterpret_cast<int32_t*>(r.h + r.o_order);
    WorkItem* items = reinterpret_cast<WorkItem*>(r.h + r.o_items);
    int64_t* soffs = reinterpret_cast<int64_t*>(r.h + r.o_soffs);
    int32_t* slens = reinterpret_cast<int32_t*>(r.h + r.o_slens);
    int32_t* snres = reinterpret_cast<int32_t*>(r.h + r.o_snres);
    // Sort keys as in a plan's work order: the top 12 bits of n*m as a float,
    // long pairs (first sequence longer than kShortRows) before short ones.
    constexpr int kKeyBits = 12, kBuckets = 1 << kKeyBits;
    std::vector<uint16_t> key((size_t)n);
    std::vector<int64_t> start(2 * kBuckets + 1, 0);
    int64_t k = 0, base = 0;
    for (const Take& t : taken) {
        const Job* j = t.j;
        const int64_t codes_off = (int64_t)(j->desc.codes - reinterpret_cast<const int8_t*>(s->arena));
        for (int i = 0; i < j->nseqs; ++i) {
            soffs[base + i] = codes_off + j->offs[i];
            slens[base + i] = j->lens[i];
            snres[base + i] = j->nres[i];
        }
        int32_t si = t.si0, sj = t.sj0;
        for (int64_t c = 0; c < t.count; ++c, ++k) {
            pairs[2 * k] = (int32_t)(base + si);
            pairs[2 * k + 1] = (int32_t)(base + sj);
            items[k] = WorkItem{j->slot, (int32_t)(t.q0 + c)};
            const float w = (float)((double)j->lens[si] * (double)j->lens[sj]);
            uint32_t bits;
            memcpy(&bits, &w, sizeof(bits));
            const int b = (j->lens[si] <= kShortRows ? kBuckets : 0) + (kBuckets - 1 - (int)(bits >> (31 - kKeyBits)));
            key[(size_t)k] = (uint16_t)b;
            ++start[b + 1];
            if (++sj >= j->nseqs) {
                ++si;
                sj = si + 1;
            }
        }
        base += j->nseqs;
    }
    for (int b = 0; b < 2 * kBuckets; ++b) start[b + 1] += start[b];
    r.nlong = start[kBuckets];
    for (int64_t q = 0; q < n; ++q) ord[start[key[(size_t)q]]++] = (int32_t)q;
    r.n = n;
    r.nseq = nseq;
    r.stats = stats;
    return n;
}

int launch_round(cwgpu_server* s, int ri, int64_t nitems) {
    Round& r = s->rounds[ri];
    cudaStream_t st = s->streams[ri];
    cudaError_t e = cudaSuccess;
    const int K = std::max(1, s->K);
    if (s->grid_K != K) {
        e = cwgpu_pair_kernel_grids(K, s->sm_count, &s->grid, &s->grid_short);
        // the scratch holds rows for 5 CTAs per SM of each kernel (their launch bound)
        s->grid = std::min(s->grid, 5 * s->sm_count);
        s->grid_short = std::min(s->grid_short, 5 * s->sm_count);
        s->grid_K = K;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.d, r.h, r.bytes_in, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const int wpc = cwgpu_pair_kernel_warps_per_cta();
        cwgpu::PairArgs gl;
        gl.codes = reinterpret_cast<const int8_t*>(s->arena);
        gl.offs = reinterpret_cast<const int64_t*>(r.d + r.o_soffs);
        gl.lens = reinterpret_cast<const int32_t*>(r.d + r.o_slens);
        gl.nres = reinterpret_cast<const int32_t*>(r.d + r.o_snres);
        gl.pairs = reinterpret_cast<const int32_t*>(r.d);
        gl.order = reinterpret_cast<const int32_t*>(r.d + r.o_order);
        gl.go_table = s->d_go;
        gl.matrix = s->d_matrix;
        gl.dist = reinterpret_cast<float*>(r.d + r.o_dist);
        gl.stats = r.stats ? reinterpret_cast<cwgpu_pair_stats*>(r.d + r.o_stats) : nullptr;
        gl.scratch = s->d_scratch[ri];
        gl.counter = s->d_counter[ri];
        gl.err = s->d_err;
        gl.cells = s->d_counter[ri] + 1;
        gl.npairs = r.nlong;
        gl.lmax = s->opts.max_seq_len;
        gl.ge = s->ge;
        const int gp1 = s->params.gap_pos1, gp2 = s->params.gap_pos2;
        gl.gp1 = (gp1 >= 0 && gp1 < CWGPU_NUMRES) ? s->dense_of[gp1] : -1;
        gl.gp2 = (gp2 >= 0 && gp2 < CWGPU_NUMRES) ? s->dense_of[gp2] : -1;
        gl.K = K;
        gl.tiny_m = 32;
        gl.tiny_n = cwgpu::kTinyMaxN;
        cwgpu::PairArgs gs = gl;
        gs.order = gl.order + r.nlong;
        gs.npairs = r.n - r.nlong;
        gs.counter = s->d_counter[ri] + 4;
        if (r.nlong > 0) gs.scratch += (size_t)5 * s->sm_count * wpc * 2 * (size_t)(s->opts.max_seq_len + 1);
        e = cwgpu_enqueue_pair_kernels(gl, gs, s->grid, s->grid_short, s->prio_high, s->prio_low, st, r.s2, r.fork,
                                       r.join);
    }
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<int64_t>((r.n + 255) / 256, 4 * (int64_t)s->sm_count);
        k_scatter<<<blocks, 256, 0, st>>>(reinterpret_cast<const WorkItem*>(r.d + r.o_items), r.n, s->d_jobs,
                                          reinterpret_cast<const float*>(r.d + r.o_dist),
                                          r.stats ? reinterpret_cast<const cwgpu_pair_stats*>(r.d + r.o_stats) : nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(r.ev, st);
    if (e != cudaSuccess) return srv_fail(s, CWGPU_ERR_CUDA, std::string("round launch: ") + cudaGetErrorString(e));
    r.busy = true;
    r.items = nitems;
    s->total_rounds++;
    s->total_items += nitems;
    return CWGPU_OK;
}

void upload_matrix(cwgpu_server* s) {
    std::vector<int32_t> dm(CWGPU_NUMRES * CWGPU_NUMRES, 0);
    for (int a = 0; a < s->K; ++a)
        for (int b = 0; b < s->K; ++b)
            dm[a * CWGPU_NUMRES + b] = s->matrix[s->code_of[a] * CWGPU_NUMRES + s->code_of[b]];
    // Both streams are idle here (no round in flight) or ordered by stream 0.
    cudaMemcpy(s->d_matrix, dm.data(), sizeof(int32_t) * dm.size(), cudaMemcpyHostToDevice);
    s->matrix_dirty = false;
}

void scheduler(cwgpu_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // 1. admission, in arrival order, while a slot and budget memory are free.
        while (!s->pending.empty() && !s->free_slots.empty()) {
            Job* j = s->pending.front();
            const size_t bytes = job_bytes(j);
            size_t off = 0;
            if (!s->alloc.alloc(bytes, &off)) break;  // wait for memory to free up
            s->pending.pop_front();
            j->slot = s->free_slots.back();
            s->free_slots.pop_back();
            j->arena_off = off;
            j->arena_bytes = bytes;
            const int rc = place_job(s, j);
            j->t_admit = now_s();
            if (rc) {
                j->state = CWGPU_JOB_FAILED;
                j->status = rc;
                s->cv.notify_all();
                continue;
            }
            j->state = CWGPU_JOB_RUNNING;
            if (j->npairs == 0) {
                finish_job(s, j);
                s->cv.notify_all();
                continue;
            }
            s->admitted.push_back(j);
        }
        // 2. keep two rounds in flight.
        bool launched = false;
        for (int tries = 0; tries < 2; ++tries) {
            const int ri = s->next_round;
            if (s->rounds[ri].busy) break;
            bool any = false;
            for (Job* j : s->admitted) any |= (j->scheduled < j->npairs);
            if (!any) break;
            if (s->matrix_dirty) {
                // Alphabet grew: wait for rounds in flight before changing the matrix.
                if (s->rounds[0].busy || s->rounds[1].busy) break;
                upload_matrix(s);
            }
            const int64_t n = build_round(s, s->rounds[ri]);
            if (n < 0) {
                s->fatal = CWGPU_ERR_OOM;
                s->error = "round buffers: allocation failed";
                break;
            }
            if (n == 0) break;
            if (launch_round(s, ri, n)) {
                s->fatal = CWGPU_ERR_CUDA;
                break;
            }
            s->next_round ^= 1;
            launched = true;
        }
        // 3. retire the oldest round in flight.
        const int old = s->next_round;  // rounds alternate, so the other one is the older
        int retire = -1;
        if (s->rounds[old].busy)
            retire = old;
        else if (s->rounds[old ^ 1].busy)
            retire = old ^ 1;
        if (retire >= 0) {
            Round& r = s->rounds[retire];
            lk.unlock();
            cudaError_t e = cudaEventSynchronize(r.ev);
            unsigned long long c[4];
            if (e == cudaSuccess) e = cudaMemcpy(c, s->d_counter[retire], sizeof(c), cudaMemcpyDeviceToHost);
            lk.lock();
            r.busy = false;
            if (e != cudaSuccess) {
                s->fatal = CWGPU_ERR_CUDA;
                s->error = std::string("round: ") + cudaGetErrorString(e);
            } else {
                for (int i = 0; i < 3; ++i) s->cells[i] += c[i + 1];
            }
            for (auto& cr : r.credit) {
                for (Job* j : s->admitted)
                    if (j->slot == cr.first) {
                        j->done += cr.second;
                        if (j->done == j->npairs) finish_job(s, j);
                        break;
                    }
            }
            s->admitted.erase(std::remove_if(s->admitted.begin(), s->admitted.end(),
                                             [](Job* j) { return j->state != CWGPU_JOB_RUNNING; }),
                              s->admitted.end());
            s->cv.notify_all();
            continue;
        }
        if (s->stop && s->pending.empty()) break;
        if (!launched) s->cv.wait_for(lk, std::chrono::milliseconds(50));
    }
}

}  // namespace

extern "C" {

int cwgpu_server_create(int device, const int32_t* matrix, const cwgpu_params* params, const cwgpu_server_opts* opts,
                        cwgpu_server** out) {
    if (!out || !matrix || !params || !opts) return CWGPU_ERR_ARG;
    *out = nullptr;
    if (opts->memory_budget_bytes <= 0 || opts->max_jobs <= 0 || opts->max_seq_len <= 0 ||
        opts->max_seq_len > CWGPU_MAX_SEQ_LEN || opts->round_cells <= 0 || opts->max_items_per_round <= 0 ||
        (opts->policy != CWGPU_SERVE_FIFO && opts->policy != CWGPU_SERVE_SRPT) || opts->srpt_age_ms < 0)
        return CWGPU_ERR_ARG;
    for (int i = 0; i < CWGPU_NUMRES * CWGPU_NUMRES; ++i)
        if (matrix[i] < -32768 || matrix[i] > 32767) return CWGPU_ERR_MATRIX;
    cwgpu_server* s = new (std::nothrow) cwgpu_server();
    if (!s) return CWGPU_ERR_OOM;
    s->device = device;
    s->opts = *opts;
    s->params = *params;
    memcpy(s->matrix, matrix, sizeof(s->matrix));
    for (int c = 0; c < CWGPU_NUMRES; ++c) s->dense_of[c] = -1;
    int32_t go = 0;
    cwgpu_gap_penalties(params, 1, 1, &go, &s->ge);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&s->arena, (size_t)opts->memory_budget_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_jobs, sizeof(JobDesc) * opts->max_jobs);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_matrix, sizeof(int32_t) * CWGPU_NUMRES * CWGPU_NUMRES);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&s->prio_low, &s->prio_high);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_go, sizeof(int32_t) * (size_t)(opts->max_seq_len + 1));
    if (e == cudaSuccess) {
        std::vector<int32_t> got((size_t)opts->max_seq_len + 1, 0);
        for (int L = 1; L <= opts->max_seq_len; ++L) {
            int32_t ge = 0;
            cwgpu_gap_penalties(params, L, L, &got[(size_t)L], &ge);
        }
        e = cudaMemcpy(s->d_go, got.data(), sizeof(int32_t) * got.size(), cudaMemcpyHostToDevice);
    }
    // Scratch rows per round: 5 CTAs per SM of each pair kernel (their launch bound).
    const size_t slots = (size_t)2 * 5 * s->sm_count * cwgpu_pair_kernel_warps_per_cta();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->rounds[i].s2, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_counter[i], 8 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&s->d_scratch[i], slots * 2 * (opts->max_seq_len + 1) * sizeof(int2));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->rounds[i].ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->rounds[i].fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->rounds[i].join, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        cwgpu_server_destroy(s);
        return e == cudaErrorMemoryAllocation ? CWGPU_ERR_OOM : CWGPU_ERR_CUDA;
    }
    s->alloc.reset((size_t)opts->memory_budget_bytes);
    for (int i = opts->max_jobs - 1; i >= 0; --i) s->free_slots.push_back(i);
    s->worker = std::thread(scheduler, s);
    *out = s;
    return CWGPU_OK;
}

void cwgpu_server_destroy(cwgpu_server* s) {
    if (!s) return;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            for (Job* j : s->pending) {
                j->state = CWGPU_JOB_FAILED;
                j->status = CWGPU_ERR_STATE;
            }
            s->pending.clear();
        }
        s->cv.notify_all();
        s->worker.join();
    }
    cudaSetDevice(s->device);
    for (int i = 0; i < 2; ++i) {
        if (s->streams[i]) cudaStreamSynchronize(s->streams[i]);
        Round& r = s->rounds[i];
        if (r.ev) cudaEventDestroy(r.ev);
        if (r.fork) cudaEventDestroy(r.fork);
        if (r.join) cudaEventDestroy(r.join);
        if (r.s2) cudaStreamDestroy(r.s2);
        if (r.h) cudaFreeHost(r.h);
        if (r.d) cudaFree(r.d);
        if (s->d_counter[i]) cudaFree(s->d_counter[i]);
        if (s->d_scratch[i]) cudaFree(s->d_scratch[i]);
        if (s->streams[i]) cudaStreamDestroy(s->streams[i]);
    }
    if (s->upload) cudaStreamDestroy(s->upload);
    if (s->arena) cudaFree(s->arena);
    if (s->d_jobs) cudaFree(s->d_jobs);
    if (s->d_matrix) cudaFree(s->d_matrix);
    if (s->d_go) cudaFree(s->d_go);
    if (s->d_err) cudaFree(s->d_err);
    for (auto& kv : s->jobs) delete kv.second;
    delete s;
}

int cwgpu_server_submit(cwgpu_server* s, int32_t nseqs, const int8_t* codes, const int64_t* offsets,
                        const int32_t* lens, int32_t want_stats, int64_t* job_id) {
    if (!s || !job_id || nseqs < 0 || (nseqs > 0 && (!offsets || !lens))) return CWGPU_ERR_ARG;
    Job* j = new (std::nothrow) Job();
    if (!j) return CWGPU_ERR_OOM;
    j->nseqs = nseqs;
    j->want_stats = want_stats ? 1 : 0;
    j->lens.assign(lens, lens + nseqs);
    for (int q = 0; q < nseqs; ++q) {
        if (lens[q] < 0 || lens[q] > s->opts.max_seq_len) {
            delete j;
            return srv_fail(s, CWGPU_ERR_ARG, "sequence longer than the server's max_seq_len");
        }
        if (lens[q] > 0 && (!codes || offsets[q] < 0)) {
            delete j;
            return CWGPU_ERR_ARG;
        }
        for (int i = 0; i < lens[q]; ++i)
            if (codes[offsets[q] + i] < 0 || codes[offsets[q] + i] >= CWGPU_NUMRES) {
                delete j;
                return srv_fail(s, CWGPU_ERR_ARG, "residue code outside [0, 31]");
            }
        j->lmax = std::max(j->lmax, (int)lens[q]);
    }
    j->npairs = (int64_t)nseqs * (nseqs - 1) / 2;
    if (j->npairs > CWGPU_MAX_PAIRS_PER_CALL) {  // work items carry 32-bit pair indices
        delete j;
        return srv_fail(s, CWGPU_ERR_ARG, "job has more than CWGPU_MAX_PAIRS_PER_CALL pairs");
    }
    int64_t before = 0;  // residues of the sequences before b
    for (int b = 0; b < nseqs; ++b) {
        j->cells_nm += before * lens[b];
        before += lens[b];
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal) {
        delete j;
        return s->fatal;
    }
    remap_job(s, j, codes, offsets);
    if (job_bytes(j) > (size_t)s->opts.memory_budget_bytes) {
        delete j;
        return srv_fail(s, CWGPU_ERR_OOM, "job larger than the server's memory budget");
    }
    j->id = s->next_id++;
    j->t_submit = now_s();
    s->jobs[j->id] = j;
    s->pending.push_back(j);
    *job_id = j->id;
    s->cv.notify_all();
    return CWGPU_OK;
}

int cwgpu_server_poll(cwgpu_server* s, int64_t job_id, int32_t* state) {
    if (!s || !state) return CWGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return CWGPU_ERR_NOT_FOUND;
    *state = it->second->state;
    return CWGPU_OK;
}

int cwgpu_server_wait(cwgpu_server* s, int64_t job_id, int32_t timeout_ms) {
    if (!s) return CWGPU_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return CWGPU_ERR_NOT_FOUND;
    Job* j = it->second;
    auto ready = [&] { return j->state == CWGPU_JOB_DONE || j->state == CWGPU_JOB_FAILED || s->fatal; };
    if (timeout_ms < 0)
        s->cv.wait(lk, ready);
    else if (!s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return CWGPU_ERR_TIMEOUT;
    if (j->state == CWGPU_JOB_FAILED) return j->status ? j->status : CWGPU_ERR_CUDA;
    if (s->fatal && j->state != CWGPU_JOB_DONE) return s->fatal;
    return CWGPU_OK;
}

int cwgpu_server_result(cwgpu_server* s, int64_t job_id, float* dist_out, cwgpu_pair_stats* stats_out,
                        double* times) {
    if (!s) return CWGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return CWGPU_ERR_NOT_FOUND;
    Job* j = it->second;
    if (j->state != CWGPU_JOB_DONE) return CWGPU_ERR_STATE;
    if (dist_out && j->npairs) memcpy(dist_out, j->dist.data(), 4 * (size_t)j->npairs);
    if (stats_out) {
        if (!j->want_stats) return CWGPU_ERR_STATE;
        if (j->npairs) memcpy(stats_out, j->stats.data(), sizeof(cwgpu_pair_stats) * j->npairs);
    }
    if (times) {
        times[0] = j->t_submit;
        times[1] = j->t_admit;
        times[2] = j->t_start;
        times[3] = j->t_done;
    }
    return CWGPU_OK;
}

int cwgpu_server_release(cwgpu_server* s, int64_t job_id) {
    if (!s) return CWGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return CWGPU_ERR_NOT_FOUND;
    Job* j = it->second;
    if (j->state == CWGPU_JOB_QUEUED || j->state == CWGPU_JOB_RUNNING) return CWGPU_ERR_STATE;
    if (j->slot >= 0) {
        s->alloc.release(j->arena_off, j->arena_bytes);
        s->free_slots.push_back(j->slot);
    }
    s->jobs.erase(it);
    delete j;
    s->cv.notify_all();  // memory freed: queued jobs may be admitted
    return CWGPU_OK;
}

int cwgpu_server_query(cwgpu_server* s, cwgpu_server_stats* out) {
    if (!s || !out) return CWGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    out->jobs_queued = (int64_t)s->pending.size();
    out->jobs_running = (int64_t)s->admitted.size();
    out->jobs_done = s->jobs_done;
    out->rounds = s->total_rounds;
    out->pairs = s->total_items;
    out->bytes_in_use = (int64_t)s->alloc.used();
    for (int i = 0; i < 3; ++i) out->cells[i] = (int64_t)s->cells[i];
    return s->fatal;
}

}  // extern "C"
