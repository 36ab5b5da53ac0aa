// cwgpu_context.h - the context behind the opaque cwgpu_context handle of
// cwgpu.h, shared by the translation units of the library (not installed).
#ifndef CWGPU_CONTEXT_H
#define CWGPU_CONTEXT_H

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "cwgpu.h"
#include "cwgpu_order.h"

struct cwgpu_fast_state;
// Frees the quick-distance tables of a context (cwgpu_fast.cu).
void cwgpu_fast_release(cwgpu_context* ctx);
// Copies inputs changed on the host since the last call into the context's
// device arena (one asynchronous copy on ctx->stream); cwgpu.cu.
int cwgpu_stage_inputs(cwgpu_context* ctx);

// The pair kernels for other callers of the library (the serving engine):
// persistent grids of the long-pair and short-pair kernels for K codes, and
// the launch a plan makes over one ordered pair list (gl: its long pairs, on
// s; gs: its short pairs, on s2 forked from s and joined back; counters of gl
// reset first, gs.counter = gl.counter + 4). cwgpu.cu.
namespace cwgpu {
struct PairArgs;
}
cudaError_t cwgpu_pair_kernel_grids(int K, int sm_count, int* grid, int* grid_short);
int cwgpu_pair_kernel_warps_per_cta();
cudaError_t cwgpu_enqueue_pair_kernels(const cwgpu::PairArgs& gl, const cwgpu::PairArgs& gs, int grid,
                                       int grid_short, int prio_high, int prio_low, cudaStream_t s, cudaStream_t s2,
                                       cudaEvent_t fork, cudaEvent_t join);

struct cwgpu_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool has_matrix = false, has_params = false, has_seqs = false;
    int32_t matrix[CWGPU_NUMRES * CWGPU_NUMRES];
    cwgpu_params params;
    int nseqs = 0;
    int lmax = 0;
    std::vector<int32_t> lens;
    std::vector<uint16_t> len_key;  // cwgpu::len_key of each length (the work order's key)
    std::vector<int64_t> offs;
    std::vector<int8_t> host_codes;  // original codes, for nres and the remap
    uint32_t codes_present = 0;      // bit c: code c occurs in some sequence
    int K = 0;                       // codes present in the sequences
    int dense_of[CWGPU_NUMRES];      // original code -> dense index, -1 if absent
    int code_of[CWGPU_NUMRES];       // dense index -> original code
    int tiny_m = 32, tiny_n = 16;    // Myers-Miller frames solved one per lane
    int short_rows = 128;            // pairs with a first sequence this short: short-pair kernel
    // One CTA per pair (k_pairwise_cta) for launches of at most cta_pairs long
    // pairs (-1: a quarter of the long-pair kernel's warps): cta_warps warps
    // per CTA (0: chosen by pairs per SM), Myers-Miller frames of at least
    // cta_large_rows rows divided by the whole CTA (0: per pair, the larger of
    // 512 and a third of its diff() box).
    int cta_pairs = -1, cta_warps = 0, cta_large_rows = 0;
    int grid_cta[5] = {0, 0, 0, 0, 0};  // CTAs of k_pairwise_cta that fit at once, by log2(warps), for grid_K
    // Inputs on the device: one arena, filled by one copy from one pinned
    // staging buffer whenever the host-side inputs changed (cwgpu_stage_inputs).
    // The pointers below point into it.
    unsigned char* d_in = nullptr;
    size_t cap_in = 0;
    unsigned char* h_in = nullptr;  // pinned staging of the arena
    size_t cap_h_in = 0;
    cudaEvent_t ev_in = nullptr;    // recorded after the last staging copy
    bool in_dirty = true;
    std::vector<int8_t> host_layout;  // d_codes as built on the host
    std::vector<int64_t> host_poffs;
    std::vector<int32_t> host_go;     // gap open by length 0..: valid for go_params
    cwgpu_params go_params;
    int8_t* d_codes = nullptr;   // pair kernels' layout (cwgpu_layout.h): guards, forward and reversed copies
    int64_t* d_poffs = nullptr;  // forward copy of each sequence in d_codes
    int64_t* d_offs = nullptr;   // each sequence in host_codes (the quick path's upload of it)
    int32_t* d_lens = nullptr;
    int32_t* d_nres = nullptr;   // set once params are
    int32_t* d_matrix = nullptr; // set once the matrix is
    int32_t* d_go = nullptr;     // set once params are
    int go_len = 0;
    int2* d_scratch = nullptr;
    size_t scratch_bytes = 0;
    unsigned long long* d_counter = nullptr;  // [0] queue head, [1..3] cell counts, [4] short-pair queue head
    int* d_err = nullptr;
    int grid = 0;        // persistent CTAs of the long-pair kernel
    int grid_short = 0;  // and of the short-pair kernel
    int grid_K = -1;  // K the grid size was computed for
    unsigned generation = 0;  // bumped whenever device inputs or scratch move
    std::string last_error;
    cwgpu_fast_state* fast = nullptr;  // quick-distance tables (cwgpu_fast.cu), built on first use
    // One-shot cwgpu_align_pairs: pinned staging of the pair list in and the
    // distances, statistics and status word out.
    unsigned char* h_io = nullptr;
    size_t cap_h_io = 0;
    // One-shot cwgpu_align_pairs: grow-only pair arrays and the second stream
    // the short-pair kernel runs on beside the long-pair one.
    unsigned char* d_call = nullptr;  // pair list, order, queue counters, status word, distances, stats
    size_t cap_call = 0;
    cudaStream_t stream_short = nullptr;
    int prio_low = 0, prio_high = 0;  // stream priority range of the device
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

#endif  // CWGPU_CONTEXT_H
