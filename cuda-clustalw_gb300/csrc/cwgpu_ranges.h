// cwgpu_ranges.h - the pair loops of the range calls (cwgpu_pairwise_align,
// cwgpu_fast_pairwise_align), cut into blocks of whole rows (not installed;
// plain C++, so tests/range_blocks_main.cpp builds it without CUDA).
#ifndef CWGPU_RANGES_H
#define CWGPU_RANGES_H

#include <algorithm>
#include <cstdint>
#include <vector>

namespace cwgpu {

// Pairs per call a range form hands to its pair-list call: whole rows up to
// this many, so that every list stays within CWGPU_MAX_PAIRS_PER_CALL and the
// host lists stay bounded whatever the set size.
constexpr int64_t kRangeBlockPairs = int64_t(1) << 28;

// Bounds of the reference's range loops (FullPairwiseAlign.cpp:97,110;
// FastPairwiseAlign.cpp:65-84, there 1-based): row si in
// [max(0, i_start), min(n, i_end)), column sj in [max(si + 1, j_start + 1),
// min(n, j_end)). Evaluated in 64 bits, so j_start = INT32_MAX selects no
// column instead of wrapping.
inline int64_t range_col_lo(int32_t si, int32_t j_start) {
    return std::max<int64_t>((int64_t)si + 1, (int64_t)j_start + 1);
}

// Calls f(pairs, npairs, first) on consecutive blocks of whole rows of those
// loops, in loop order. A block holds at most max_pairs pairs unless one row
// alone has more, in which case that row is a block of its own. `pairs` holds
// 0-based (si, sj); `first` is the loop-order index of the block's first
// pair. An empty range makes one call with npairs = 0 so that the callee's
// state checks still run. Returns the first non-zero status of f, else 0.
template <class F>
int for_range_blocks(int32_t n, int32_t i_start, int32_t i_end, int32_t j_start, int32_t j_end, int64_t max_pairs,
                     F&& f) {
    std::vector<int32_t> pairs;
    int64_t first = 0;
    const int64_t hi = std::min(n, j_end);
    const int32_t row_end = std::min(n, i_end);
    for (int32_t si = std::max<int32_t>(0, i_start); si < row_end; ++si) {
        const int64_t lo = range_col_lo(si, j_start);
        if (hi <= lo) continue;
        const int64_t have = (int64_t)(pairs.size() / 2);
        if (have > 0 && have + (hi - lo) > max_pairs) {
            const int rc = f(pairs.data(), have, first);
            if (rc) return rc;
            first += have;
            pairs.clear();
        }
        for (int64_t sj = lo; sj < hi; ++sj) {
            pairs.push_back(si);
            pairs.push_back((int32_t)sj);
        }
    }
    const int64_t have = (int64_t)(pairs.size() / 2);
    if (have > 0 || first == 0) return f(pairs.data(), have, first);
    return 0;
}

}  // namespace cwgpu

#endif  // CWGPU_RANGES_H
