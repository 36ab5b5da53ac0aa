// Prints the row blocks cwgpu::for_range_blocks makes, for the range cases on
// standard input (one "n i_start i_end j_start j_end max_pairs" per line):
// per case a line "case", then per block "block first npairs" and its pairs
// as "si sj ..." on one line. tests/test_range_blocks.py compares them with
// the reference's loop order.
#include <cstdio>

#include "cwgpu_ranges.h"

int main() {
    long long n, i0, i1, j0, j1, mx;
    while (std::scanf("%lld %lld %lld %lld %lld %lld", &n, &i0, &i1, &j0, &j1, &mx) == 6) {
        std::printf("case\n");
        cwgpu::for_range_blocks((int32_t)n, (int32_t)i0, (int32_t)i1, (int32_t)j0, (int32_t)j1, (int64_t)mx,
                                [](const int32_t* pairs, int64_t np, int64_t first) {
                                    std::printf("block %lld %lld\n", (long long)first, (long long)np);
                                    for (int64_t q = 0; q < 2 * np; ++q) std::printf("%d ", pairs[q]);
                                    std::printf("\n");
                                    return 0;
                                });
    }
    return 0;
}
