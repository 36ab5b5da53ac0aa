// Host-only pieces of the library on the CPU, for tests/test_host_order.py.
// Reads commands on standard input:
//   key L                         -> "key <len_key(L)>"
//   order n short_rows np         then n lengths and 2*np pair indices
//                                 -> "nlong <k>" and the order on one line
//   layout n                      then n lengths, 32 remap entries and the
//                                 codes of all sequences back to back
//                                 -> "offs ..." and "bytes ..." on two lines
#ifndef __CUDACC__
#define __host__
#define __device__
#endif
#include <cstdio>
#include <cstring>
#include <vector>

#include "cwgpu_layout.h"
#include "cwgpu_order.h"

int main() {
    char cmd[16];
    while (std::scanf("%15s", cmd) == 1) {
        if (!std::strcmp(cmd, "key")) {
            int L;
            if (std::scanf("%d", &L) != 1) return 1;
            std::printf("key %d\n", cwgpu::len_key(L));
        } else if (!std::strcmp(cmd, "order")) {
            int n, short_rows;
            long long np;
            if (std::scanf("%d %d %lld", &n, &short_rows, &np) != 3) return 1;
            std::vector<int32_t> lens(n), pairs(2 * np), order(np);
            std::vector<uint16_t> lk(n);
            for (int s = 0; s < n; ++s) {
                if (std::scanf("%d", &lens[s]) != 1) return 1;
                lk[s] = (uint16_t)cwgpu::len_key(lens[s]);
            }
            for (long long q = 0; q < 2 * np; ++q)
                if (std::scanf("%d", &pairs[q]) != 1) return 1;
            int64_t nlong = -1;
            cwgpu::work_order(lens.data(), lk.data(), short_rows, pairs.data(), np, order.data(), &nlong);
            std::printf("nlong %lld\n", (long long)nlong);
            for (long long q = 0; q < np; ++q) std::printf("%d ", order[q]);
            std::printf("\n");
        } else if (!std::strcmp(cmd, "layout")) {
            int n;
            if (std::scanf("%d", &n) != 1) return 1;
            std::vector<int32_t> lens(n);
            std::vector<int64_t> start(n + 1, 0);
            for (int s = 0; s < n; ++s) {
                if (std::scanf("%d", &lens[s]) != 1) return 1;
                start[s + 1] = start[s] + lens[s];
            }
            int8_t remap[32];
            for (int c = 0; c < 32; ++c) {
                int v;
                if (std::scanf("%d", &v) != 1) return 1;
                remap[c] = (int8_t)v;
            }
            std::vector<int8_t> codes((size_t)start[n] + 1);
            for (int64_t i = 0; i < start[n]; ++i) {
                int v;
                if (std::scanf("%d", &v) != 1) return 1;
                codes[(size_t)i] = (int8_t)v;
            }
            std::vector<int8_t> out;
            std::vector<int64_t> offs;
            cwgpu::build_layout(
                n, lens.data(), [&](int s) { return lens[s] > 0 ? codes.data() + start[s] : nullptr; }, remap, out,
                offs);
            std::printf("offs");
            for (int s = 0; s < n; ++s) std::printf(" %lld", (long long)offs[s]);
            std::printf("\nbytes");
            for (size_t i = 0; i < out.size(); ++i) std::printf(" %d", out[i]);
            std::printf("\n");
        } else {
            return 2;
        }
    }
    return 0;
}
