// cwgpu_order.h - the order in which the persistent pair kernels take a
// call's pairs (shared by the translation units of the library; not
// installed; host code only).
//
// Pairs whose first sequence is longer than short_rows (the long-pair
// kernel's) come first, then the rest (the short-pair kernel's); each part is
// longest first by n*m, so the tail of each persistent queue holds its
// shortest work. The order only balances the load, so a stable counting sort
// on a coarse key does: len_key(n) + len_key(m), about 16 log2(n m), which
// grows with n and with m.
#ifndef CWGPU_ORDER_H
#define CWGPU_ORDER_H

#include <cstdint>
#include <vector>

namespace cwgpu {

// Sort key of a sequence length, like the exponent and top mantissa bits of a
// float: 16 * floor(log2 L) plus the 4 bits below the leading one (buckets
// 1/32 to 1/16 of L wide; 16 log2 L - 2.4 < key <= 16 log2 L), 0 for L = 0;
// below kLenKeys for L <= 65535.
constexpr int kLenKeys = 16 * 16;
inline int len_key(int L) {
    if (L <= 0) return 0;
    const int e = 31 - __builtin_clz((unsigned)L);
    const int m = e >= 4 ? (L >> (e - 4)) & 15 : (L << (4 - e)) & 15;
    return 16 * e + m;
}

// Writes the npairs pair indices to `order` and the number of long pairs to
// *nlong. lens[s] and lk[s] = len_key(lens[s]) for every sequence the pairs
// name (pairs already validated).
inline void work_order(const int32_t* lens, const uint16_t* lk, int short_rows, const int32_t* pairs,
                       int64_t npairs, int32_t* order, int64_t* nlong) {
    constexpr int kPairKeys = 2 * (kLenKeys - 1) + 1;  // len_key(n) + len_key(m)
    constexpr int kBuckets = 2 * kPairKeys;            // long pairs' keys first
    std::vector<uint16_t> key((size_t)npairs);
    int64_t start[kBuckets + 1] = {0};
    int64_t nl = 0;
    for (int64_t q = 0; q < npairs; ++q) {
        const int a = pairs[2 * q], b = pairs[2 * q + 1];
        const bool is_short = lens[a] <= short_rows;
        const int k = (is_short ? kPairKeys : 0) + (kPairKeys - 1 - lk[a] - lk[b]);
        key[(size_t)q] = (uint16_t)k;
        ++start[k + 1];
        nl += !is_short;
    }
    *nlong = nl;
    for (int k = 1; k <= kBuckets; ++k) start[k] += start[k - 1];
    for (int64_t q = 0; q < npairs; ++q) order[start[key[(size_t)q]]++] = (int32_t)q;
}

}  // namespace cwgpu

#endif  // CWGPU_ORDER_H
