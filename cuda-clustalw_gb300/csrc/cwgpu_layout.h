// cwgpu_layout.h - device layout of the residue codes the pair kernels read
// (shared by the translation units of the library; not installed).
//
// [kGuard zero bytes]
// for every sequence s:
//   its len codes, zero-padded to a 16-byte boundary          (offset offs[s])
//   the same codes in reverse order, zero-padded likewise      (offs[s] + rev_offset(len))
// [kGuard zero bytes]
//
// The sweeps that run backwards over a sequence (reversePass, the reverse
// half of every Myers-Miller frame) read the reversed copy, so every sweep
// reads its residues in ascending address order; the guards let the lanes of a
// stripe's fill and drain steps read up to kGuard positions outside a copy
// without a bounds check (those residues are never used).
#ifndef CWGPU_LAYOUT_H
#define CWGPU_LAYOUT_H

#include <cstdint>
#include <cstring>
#include <vector>

namespace cwgpu {

constexpr int kGuard = 64;

__host__ __device__ inline long long rev_offset(int len) { return ((long long)len + 15) & ~15LL; }

// Lays out n sequences: sequence s is the lens[s] codes at row(s), each code c
// (in [0, 31]) stored as remap[c]. Fills `out` (the whole buffer) and `offs`
// (offset of each forward copy). The remap table is copied to a local array
// so that the byte stores of the layout cannot alias it.
template <class Row>
void build_layout(int n, const int32_t* lens, Row row, const int8_t* remap, std::vector<int8_t>& out,
                  std::vector<int64_t>& offs) {
    offs.resize((size_t)n);
    int64_t total = kGuard;
    for (int s = 0; s < n; ++s) {
        offs[(size_t)s] = total;
        total += 2 * rev_offset(lens[s]);
    }
    total += kGuard;
    out.assign((size_t)total, 0);
    int8_t map[32];
    memcpy(map, remap, sizeof(map));
    for (int s = 0; s < n; ++s) {
        const int8_t* src = row(s);
        int8_t* f = out.data() + offs[(size_t)s];
        const int L = lens[s];
        int8_t* r = f + rev_offset(L) + (L - 1);
        for (int i = 0; i < L; ++i) {
            const int8_t c = map[src[i] & 31];
            f[i] = c;
            r[-i] = c;
        }
    }
}

}  // namespace cwgpu

#endif  // CWGPU_LAYOUT_H
