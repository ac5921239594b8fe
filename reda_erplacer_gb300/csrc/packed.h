// Packed launches (batches): one grid over the blocks of many instances of one
// kernel.  Instance i owns blocks [block0[i], block0[i + 1]) and reads its
// arguments from tab[i].  Each instance's blocks see the block index and the
// grid size they would have in a launch of their own, so every instance
// computes the same bits as alone.
//
// The header compiles for the device and for the host, so that a host program
// can check the block-to-instance mapping (tests/test_packed_map.py).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define ERP_PK_FN __host__ __device__ __forceinline__
#else
#define ERP_PK_FN static inline
#endif

namespace erp {

template <typename P>
struct Packed {
    const P *tab;
    const int32_t *block0;
    int32_t n;
};

// The instance that owns block b: the last i with block0[i] <= b.  block0 holds
// n + 1 ascending prefixes, block0[0] = 0, and every instance owns at least one
// block (0 <= b < block0[n]).
ERP_PK_FN int packed_instance(const int32_t *__restrict__ block0, int n, int b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
#if defined(__CUDA_ARCH__)
        const int v = __ldg(block0 + mid);
#else
        const int v = block0[mid];
#endif
        if (v <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace erp

#undef ERP_PK_FN
