// Deterministic reductions: FP64 block sums with a fixed thread->data mapping,
// then a last-block finalize that sums the per-block partials in index order.
// No block ever waits for another (the last block to arrive does the final
// sum), so there is no spin-wait anywhere.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace erp {

// Sum of v over the block; result valid in thread 0.  sh: >= blockDim/32 doubles.
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < nw) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// Thread 0 publishes `nv` values of this block into partials[slot*nv + k];
// returns true (in every thread) in the block that arrives last.
__device__ __forceinline__ bool arrive_last(double *partials, int slot, int nv, const double *vals,
                                            uint32_t *ctr, uint32_t nblocks) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        for (int k = 0; k < nv; ++k) partials[(size_t)slot * nv + k] = vals[k];
        __threadfence();
        const uint32_t t = atomicAdd(ctr, 1u);
        s_last = (t == nblocks - 1);
    }
    __syncthreads();
    const bool last = s_last != 0;
    if (last) __threadfence();
    return last;
}

// In the last block: sum partials[k*nv + j] over k < count for value j (fixed order).
__device__ __forceinline__ double sum_partials(const double *partials, int count, int nv, int j,
                                               double *sh) {
    double v = 0.0;
    for (int k = threadIdx.x; k < count; k += blockDim.x) v += __ldcg(partials + (size_t)k * nv + j);
    return block_sum(v, sh);
}

}  // namespace erp
