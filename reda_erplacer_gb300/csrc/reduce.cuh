// Deterministic reductions in double-float arithmetic (dfloat.h): a sum is
// carried as an unevaluated pair hi + lo of FP32 values, about 44 significant
// bits, and converted to FP64 once, at the end.  FP64 issues at a small
// fraction of the FP32 rate on this GPU: with FP64 block sums every reduction
// tail was a long dependent chain on that pipe.
//
// Block sums use a fixed thread -> data mapping and shuffle tree; the block
// that arrives last sums the per-block partials in index order.  No block ever
// waits for another, so there is no spin-wait anywhere, and the result depends
// only on the data and the grid.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.h"

namespace erp {

// a partial slot (8 bytes, allocated as double) holds one pair
static_assert(sizeof(Df) == sizeof(double), "partial slot size");

__device__ __forceinline__ Df df_shfl_down(Df v, int o) {
    return Df{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

// Sum of v over the block; result valid in thread 0.  sh: >= blockDim/32 slots.
__device__ __forceinline__ Df block_sum(Df v, double *sh) {
    Df *shp = reinterpret_cast<Df *>(sh);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, df_shfl_down(v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) shp[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < nw) ? shp[l] : df_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = df_add(v, df_shfl_down(v, o));
    }
    return v;
}

__device__ __forceinline__ Df block_sum(float v, double *sh) { return block_sum(Df{v, 0.0f}, sh); }

// Thread 0 publishes `nv` sums of this block into partial slots slot*nv + k;
// returns true (in every thread) in the block that arrives last.
__device__ __forceinline__ bool arrive_last(double *partials, int slot, int nv, const Df *vals, uint32_t *ctr,
                                            uint32_t nblocks) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        Df *p = reinterpret_cast<Df *>(partials);
        for (int k = 0; k < nv; ++k) p[(size_t)slot * nv + k] = vals[k];
        __threadfence();
        const uint32_t t = atomicAdd(ctr, 1u);
        s_last = (t == nblocks - 1);
    }
    __syncthreads();
    const bool last = s_last != 0;
    if (last) __threadfence();
    return last;
}

// In the last block: the sum of partial slots k*nv + j over k < count (fixed
// order), as FP64 in thread 0.
__device__ __forceinline__ double sum_partials(const double *partials, int count, int nv, int j, double *sh) {
    const float2 *p = reinterpret_cast<const float2 *>(partials);
    Df v = df_zero();
    for (int k = threadIdx.x; k < count; k += blockDim.x) {
        const float2 q = __ldcg(p + (size_t)k * nv + j);
        v = df_add(v, Df{q.x, q.y});
    }
    return df_value(block_sum(v, sh));
}

}  // namespace erp
