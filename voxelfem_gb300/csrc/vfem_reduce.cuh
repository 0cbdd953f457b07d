// Warp-shuffle block reductions (deterministic for a fixed launch shape).
#pragma once
#include <cuda_runtime.h>

namespace vfem {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; the result is valid in thread 0. Every thread must call it.
template <int BS>
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[BS / 32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0;
    if (w == 0) {
        r = (lane < BS / 32) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

}  // namespace vfem
