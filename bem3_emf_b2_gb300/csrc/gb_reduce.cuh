// gb_reduce.cuh -- warp and block reductions of small FP64 vectors.
#pragma once
#include "gb_common.cuh"

// Sum NV doubles over the 32 lanes of a warp; every lane receives the sum.
template <int NV>
__device__ __forceinline__ void warp_allreduce(double* v) {
#pragma unroll
  for (int i = 0; i < NV; i++) {
    double x = v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    v[i] = x;
  }
}

// Sum NV doubles over the block (blockDim.x a multiple of 32, <= 1024).
// smem must hold NV * (blockDim.x / 32) doubles.  The result is returned in
// v[] of thread 0 only.
template <int NV>
__device__ __forceinline__ void block_reduce(double* v, double* smem) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; i++) {
    double x = v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) smem[i * nw + wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; i++) {
      double s = 0.0;
      for (int w = 0; w < nw; w++) s += smem[i * nw + w];
      v[i] = s;
    }
  }
}
