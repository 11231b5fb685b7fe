// rpd_scan.cuh -- warp and block prefix sums shared by the kernels that
// scan per-thread counts (scans, compactions, polygon offsets), for 32- and
// 64-bit values.
#pragma once

#include <cuda_runtime.h>

namespace rpd {

// inclusive prefix sum of v over the lanes of a full warp
template <class T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// block-wide exclusive prefix sum of one value per thread (every thread of
// the block calls it; blockDim.x a multiple of 32, at most 1024); returns
// the thread's exclusive prefix and writes the block total to *total
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* total) {
  __shared__ T wsum[32];
  __shared__ T wtot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const T incl = warp_incl_scan<T>(v, lane);
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    const T x = lane < nw ? wsum[lane] : T(0);
    const T xi = warp_incl_scan<T>(x, lane);
    if (lane < nw) wsum[lane] = xi - x;
    if (lane == 31) wtot = xi;
  }
  __syncthreads();
  const T res = incl - v + wsum[wid];
  if (total) *total = wtot;
  __syncthreads();
  return res;
}

}  // namespace rpd
