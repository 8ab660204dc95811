// Fixed-order block reductions (bitwise reproducible from run to run).
#pragma once

#include "vmc_common.cuh"

namespace vmc {

// Number of blocks of a grid-stride reduction: two per SM of a GB300.
constexpr int kReduceBlocks = 304;

// Sum over the threads of a block (blockDim.x a multiple of 32, <= 1024).
// All threads receive the result.
template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T s_part[32];
  __shared__ T s_total;
  v = warp_sum(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) s_part[w] = v;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    T x = l < nw ? s_part[l] : T(0);
    x = warp_sum(x);
    if (l == 0) s_total = x;
  }
  __syncthreads();
  T r = s_total;
  __syncthreads();
  return r;
}

}  // namespace vmc

extern "C" size_t vmc_reduce_workspace_bytes(int64_t num_outputs);
