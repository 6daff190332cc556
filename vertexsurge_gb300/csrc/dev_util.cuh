// Warp/block reduction helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vs {

constexpr unsigned FULLMASK = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}

// Block-wide sum of per-thread counters, one atomic per block.  Every thread
// of the block must call it.
__device__ __forceinline__ void block_add(unsigned long long v, unsigned long long *dst) {
  __shared__ unsigned long long part[32];
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0ull;
    v = warp_sum(v);
    if (threadIdx.x == 0 && v) atomicAdd(dst, v);
  }
}

}  // namespace vs
