// Block reductions with a fixed combination order (results are reproducible
// run to run): warp shuffles, then one warp over the per-warp values.
#pragma once
#include <cuda_runtime.h>

namespace stocha {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sums (a, b) over the block; thread 0 writes out[0] = sum a, out[1] = sum b.
// Every thread of the block must call it.
__device__ __forceinline__ void block_sum2_store(double a, double b, double* out) {
  __shared__ double sa[32], sb[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  __syncthreads();  // protects sa/sb against a previous call's readers
  if (lane == 0) {
    sa[wid] = a;
    sb[wid] = b;
  }
  __syncthreads();
  if (wid == 0) {
    a = lane < nw ? sa[lane] : 0.0;
    b = lane < nw ? sb[lane] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
      out[0] = a;
      out[1] = b;
    }
  }
}

}  // namespace stocha
