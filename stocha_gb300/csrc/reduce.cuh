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

// Sums v[0..N) over the block; threads j < N write out[j] = total of value j
// (warp trees, then the warps in order).  Every thread must call it.
template <int N>
__device__ __forceinline__ void block_sum_n_store(const double* v, double* out) {
  __shared__ double red[32][N];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();  // protects red against a previous call's readers
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const double w = warp_sum(v[j]);
    if (lane == 0) red[wid][j] = w;
  }
  __syncthreads();
  if ((int)threadIdx.x < N) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// Block totals of N compensated FP32 sums (value = s[j] - c[j] per thread):
// warp trees that carry the compensation (Knuth's two-sum at every level,
// error-free in FP32), then one warp adds the warps' pairs in FP64 in warp
// order.  Threads j < N write out[j].  FP64 instructions issue at 1/64 of the
// FP32 rate on this GPU: this keeps them to one warp's worth per block.
// Every thread must call it.
template <int N>
__device__ __forceinline__ void block_sum_kahan_store(const float* s, const float* c, double* out) {
  __shared__ float red_s[32][N], red_c[32][N];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();  // protects red_* against a previous call's readers
#pragma unroll
  for (int j = 0; j < N; ++j) {
    float a = s[j], ca = c[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float b = __shfl_down_sync(0xffffffffu, a, o);
      const float cb = __shfl_down_sync(0xffffffffu, ca, o);
      const float t = a + b;
      const float bp = t - a;
      const float e = (a - (t - bp)) + (b - bp);  // t + e == a + b exactly
      a = t;
      ca = (ca + cb) - e;
    }
    if (lane == 0) {
      red_s[wid][j] = a;
      red_c[wid][j] = ca;
    }
  }
  __syncthreads();
  if ((int)threadIdx.x < N) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += (double)red_s[w][threadIdx.x] - (double)red_c[w][threadIdx.x];
    out[threadIdx.x] = t;
  }
}

}  // namespace stocha
