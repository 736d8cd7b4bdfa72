// VaR / CVaR of a return series on the device (src/risk/var_cvar.rs:7-43).
//
// The reference negates the returns into losses, sorts them with total_cmp
// and reads the loss at rank idx = min(ceil(confidence * n), n - 1); CVaR is
// the mean of the sorted tail losses[idx..].  Here nothing is sorted: losses
// are mapped to 64-bit keys whose unsigned order is total_cmp's order, and an
// 8-pass radix select (8 bits per pass, histograms in shared memory; the
// first pass also checks that every return is finite) finds the key of rank
// idx, the number of smaller keys and the number of equal keys.
// The tail is then every loss with a larger key plus the copies of the VaR
// value that the sorted order places at or after idx.  VaR is exact; CVaR
// differs from the reference's sequential sum by summation order only.
#include <cuda_runtime.h>

#include "reduce.cuh"
#include "risk_kernels.h"

namespace stocha {
namespace {

// total_cmp order as unsigned order: flip all bits of negatives, the sign bit
// of the rest.  The loss -ret is the return with its sign bit flipped.  The
// returns are read as 64-bit integers so that all of this stays on the
// integer pipes (GB300 runs FP64 at 1/64 of the FP32 rate).
__device__ __forceinline__ uint64_t loss_key(uint64_t ret_bits) {
  const uint64_t b = ret_bits ^ 0x8000000000000000ull;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// One select pass: histogram of digit `shift` of the keys that carry the
// prefix found so far.  The first pass (shift 56, every key matches) also
// flags a NaN or infinite return (exponent field all ones) in *bad.
__global__ void __launch_bounds__(256) k_select_hist(const double* __restrict__ r, uint64_t n,
                                                     const SelectState* __restrict__ st, int shift,
                                                     unsigned long long* __restrict__ hist,
                                                     unsigned* __restrict__ bad) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t prefix = st->prefix, mask = st->mask;
  const uint64_t* __restrict__ rb = reinterpret_cast<const uint64_t*>(r);
  bool nonfinite = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t bits = rb[i];
    if (shift == 56) nonfinite |= ((bits >> 52) & 0x7FF) == 0x7FF;
    const uint64_t k = loss_key(bits);
    if ((k & mask) == prefix) atomicAdd(&h[(k >> shift) & 0xFF], 1u);
  }
  if (shift == 56 && __syncthreads_or(nonfinite) && threadIdx.x == 0) atomicOr(bad, 1u);
  __syncthreads();
  if (h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

// One thread: the digit holding the wanted rank; clears the histogram.
__global__ void k_select_step(SelectState* __restrict__ st, int shift, unsigned long long* __restrict__ hist) {
  if (threadIdx.x != 0) return;
  uint64_t rank = st->rank, below = 0;
  int d = 0;
  for (; d < 255; ++d) {
    if (rank < below + hist[d]) break;
    below += hist[d];
  }
  st->less += below;
  st->rank = rank - below;
  st->equal = hist[d];
  st->prefix |= (uint64_t)d << shift;
  st->mask |= (uint64_t)0xFF << shift;
  for (int j = 0; j < 256; ++j) hist[j] = 0;
}

// Sum of the losses with keys above the selected one.
__global__ void __launch_bounds__(256) k_tail_sum(const double* __restrict__ r, uint64_t n,
                                                  const SelectState* __restrict__ st, double* __restrict__ part) {
  const uint64_t key = st->prefix;
  const uint64_t* __restrict__ rb = reinterpret_cast<const uint64_t*>(r);
  double s = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t bits = rb[i];
    // Only the tail (a fraction 1 - confidence of the returns) is added.  A
    // warp issues the FP64 add (1/64 of the FP32 rate on GB300) only when one
    // of its lanes holds a tail loss; a predicated add would occupy the FP64
    // pipe for every element.
    const bool take = loss_key(bits) > key;
    if (__any_sync(__activemask(), take) && take) s -= __longlong_as_double((long long)bits);
  }
  block_sum2_store(s, 0.0, part + 2 * (uint64_t)blockIdx.x);
}

}  // namespace

void launch_select(const double* r, uint64_t n, SelectState* state, unsigned long long* hist, unsigned* bad,
                   int grid, cudaStream_t st) {
  for (int shift = 56; shift >= 0; shift -= 8) {
    k_select_hist<<<grid, 256, 0, st>>>(r, n, state, shift, hist, bad);
    k_select_step<<<1, 32, 0, st>>>(state, shift, hist);
  }
}

void launch_tail_sum(const double* r, uint64_t n, const SelectState* state, double* part, int grid,
                     cudaStream_t st) {
  k_tail_sum<<<grid, 256, 0, st>>>(r, n, state, part);
}

}  // namespace stocha
