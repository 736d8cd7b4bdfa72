// Peak-rate microbenchmarks for the roofline denominators of pipes that a copy
// or GEMM benchmark does not measure (the machine's measured peaks cover HBM
// copy bandwidth and bf16 tensor throughput only):
//   0  FP32 FFMA        (independent chains, ops = 2 flop each)
//   1  FP64 DFMA
//   2  32-bit IMAD
//   3  PCG64DXSM draws  (the generator alone: 128-bit LCG step + DXSM output,
//                        the irreducible work of every path kernel)
// Each kernel writes one word per thread so nothing is dead code.
#include <cuda_runtime.h>

#include "mc_device.cuh"

namespace stocha {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_ffma(int iters, float a, float b, float* out) {
  float v[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) v[i] = (float)(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = fmaf(v[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += v[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_dfma(int iters, double a, double b, double* out) {
  double v[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) v[i] = (double)(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = fma(v[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += v[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_imad(int iters, unsigned a, unsigned b, unsigned* out) {
  unsigned v[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) v[i] = threadIdx.x + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = v[i] * a + b;
  }
  unsigned s = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s ^= v[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Two independent streams per thread (the path kernels run one stream per
// thread; two give the scheduler the same ILP a second resident warp would).
__global__ void __launch_bounds__(256) k_pcg(int iters, uint64_t inc_lo, uint64_t inc_hi, uint64_t* out) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  DevPcg s0{t * 0x9E3779B97F4A7C15ull, t}, s1{~t, t * 3};
  uint64_t acc = 0;
  for (int it = 0; it < iters; ++it) {
    acc ^= pcg_next(s0, inc_lo, inc_hi);
    acc += pcg_next(s1, inc_lo, inc_hi);
  }
  out[t] = acc;
}

}  // namespace

// Returns ops/s for the requested kind (FFMA: flop/s; DFMA: flop/s; IMAD:
// ops/s; PCG: draws/s), timed with CUDA events on `st`.
double measure_peak(int kind, cudaStream_t st) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256, grid = sms * 8;
  const uint64_t threads = (uint64_t)grid * block;
  void* buf = nullptr;
  if (cudaMalloc(&buf, threads * 8) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = kind == 1 ? 256 : kind == 3 ? 2048 : 4096;
  auto launch = [&]() {
    if (kind == 0) k_ffma<<<grid, block, 0, st>>>(iters, 0.999f, 0.001f, (float*)buf);
    if (kind == 1) k_dfma<<<grid, block, 0, st>>>(iters, 0.999, 0.001, (double*)buf);
    if (kind == 2) k_imad<<<grid, block, 0, st>>>(iters, 2654435761u, 12345u, (unsigned*)buf);
    if (kind == 3) k_pcg<<<grid, block, 0, st>>>(iters, 0x5851F42D4C957F2Dull | 1, 0x14057B7EF767814Full, (uint64_t*)buf);
  };
  for (int w = 0; w < 3; ++w) launch();
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0, st);
    launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  const double per_thread = kind == 3 ? 2.0 * iters : (double)kChains * iters * (kind <= 1 ? 2.0 : 1.0);
  return per_thread * (double)threads / (best * 1e-3);
}

}  // namespace stocha
