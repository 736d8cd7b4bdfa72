// FP32 path kernels.  Same streams, same draws and the same discretisation as
// the FP64 kernels (the samplers consume exactly the reference's u64s, so the
// FP32 result differs from the FP64 one by rounding only, not by Monte Carlo
// noise).  The recurrences are carried in log space:
//   GBM    log S_k = log s0 + k*drift + diffusion * sum_{i<=k} z_i
//   multi  log S_k = log s0 + k*drift + diffusion * (L * sum z)_k
//   Merton log S_k = log s0 + k*drift + diffusion * sum z + sum jumps
//   Heston log S_k += (mu - v+/2) dt + sqrt(v+ dt) dw1   (v in FP32)
// which equal the reference's products of exponentials (gbm.rs:71,
// multi_gbm.rs:246, jump_diffusion.rs:87, heston.rs:69) in exact arithmetic.
// Sums over steps are compensated (Kahan); payoff sums over paths are
// compensated FP32 per thread and FP64 per block.
#include <cuda_runtime.h>

#include "engine.h"
#include "mc_device.cuh"
#include "reduce.cuh"

namespace stocha {
namespace {

struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s - c; }
};

__device__ __forceinline__ float payoff_f32(float s, float k, int kind) {
  return kind == kCall ? fmaxf(s - k, 0.0f) : fmaxf(k - s, 0.0f);
}

__device__ __forceinline__ void store32(const PathLaunch& a, uint64_t lrow, uint64_t step, uint64_t width,
                                        uint64_t col, float v) {
  if (a.time_major)
    a.out_f32[(step * width + col) * a.rows + lrow] = v;
  else
    a.out_f32[(lrow * (a.steps + 1) + step) * width + col] = v;
}

template <bool kStore>
__global__ void __launch_bounds__(256) k_gbm_f32(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  Kahan acc, acc2;
  const float s0 = (float)a.gbm.s0, drift = (float)a.gbm.drift, diffusion = (float)a.gbm.diffusion;
  const float strike = (float)a.strike;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t lrow = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; lrow < a.rows; lrow += nthreads) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    Kahan w;
    float kf = 0.0f;  // step count as float (no per-step integer conversion)
    if (kStore) store32(a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      float z = normal_f32(s, c, zs, err);
      w.add(neg ? -z : z);
      kf += 1.0f;
      if (kStore) store32(a, lrow, k, 1, 0, s0 * expf(fmaf(kf, drift, diffusion * w.value())));
    }
    if (!kStore) {
      float sT = s0 * expf(fmaf(diffusion, w.value(), a.f32.g_kdrift));
      float p = payoff_f32(sT, strike, a.payoff);
      acc.add(p);
      acc2.add(p * p);
    }
  }
  if (!kStore) block_sum2_store((double)acc.value(), (double)acc2.value(), a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

template <int NA, bool kStore>
__global__ void __launch_bounds__(256) k_multi_gbm_f32(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  constexpr int CAP = NA > 0 ? NA : kMaxAssets;
  const int na = NA > 0 ? NA : a.multi.na;
  unsigned err = 0;
  Kahan acc[CAP], acc2[CAP];
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t lrow = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; lrow < a.rows; lrow += nthreads) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    Kahan w[CAP];
    const F32K& f = a.f32;
    float kf = 0.0f;
    if (kStore)
      for (int i = 0; i < na; ++i) store32(a, lrow, 0, na, i, f.a_s0[i]);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
#pragma unroll
      for (int i = 0; i < na; ++i) {
        float z = normal_f32(s, c, zs, err);
        w[i].add(neg ? -z : z);
      }
      kf += 1.0f;
      if (kStore) {
#pragma unroll
        for (int i = 0; i < na; ++i) {
          float eps = 0.0f;
#pragma unroll
          for (int m = 0; m <= i; ++m) eps = fmaf(f.a_L[i * kMaxAssets + m], w[m].value(), eps);
          float lg = fmaf(kf, f.a_drift[i], f.a_diff[i] * eps);
          store32(a, lrow, k, na, i, f.a_s0[i] * expf(lg));
        }
      }
    }
    if (!kStore) {
#pragma unroll
      for (int i = 0; i < na; ++i) {
        float eps = 0.0f;
#pragma unroll
        for (int m = 0; m <= i; ++m) eps = fmaf(f.a_L[i * kMaxAssets + m], w[m].value(), eps);
        float lg = fmaf(f.a_diff[i], eps, f.a_kdrift[i]);
        float p = payoff_f32(f.a_s0[i] * expf(lg), f.strike, a.payoff);
        acc[i].add(p);
        acc2[i].add(p * p);
      }
    }
  }
  if (!kStore)
    for (int i = 0; i < na; ++i)
      block_sum2_store((double)acc[i].value(), (double)acc2[i].value(),
                       a.partials + (2 * (uint64_t)blockIdx.x) * na + 2 * i);
  if (err) atomicOr(a.err, err);
}

template <bool kStore>
__global__ void __launch_bounds__(256) k_heston_euler_f32(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const HestonK& h = a.heston;
  const float rho = (float)h.rho, rho_comp = (float)h.rho_comp, kappa_dt = (float)(h.kappa * h.dt);
  const float theta = (float)h.theta, xi_sdt = (float)(h.xi * h.sqrt_dt), sdt = (float)h.sqrt_dt;
  const float mu_dt = (float)(h.mu * h.dt), half_dt = (float)(0.5 * h.dt), s0 = (float)h.s0;
  unsigned err = 0;
  Kahan acc, acc2;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t lrow = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; lrow < a.rows; lrow += nthreads) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    float v = (float)h.v0;
    Kahan lg;
    if (kStore) store32(a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      float dw1 = normal_f32(s, c, zs, err);
      float dz = normal_f32(s, c, zs, err);
      float dw2 = fmaf(rho, dw1, rho_comp * dz);
      float v_plus = fmaxf(v, 0.0f);
      float sqrt_v = sqrtf(v_plus);
      v += fmaf(kappa_dt, theta - v_plus, xi_sdt * sqrt_v * dw2);
      lg.add(fmaf(-half_dt, v_plus, mu_dt) + sqrt_v * sdt * dw1);
      if (kStore) store32(a, lrow, k, 1, 0, s0 * expf(lg.value()));
    }
    if (!kStore) {
      float p = payoff_f32(s0 * expf(lg.value()), a.f32.strike, a.payoff);
      acc.add(p);
      acc2.add(p * p);
    }
  }
  if (!kStore) block_sum2_store((double)acc.value(), (double)acc2.value(), a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

template <bool kStore>
__global__ void __launch_bounds__(256) k_merton_f32(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const MertonK& M = a.merton;
  const float drift = (float)M.drift, diffusion = (float)M.diffusion, mu_j = (float)M.mu_j;
  const float sigma_j = (float)M.sigma_j, s0 = (float)M.s0;
  unsigned err = 0;
  Kahan acc, acc2;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t lrow = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; lrow < a.rows; lrow += nthreads) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    Kahan w;
    float jumps = 0.0f, kf = 0.0f;
    if (kStore) store32(a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      w.add(normal_f32(s, c, zs, err));
      uint64_t u = s.next();
      if ((u >> 11) < M.jump_thr) jumps += fmaf(sigma_j, normal_f32(s, c, zs, err), mu_j);
      kf += 1.0f;
      if (kStore) store32(a, lrow, k, 1, 0, s0 * expf(fmaf(kf, drift, diffusion * w.value()) + jumps));
    }
    if (!kStore) {
      float sT = s0 * expf(fmaf(diffusion, w.value(), a.f32.m_kdrift) + jumps);
      float p = payoff_f32(sT, a.f32.strike, a.payoff);
      acc.add(p);
      acc2.add(p * p);
    }
  }
  if (!kStore) block_sum2_store((double)acc.value(), (double)acc2.value(), a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

template <bool kStore>
void launch_multi32(const PathLaunch& L, dim3 g, dim3 b, cudaStream_t st) {
  switch (L.multi.na) {
    case 1: k_multi_gbm_f32<1, kStore><<<g, b, 0, st>>>(L); break;
    case 2: k_multi_gbm_f32<2, kStore><<<g, b, 0, st>>>(L); break;
    case 3: k_multi_gbm_f32<3, kStore><<<g, b, 0, st>>>(L); break;
    case 4: k_multi_gbm_f32<4, kStore><<<g, b, 0, st>>>(L); break;
    default: k_multi_gbm_f32<0, kStore><<<g, b, 0, st>>>(L); break;
  }
}

}  // namespace

int launch_paths_f32(const PathLaunch& L, cudaStream_t st) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int b = 256;
  const bool store = L.out_f32 != nullptr;
  // Persistent grid: exactly the blocks that are resident at once, so the
  // grid-stride loop gives every thread the same number of paths (+-1) in a
  // single wave instead of a partial second wave of blocks.
  const void* fn = nullptr;
  switch (L.model) {
    case kGbm: fn = store ? (const void*)k_gbm_f32<true> : (const void*)k_gbm_f32<false>; break;
    case kHeston: fn = store ? (const void*)k_heston_euler_f32<true> : (const void*)k_heston_euler_f32<false>; break;
    case kMerton: fn = store ? (const void*)k_merton_f32<true> : (const void*)k_merton_f32<false>; break;
    default: fn = store ? (const void*)k_multi_gbm_f32<3, true> : (const void*)k_multi_gbm_f32<3, false>; break;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, b, 0) != cudaSuccess || per_sm < 1) per_sm = 2;
  uint64_t g = (L.rows + b - 1) / b;
  const uint64_t cap = (uint64_t)sms * per_sm;
  if (g > cap && !L.flat_grid) g = cap;
  if (g < 1) g = 1;
  dim3 G((unsigned)g), B(b);
  switch (L.model) {
    case kGbm:
      if (store) k_gbm_f32<true><<<G, B, 0, st>>>(L); else k_gbm_f32<false><<<G, B, 0, st>>>(L);
      break;
    case kHeston:
      if (L.heston.scheme != 0) return -1;  // QE has no FP32 form
      if (store) k_heston_euler_f32<true><<<G, B, 0, st>>>(L); else k_heston_euler_f32<false><<<G, B, 0, st>>>(L);
      break;
    case kMerton:
      if (store) k_merton_f32<true><<<G, B, 0, st>>>(L); else k_merton_f32<false><<<G, B, 0, st>>>(L);
      break;
    case kMultiGbm:
      if (store) launch_multi32<true>(L, G, B, st); else launch_multi32<false>(L, G, B, st);
      break;
    default:
      return -1;
  }
  return cudaPeekAtLastError() == cudaSuccess ? (int)g : -1;
}

}  // namespace stocha
