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
// Sums over steps are compensated (Kahan) where each partial sum is stored
// and plain in the fused forms (see Plain); payoff sums over paths are
// compensated FP32 per thread and FP64 per block.
#include <cuda_runtime.h>

#include <type_traits>

#include "engine.h"
#include "mc_device.cuh"
#include "reduce.cuh"
#include "row_store.cuh"

namespace stocha {
namespace {

// Staging area of the row-major stores: RowStore<float>::bytes(blockDim.x)
// bytes, passed at launch in the kRows mode.
extern __shared__ __align__(16) unsigned char dyn_smem[];

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

// Plain FP32 running sum, for the per-path sums of the fused forms: over 252
// steps its rounding error (~sqrt(steps) * ulp(sqrt(steps)) / 3.5, about 5e-6
// absolute for a sum of normals) is of the order of the FP32 normals' own
// error, so compensation (3 more adds per term) buys nothing there.
struct Plain {
  float s = 0.0f;
  __device__ __forceinline__ void add(float v) { s += v; }
  __device__ __forceinline__ float value() const { return s; }
};

// Resident 256-thread blocks per SM the fused kernels are compiled for (a
// register cap of 48).  These kernels are issue-bound: 5 blocks (40 warps)
// instead of the 4 that 64 registers allow hide more of the generator's
// dependent-issue latency, and the values the cap spills belong to the rare
// wedge and tail paths (measured on GB300: multi-GBM 2.97 -> 2.74 ms, Heston
// 2.08 -> 2.02 ms, Merton 1.52 -> 1.48 ms; 6 blocks spilled into the common
// path).  The warp-uniform forms carry more state (the sampler feed's pending
// draw and value): 4 blocks, 64 registers (a 56-register cap measured within
// noise, 48 spilled on the common path).
constexpr int kFusedMinBlocks = 5;
constexpr int kUfMinBlocks = 4;
// The materialised and element-store forms (staged row store, time-major
// columns): 4 resident 256-thread blocks (64 registers; 3 blocks at 76
// registers before).  Measured on GB300 at 1e6 x 252: FP32 materialised
// 7.79 -> 7.54 ms (multi-GBM 3.80 -> 3.65, Heston 2.28 -> 2.22, Merton
// 1.71 -> 1.67); 3 blocks gave 7.73 ms.
constexpr int kMatMinBlocks = 4;

// Per-path running sum: compensated where every partial sum is stored (the
// materialised paths), plain where only the last one is used.
template <bool kStore>
using PathSum = typename std::conditional<kStore, Kahan, Plain>::type;

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

template <int kMode>
__device__ __forceinline__ void emit32(PathOut<float, kMode>& out, const PathLaunch& a, uint64_t lrow, uint64_t step,
                                       uint64_t width, uint64_t col, float v) {
  if (kMode == kRows)
    out.rs.put(v);
  else if (kMode == kElems)
    store32(a, lrow, step, width, col, v);
}

// Block partial record: {sum payoff, sum payoff^2} per asset, compensated
// FP32 per thread and FP64 across the block (all threads must call it).
template <int NV>
__device__ __forceinline__ void store_partials(const PathLaunch& a, const Kahan* acc, const Kahan* acc2) {
  float s[2 * NV], c[2 * NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    s[2 * i] = acc[i].s;
    c[2 * i] = acc[i].c;
    s[2 * i + 1] = acc2[i].s;
    c[2 * i + 1] = acc2[i].c;
  }
  block_sum_kahan_store<2 * NV>(s, c, a.partials + (uint64_t)blockIdx.x * 2 * NV);
}

// Row driver of the fused kernels.  batch(b, p) prices row b + lane of a
// warp's batch of 32 consecutive rows (called by all 32 lanes; it returns
// false, without simulating, for a row past the end) and leaves the row's
// payoff per asset in p.
//   * static (a.work null): warp batches in grid-stride order; one record per
//     block (store_partials).
//   * work queue: a warp takes a.batch_rows consecutive rows at a time from
//     the launch counter *a.work and writes one record per batch, the batch's
//     sums in a fixed lane order (FP64 warp tree).  Every SM stays busy until
//     the last batch (a static grid of P paths per thread leaves most SMs idle
//     through the last round when the rows are not a multiple of the
//     resident threads), and the records do not depend on which warp ran
//     which batch, so the price is the same run to run.
template <int NV, class Batch>
__device__ __forceinline__ void run_rows(const PathLaunch& a, Batch&& batch) {
  const unsigned lane = threadIdx.x & 31u;
  if (a.work) {
    const uint32_t per_lane = a.batch_rows >> 5;
#pragma unroll 1
    for (;;) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(a.work, (unsigned long long)a.batch_rows);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= a.rows) break;
      double* rec = a.partials + (base / a.batch_rows) * (2 * NV);
      // Each group of 32 rows is added into the record at once (FP64 warp
      // tree, then lane 0 adds it to the record in group order), so no sum
      // stays live in registers while the next row is simulated.
#pragma unroll 1
      for (uint32_t j = 0; j < per_lane; ++j) {
        const uint64_t b = base + 32ull * j;
        if (b >= a.rows) break;  // warp-uniform
        float p[NV];
        const bool ok = batch(b, p);
#pragma unroll
        for (int i = 0; i < NV; ++i) {
          const double v = warp_sum(ok ? (double)p[i] : 0.0);
          const double v2 = warp_sum(ok ? (double)(p[i] * p[i]) : 0.0);
          if (lane == 0) {
            rec[2 * i] = j ? rec[2 * i] + v : v;
            rec[2 * i + 1] = j ? rec[2 * i + 1] + v2 : v2;
          }
        }
      }
    }
    return;
  }
  Kahan acc[NV], acc2[NV];
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
#pragma unroll 1
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); b < a.rows; b += nthreads) {
    float p[NV];
    if (batch(b, p)) {
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        acc[i].add(p[i]);
        acc2[i].add(p[i] * p[i]);
      }
    }
  }
  store_partials<NV>(a, acc, acc2);
}

template <int kMode>
__global__ void __launch_bounds__(256, kMode != kFused ? kMatMinBlocks : 1) k_gbm_f32(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  PathOut<float, kMode> out;
  out.init(dyn_smem);
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  // FP32 constants rounded once on the host (F32K): under the register cap a
  // value converted here from the double parameters could be rematerialised
  // inside the path loop, putting a conversion on the FP64 pipe every step
  const float s0 = a.f32.g_s0, drift = a.f32.g_drift, diffusion = a.f32.g_diff;
  const float strike = a.f32.strike;
  // one path: materialised rows (kStore) or the payoff of S_T
  auto path = [&](uint64_t lrow, float* pay) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    PathSum<kStore> w;
    float kf = 0.0f;  // step count as float (no per-step integer conversion)
    if (kMode == kRows) out.begin(a.out_f32 + lrow * (a.steps + 1));
    if (kStore) emit32(out, a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      float z = normal_f32(s, c, zs, err);
      if (kStore) {
        w.add(neg ? -z : z);
        kf += 1.0f;
        emit32(out, a, lrow, k, 1, 0, s0 * expf(fmaf(kf, drift, diffusion * w.value())));
      } else {
        w.add(z);  // the antithetic sign is applied to the sum (negation is exact)
      }
    }
    if (!kStore) {
      const float sum = neg ? -w.value() : w.value();
      pay[0] = payoff_f32(s0 * expf(fmaf(diffusion, sum, a.f32.g_kdrift)), strike, a.payoff);
    }
  };
  if constexpr (kStore) {
    for_rows(a.rows, out, [&](uint64_t lrow) { path(lrow, nullptr); });
  } else {
    run_rows<1>(a, [&](uint64_t b, float* p) {
      const uint64_t lrow = b + (threadIdx.x & 31u);
      if (lrow >= a.rows) return false;
      path(lrow, p);
      return true;
    });
  }
  if (err) atomicOr(a.err, err);
}

template <int NA, int kMode>
__global__ void __launch_bounds__(256, kMode != kFused ? kMatMinBlocks : kFusedMinBlocks) k_multi_gbm_f32(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  PathOut<float, kMode> out;
  out.init(dyn_smem);
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  constexpr int CAP = NA > 0 ? NA : kMaxAssets;
  const int na = NA > 0 ? NA : a.multi.na;
  unsigned err = 0;
  const F32K& f = a.f32;
  auto path = [&](uint64_t lrow, float* pay) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    PathSum<kStore> w[CAP];
    float kf = 0.0f;
    if (kMode == kRows) out.begin(a.out_f32 + lrow * (a.steps + 1) * na);
    if (kStore)
      for (int i = 0; i < na; ++i) emit32(out, a, lrow, 0, na, i, f.a_s0[i]);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
#pragma unroll
      for (int i = 0; i < na; ++i) {
        float z = normal_f32(s, c, zs, err);
        w[i].add(kStore && neg ? -z : z);  // fused: the sign is applied to the sums
      }
      kf += 1.0f;
      if (kStore) {
#pragma unroll
        for (int i = 0; i < na; ++i) {
          float eps = 0.0f;
#pragma unroll
          for (int m = 0; m <= i; ++m) eps = fmaf(f.a_L[i * kMaxAssets + m], w[m].value(), eps);
          float lg = fmaf(kf, f.a_drift[i], f.a_diff[i] * eps);
          emit32(out, a, lrow, k, na, i, f.a_s0[i] * expf(lg));
        }
      }
    }
    if (!kStore) {
#pragma unroll
      for (int i = 0; i < na; ++i) {
        float eps = 0.0f;
#pragma unroll
        for (int m = 0; m <= i; ++m) eps = fmaf(f.a_L[i * kMaxAssets + m], neg ? -w[m].value() : w[m].value(), eps);
        float lg = fmaf(f.a_diff[i], eps, f.a_kdrift[i]);
        pay[i] = payoff_f32(f.a_s0[i] * expf(lg), f.strike, a.payoff);
      }
    }
  };
  if constexpr (!kStore && NA > 0) {
    run_rows<NA>(a, [&](uint64_t b, float* p) {
      const uint64_t lrow = b + (threadIdx.x & 31u);
      if (lrow >= a.rows) return false;
      path(lrow, p);
      return true;
    });
  } else {
    // materialised rows, or the fused form for more than 4 assets (static,
    // one record of na assets per block)
    Kahan acc[CAP], acc2[CAP];
    for_rows(a.rows, out, [&](uint64_t lrow) {
      float p[CAP];
      path(lrow, p);
      if (!kStore)
        for (int i = 0; i < na; ++i) {
          acc[i].add(p[i]);
          acc2[i].add(p[i] * p[i]);
        }
    });
    if (!kStore)
      for (int i = 0; i < na; ++i)
        block_sum2_store((double)acc[i].value(), (double)acc2[i].value(),
                         a.partials + (2 * (uint64_t)blockIdx.x) * na + 2 * i);
  }
  if (err) atomicOr(a.err, err);
}

template <int kMode>
__global__ void __launch_bounds__(256, kMode != kFused ? kMatMinBlocks : kFusedMinBlocks) k_heston_euler_f32(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  PathOut<float, kMode> out;
  out.init(dyn_smem);
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  // FP32 constants rounded once on the host (F32K): converted here from the
  // double parameters, the register cap made the compiler redo the DMUL and
  // conversions inside the step loop (22 % of the FP64 pipe busy)
  const F32K& f = a.f32;
  const float rho = f.h_rho, rho_comp = f.h_rho_comp, kappa_dt = f.h_kdt;
  const float theta = f.h_theta, xi_sdt = f.h_xsdt, sdt = f.h_sdt;
  const float mu_dt = f.h_mudt, nhalf_dt = f.h_nhdt, s0 = f.h_s0;
  unsigned err = 0;
  auto path = [&](uint64_t lrow, float* pay) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    float v = f.h_v0;
    PathSum<kStore> lg;
    if (kMode == kRows) out.begin(a.out_f32 + lrow * (a.steps + 1));
    if (kStore) emit32(out, a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      float dw1 = normal_f32(s, c, zs, err);
      float dz = normal_f32(s, c, zs, err);
      float dw2 = fmaf(rho, dw1, rho_comp * dz);
      float v_plus = fmaxf(v, 0.0f);
      float sqrt_v = sqrt_approx(v_plus);
      v += fmaf(kappa_dt, theta - v_plus, xi_sdt * sqrt_v * dw2);
      lg.add(fmaf(nhalf_dt, v_plus, mu_dt) + sqrt_v * sdt * dw1);
      if (kStore) emit32(out, a, lrow, k, 1, 0, s0 * expf(lg.value()));
    }
    if (!kStore) pay[0] = payoff_f32(s0 * expf(lg.value()), a.f32.strike, a.payoff);
  };
  if constexpr (kStore) {
    for_rows(a.rows, out, [&](uint64_t lrow) { path(lrow, nullptr); });
  } else {
    run_rows<1>(a, [&](uint64_t b, float* p) {
      const uint64_t lrow = b + (threadIdx.x & 31u);
      if (lrow >= a.rows) return false;
      path(lrow, p);
      return true;
    });
  }
  if (err) atomicOr(a.err, err);
}

// Heston QE (heston.rs:89-174) in FP32: the same branches and the same draws
// as the FP64 form (a normal in the quadratic branch, one uniform in the
// exponential one, then the log-price normal), v in FP32 and the log price
// carried as a running sum with the reference's clamp to [-500, 500].  A
// branch decision psi <= 1.5 computed in FP32 can differ from FP64's for psi
// within ~1e-6 of 1.5; that path then draws differently from there on (a
// valid path of the same scheme), which is rare enough to stay inside the
// FP32 price bar.
template <int kMode>
__global__ void __launch_bounds__(256, kMode != kFused ? kMatMinBlocks : kFusedMinBlocks) k_heston_qe_f32(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  PathOut<float, kMode> out;
  out.init(dyn_smem);
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  unsigned err = 0;
  auto path = [&](uint64_t lrow, float* pay) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    float v = f.h_v0;
    PathSum<kStore> lg;
    lg.add(f.q_ls0);
    if (kMode == kRows) out.begin(a.out_f32 + lrow * (a.steps + 1));
    if (kStore) emit32(out, a, lrow, 0, 1, 0, f.h_s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      const float vp = fmaxf(v, 0.0f);
      const float m = fmaxf(fmaf(vp, f.q_ekdt, f.q_m0), 1e-15f);
      const float s2 = fmaf(vp, f.q_cs2, f.q_s2b);
      const float psi = s2 / (m * m);
      float vn;
      if (psi <= 1.5f) {  // quadratic branch: V ~ a (b + Z)^2
        const float ip = 2.0f / psi;
        const float b2 = fmaxf(ip - 1.0f + sqrtf(ip * (ip - 1.0f)), 0.0f);
        const float aa = m / (1.0f + b2);
        const float b = sqrtf(b2);
        const float z = normal_f32(s, c, zs, err);
        vn = aa * (b + z) * (b + z);
      } else {  // exponential branch: point mass at 0 and an exponential
        const float p = (psi - 1.0f) / (psi + 1.0f);
        const float beta = (1.0f - p) / m;
        const uint64_t mu = s.next() >> 11;  // next_f64 = mu 2^-53
        // 1 - u from the integer, so it is never rounded to 0
        const float one_m_u = __ull2float_rn((1ull << 53) - mu) * 0x1p-53f;
        vn = __ull2float_rn(mu) * 0x1p-53f <= p ? 0.0f : logf((1.0f - p) / one_m_u) / beta;
      }
      vn = fmaxf(vn, 0.0f);
      const float z1 = normal_f32(s, c, zs, err);
      const float var = fmaxf(fmaf(f.q_k3, vp, f.q_k4 * vn), 0.0f);
      lg.add(fmaf(sqrtf(var), z1, fmaf(f.q_k2, vn, fmaf(f.q_k1, vp, f.q_k0))));
      const float lv = lg.value();
      if (!(lv <= 500.0f && lv >= -500.0f)) {  // the reference's clamp of log S
        lg = PathSum<kStore>();
        lg.add(fminf(fmaxf(lv, -500.0f), 500.0f));
      }
      v = vn;
      if (kStore) emit32(out, a, lrow, k, 1, 0, expf(lg.value()));
    }
    if (!kStore) pay[0] = payoff_f32(expf(lg.value()), f.strike, a.payoff);
  };
  if constexpr (kStore) {
    for_rows(a.rows, out, [&](uint64_t lrow) { path(lrow, nullptr); });
  } else {
    run_rows<1>(a, [&](uint64_t b, float* p) {
      const uint64_t lrow = b + (threadIdx.x & 31u);
      if (lrow >= a.rows) return false;
      path(lrow, p);
      return true;
    });
  }
  if (err) atomicOr(a.err, err);
}

template <int kMode>
__global__ void __launch_bounds__(256, kMode != kFused ? kMatMinBlocks : kFusedMinBlocks) k_merton_f32(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  PathOut<float, kMode> out;
  out.init(dyn_smem);
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const MertonK& M = a.merton;
  // FP32 constants rounded once on the host (F32K), not converted here
  const float drift = a.f32.m_drift, diffusion = a.f32.m_diff, mu_j = a.f32.m_mu_j;
  const float sigma_j = a.f32.m_sigma_j, s0 = a.f32.m_s0;
  unsigned err = 0;
  auto path = [&](uint64_t lrow, float* pay) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    PathSum<kStore> w;
    float jumps = 0.0f, kf = 0.0f;
    if (kMode == kRows) out.begin(a.out_f32 + lrow * (a.steps + 1));
    if (kStore) emit32(out, a, lrow, 0, 1, 0, s0);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      w.add(normal_f32(s, c, zs, err));
      uint64_t u = s.next();
      if ((u >> 11) < M.jump_thr) jumps += fmaf(sigma_j, normal_f32(s, c, zs, err), mu_j);
      kf += 1.0f;
      if (kStore) emit32(out, a, lrow, k, 1, 0, s0 * expf(fmaf(kf, drift, diffusion * w.value()) + jumps));
    }
    if (!kStore)
      pay[0] = payoff_f32(s0 * expf(fmaf(diffusion, w.value(), a.f32.m_kdrift) + jumps), a.f32.strike, a.payoff);
  };
  if constexpr (kStore) {
    for_rows(a.rows, out, [&](uint64_t lrow) { path(lrow, nullptr); });
  } else {
    run_rows<1>(a, [&](uint64_t b, float* p) {
      const uint64_t lrow = b + (threadIdx.x & 31u);
      if (lrow >= a.rows) return false;
      path(lrow, p);
      return true;
    });
  }
  if (err) atomicOr(a.err, err);
}

// ------------------------------------------------------------ fused -------
// Fused pricing (payoff sums only) with ILP paths per thread in lockstep: the
// paths' generator steps are independent instruction chains (normal2_f32), so
// the issue slots fill from two streams per warp.  The block size, ILP and
// grid waves are chosen per model by the autotuner (set_fused_tune); every
// choice draws the same values for every path, only the grouping of the
// FP32 payoff partial sums (hence their last bits) changes with it.

template <int ILP>
__device__ __forceinline__ void normals(PcgGen* s, float* z, const SamplerCtx& c, const ZigShared& zs, unsigned& err) {
  if constexpr (ILP == 1)
    z[0] = normal_f32(s[0], c, zs, err);
  else
    normal2_f32(s[0], s[1], c, zs, err, z[0], z[1]);
}

// Rows l0 + j * nthreads (j < ILP) of one lockstep group; a row past the end
// runs on a copy of the first row's stream and contributes nothing.
template <int ILP>
__device__ __forceinline__ void group_rows(const PathLaunch& a, uint64_t l0, uint64_t nthreads, bool* ok, bool* neg,
                                           PcgGen* s) {
#pragma unroll
  for (int j = 0; j < ILP; ++j) {
    const uint64_t lrow = l0 + (uint64_t)j * nthreads;
    ok[j] = lrow < a.rows;
    const uint64_t row = a.row_begin + (ok[j] ? lrow : l0);
    neg[j] = row >= a.base_paths;
    s[j] = PcgGen{pcg_path_state(a.ss, neg[j] ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
  }
}

// Rows of a lockstep kernel: static groups of ILP rows l0 + j * nthreads
// (store_partials per block), or, with ILP 1 and a work queue, the queue's
// batches (run_rows).  group(l0, stride, ok, p) prices rows l0 + j * stride
// into p[j * NV + i] and flags the rows that exist.
template <int ILP, int NV, class Group>
__device__ __forceinline__ void lockstep_rows(const PathLaunch& a, Group&& group) {
  if constexpr (ILP == 1) {
    if (a.work) {
      run_rows<NV>(a, [&](uint64_t b, float* p) {
        const uint64_t lrow = b + (threadIdx.x & 31u);
        if (lrow >= a.rows) return false;
        bool ok[1];
        group(lrow, 0, ok, p);
        return ok[0];
      });
      return;
    }
  }
  Kahan acc[NV], acc2[NV];
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t l0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l0 < a.rows; l0 += nthreads * ILP) {
    bool ok[ILP];
    float p[ILP * NV];
    group(l0, nthreads, ok, p);
#pragma unroll
    for (int j = 0; j < ILP; ++j)
      if (ok[j]) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
          acc[i].add(p[j * NV + i]);
          acc2[i].add(p[j * NV + i] * p[j * NV + i]);
        }
      }
  }
  store_partials<NV>(a, acc, acc2);
}

template <int ILP>
__global__ void __launch_bounds__(256, ILP == 1 ? kFusedMinBlocks : 1) k_gbm_fused(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const float s0 = a.f32.g_s0, diffusion = a.f32.g_diff, kdrift = a.f32.g_kdrift, strike = a.f32.strike;
  lockstep_rows<ILP, 1>(a, [&](uint64_t l0, uint64_t stride, bool* ok, float* p) {
    bool neg[ILP];
    PcgGen s[ILP];
    Plain w[ILP];
    group_rows<ILP>(a, l0, stride, ok, neg, s);
#pragma unroll 1
    for (uint64_t k = 0; k < a.steps; ++k) {
      float z[ILP];
      normals<ILP>(s, z, c, zs, err);
#pragma unroll
      for (int j = 0; j < ILP; ++j) w[j].add(neg[j] ? -z[j] : z[j]);
    }
#pragma unroll
    for (int j = 0; j < ILP; ++j)
      if (ok[j]) p[j] = payoff_f32(s0 * expf(fmaf(diffusion, w[j].value(), kdrift)), strike, a.payoff);
  });
  if (err) atomicOr(a.err, err);
}

template <int ILP>
__global__ void __launch_bounds__(256, ILP == 1 ? kFusedMinBlocks : 1) k_heston_fused(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  const float rho = f.h_rho, rho_comp = f.h_rho_comp, kappa_dt = f.h_kdt, theta = f.h_theta;
  const float xi_sdt = f.h_xsdt, sdt = f.h_sdt, mu_dt = f.h_mudt, nhdt = f.h_nhdt, s0 = f.h_s0;
  unsigned err = 0;
  lockstep_rows<ILP, 1>(a, [&](uint64_t l0, uint64_t stride, bool* ok, float* p) {
    bool neg[ILP];
    PcgGen s[ILP];
    Plain lg[ILP];
    float v[ILP];
    group_rows<ILP>(a, l0, stride, ok, neg, s);
#pragma unroll
    for (int j = 0; j < ILP; ++j) v[j] = f.h_v0;
#pragma unroll 1
    for (uint64_t k = 0; k < a.steps; ++k) {
      float dw1[ILP], dz[ILP];
      normals<ILP>(s, dw1, c, zs, err);
      normals<ILP>(s, dz, c, zs, err);
#pragma unroll
      for (int j = 0; j < ILP; ++j) {
        const float dw2 = fmaf(rho, dw1[j], rho_comp * dz[j]);
        const float v_plus = fmaxf(v[j], 0.0f);
        const float sqrt_v = sqrt_approx(v_plus);
        v[j] += fmaf(kappa_dt, theta - v_plus, xi_sdt * sqrt_v * dw2);
        lg[j].add(fmaf(nhdt, v_plus, mu_dt) + sqrt_v * sdt * dw1[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < ILP; ++j)
      if (ok[j]) p[j] = payoff_f32(s0 * expf(lg[j].value()), f.strike, a.payoff);
  });
  if (err) atomicOr(a.err, err);
}

template <int ILP>
__global__ void __launch_bounds__(256, ILP == 1 ? kFusedMinBlocks : 1) k_merton_fused(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  const float diffusion = f.m_diff, kdrift = f.m_kdrift, mu_j = f.m_mu_j, sigma_j = f.m_sigma_j, s0 = f.m_s0;
  const uint64_t thr = a.merton.jump_thr;
  unsigned err = 0;
  lockstep_rows<ILP, 1>(a, [&](uint64_t l0, uint64_t stride, bool* ok, float* p) {
    bool neg[ILP];
    PcgGen s[ILP];
    Plain w[ILP];
    float jumps[ILP];
    group_rows<ILP>(a, l0, stride, ok, neg, s);
#pragma unroll
    for (int j = 0; j < ILP; ++j) jumps[j] = 0.0f;
#pragma unroll 1
    for (uint64_t k = 0; k < a.steps; ++k) {
      float z[ILP];
      normals<ILP>(s, z, c, zs, err);
#pragma unroll
      for (int j = 0; j < ILP; ++j) {
        w[j].add(z[j]);
        if ((s[j].next() >> 11) < thr) jumps[j] += fmaf(sigma_j, normal_f32(s[j], c, zs, err), mu_j);
      }
    }
#pragma unroll
    for (int j = 0; j < ILP; ++j)
      if (ok[j]) p[j] = payoff_f32(s0 * expf(fmaf(diffusion, w[j].value(), kdrift) + jumps[j]), f.strike, a.payoff);
  });
  if (err) atomicOr(a.err, err);
}

template <int NA, int ILP>
__global__ void __launch_bounds__(256, ILP == 1 ? kFusedMinBlocks : 1) k_multi_fused(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  unsigned err = 0;
  lockstep_rows<ILP, NA>(a, [&](uint64_t l0, uint64_t stride, bool* ok, float* p) {
    bool neg[ILP];
    PcgGen s[ILP];
    Plain w[ILP][NA];
    group_rows<ILP>(a, l0, stride, ok, neg, s);
#pragma unroll 1
    for (uint64_t k = 0; k < a.steps; ++k) {
#pragma unroll
      for (int i = 0; i < NA; ++i) {
        float z[ILP];
        normals<ILP>(s, z, c, zs, err);
#pragma unroll
        for (int j = 0; j < ILP; ++j) w[j][i].add(neg[j] ? -z[j] : z[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < ILP; ++j)
      if (ok[j]) {
#pragma unroll
        for (int i = 0; i < NA; ++i) {
          float eps = 0.0f;
#pragma unroll
          for (int m = 0; m <= i; ++m) eps = fmaf(f.a_L[i * kMaxAssets + m], w[j][m].value(), eps);
          p[j * NA + i] = payoff_f32(f.a_s0[i] * expf(fmaf(f.a_diff[i], eps, f.a_kdrift[i])), f.strike, a.payoff);
        }
      }
  });
  if (err) atomicOr(a.err, err);
}

// ------------------------------------------------ fused, warp-uniform -------
// The same fused pricing with the ziggurat fed one draw per iteration
// (ZigFeed): each iteration every lane of the warp takes one generator step
// and feeds it to its own sampler state; a lane that completes a normal hands
// it to the model.  A warp prices 32 consecutive rows together and iterates
// until all 32 have their normals (a lane that is done keeps stepping a
// stream nobody reads).  Draws and values per path are those of the kernels
// above; only the interleaving of lanes changes.

// Rows of one warp: base (warp-uniform) + lane.  A lane past the end runs on
// the first row's stream and contributes nothing.  The kernels draw with
// pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi), reading the stream increment from
// the launch parameters at every draw (the constant bank, not four registers
// of every lane).
struct WarpRow {
  bool ok, neg;
  DevPcg st;
};

__device__ __forceinline__ WarpRow warp_row(const PathLaunch& a, uint64_t base) {
  WarpRow r;
  const uint64_t lrow = base + (threadIdx.x & 31u);
  r.ok = lrow < a.rows;
  const uint64_t row = a.row_begin + (r.ok ? lrow : base);
  r.neg = row >= a.base_paths;
  r.st = pcg_path_state(a.ss, r.neg ? row - a.base_paths : row);
  return r;
}

// GBM (NA = 0) and multi-GBM with NA assets: only the per-asset sums of the
// normals matter.  The sum being filled is always w[0]; after each normal the
// sums rotate, so after steps * NA normals they are back in asset order.
template <int NA>
__global__ void __launch_bounds__(256, kUfMinBlocks) k_gbm_uf(const __grid_constant__ PathLaunch a) {
  constexpr int N = NA > 0 ? NA : 1;
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  unsigned err = 0;
  const uint32_t need_all = (uint32_t)a.steps * N, cap = uf_cap(need_all);
  run_rows<N>(a, [&](uint64_t base, float* pay) {
    WarpRow r = warp_row(a, base);
    Plain w[N];
    ZigFeed q;
    const uint32_t need = r.ok ? need_all : 0;
    uint32_t cnt = 0;
    uf_drive(cnt, need, cap, err, [&]() {
      float z;
      if (q.feed(pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z) & (cnt < need)) {
        w[0].add(z);  // the antithetic sign is applied to the sums
        ++cnt;
        if constexpr (N > 1) {
          const Plain t = w[0];
#pragma unroll
          for (int i = 0; i + 1 < N; ++i) w[i] = w[i + 1];
          w[N - 1] = t;
        }
      }
    });
    if (r.ok) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        float lg;
        float s0;
        if constexpr (NA == 0) {
          lg = fmaf(f.g_diff, r.neg ? -w[0].value() : w[0].value(), f.g_kdrift);
          s0 = f.g_s0;
        } else {
          float eps = 0.0f;
#pragma unroll
          for (int m = 0; m <= i; ++m)
            eps = fmaf(f.a_L[i * kMaxAssets + m], r.neg ? -w[m].value() : w[m].value(), eps);
          lg = fmaf(f.a_diff[i], eps, f.a_kdrift[i]);
          s0 = f.a_s0[i];
        }
        pay[i] = payoff_f32(s0 * expf(lg), f.strike, a.payoff);
      }
    }
    return r.ok;
  });
  if (err) atomicOr(a.err, err);
}

// Heston (Euler): normals pair up as (dw1, dz) of one step.  Each call feeds
// two draws, and at most one step completes per call: the lane's phase (half:
// a dw1 is carried from an earlier call) picks the step's two normals from
// the carried one and this call's.  Lanes drift out of phase after rejected
// attempts; with one draw a call the step's arithmetic issued for the warp in
// almost every call (85 warp instructions a draw on GB300), with two it issues
// once per two draws.
__global__ void __launch_bounds__(256, kUfMinBlocks) k_heston_uf(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  const float rho = f.h_rho, rho_comp = f.h_rho_comp, kappa_dt = f.h_kdt, theta = f.h_theta;
  const float xi_sdt = f.h_xsdt, sdt = f.h_sdt, mu_dt = f.h_mudt, nhdt = f.h_nhdt;
  unsigned err = 0;
  const uint32_t cap = uf_cap(2 * (uint32_t)a.steps);
  run_rows<1>(a, [&](uint64_t base, float* pay) {
    WarpRow r = warp_row(a, base);
    ZigFeed q;
    Plain lg;
    float v = f.h_v0, zc = 0.0f;
    bool half = false;
    const uint32_t need = r.ok ? (uint32_t)a.steps : 0;
    uint32_t cnt = 0;
    uf_drive<kUfUnroll / 2>(cnt, need, cap, err, [&]() {
      float z1, z2;
      const bool a1 = q.feed(pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z1);
      const bool a2 = q.feed(pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z2);
      const float first = a1 ? z1 : z2;
      const bool two = a1 & a2, one = a1 ^ a2;
      const bool step = half ? (a1 | a2) : two;
      const float dw1 = half ? zc : z1;
      const float dz = half ? first : z2;
      if (half) {
        if (two) zc = z2;
      } else if (one) {
        zc = first;
      }
      half ^= one;
      if (step & (cnt < need)) {
        const float dw2 = fmaf(rho, dw1, rho_comp * dz);
        const float v_plus = fmaxf(v, 0.0f);
        const float sqrt_v = sqrt_approx(v_plus);
        v += fmaf(kappa_dt, theta - v_plus, xi_sdt * sqrt_v * dw2);
        lg.add(fmaf(nhdt, v_plus, mu_dt) + sqrt_v * sdt * dw1);
        ++cnt;
      }
    });
    if (r.ok) pay[0] = payoff_f32(f.h_s0 * expf(lg.value()), f.strike, a.payoff);
    return r.ok;
  });
  if (err) atomicOr(a.err, err);
}

// Merton: after the diffusion normal of a step the lane takes the jump
// uniform at once (a second generator step in the same iteration); on a jump
// its next normal is the jump size.
__global__ void __launch_bounds__(256, kUfMinBlocks) k_merton_uf(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  const float mu_j = f.m_mu_j, sigma_j = f.m_sigma_j;
  const uint64_t thr = a.merton.jump_thr;
  unsigned err = 0;
  const uint32_t cap = uf_cap(2 * (uint32_t)a.steps);
  run_rows<1>(a, [&](uint64_t base, float* pay) {
    WarpRow r = warp_row(a, base);
    ZigFeed q;
    Plain w;
    float jumps = 0.0f;
    bool in_jump = false;
    const uint32_t need = r.ok ? (uint32_t)a.steps : 0;
    uint32_t cnt = 0;
    uf_drive(cnt, need, cap, err, [&]() {
      float z;
      if (q.feed(pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z) & (cnt < need)) {
        if (in_jump) {
          jumps += fmaf(sigma_j, z, mu_j);
          in_jump = false;
          ++cnt;
        } else {
          w.add(z);
          if ((pcg_next(r.st, a.ss.inc_lo, a.ss.inc_hi) >> 11) < thr)
            in_jump = true;
          else
            ++cnt;
        }
      }
    });
    if (r.ok) pay[0] = payoff_f32(f.m_s0 * expf(fmaf(f.m_diff, w.value(), f.m_kdrift) + jumps), f.strike, a.payoff);
    return r.ok;
  });
  if (err) atomicOr(a.err, err);
}

// ------------------------------------- materialised rows, warp-uniform -----
// Heston (Euler) and Merton paths written row by row through the staged
// sector writer, on the warp-uniform sampler feed.  A step completes at most
// once a call (Heston: two draws a call, the step's normals picked by the
// lane's phase; Merton: the jump uniform in the diffusion normal's call), and
// its arithmetic and compensated sums are those of k_heston_euler_f32 and
// k_merton_f32, so the rows are the same floats.  Lanes drift out of phase
// after rejected attempts, so each lane puts its values as its steps complete
// (the writer keeps a ring per lane); the warp ends its 32 rows together.
__global__ void __launch_bounds__(256, kMatMinBlocks) k_heston_rows_uf(const __grid_constant__ PathLaunch a) {
  PathOut<float, kRows> out;
  out.init(dyn_smem);
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const F32K& f = a.f32;
  const float rho = f.h_rho, rho_comp = f.h_rho_comp, kappa_dt = f.h_kdt;
  const float theta = f.h_theta, xi_sdt = f.h_xsdt, sdt = f.h_sdt;
  const float mu_dt = f.h_mudt, nhalf_dt = f.h_nhdt, s0 = f.h_s0;
  unsigned err = 0;
  for_rows_warp(a.rows, out, [&](uint64_t lrow, bool on) {
    DevPcg st = pcg_path_state(a.ss, a.row_begin + lrow);
    ZigFeed q;
    float v = f.h_v0, zc = 0.0f;
    Kahan lg;
    bool half = false;
    if (on) {
      out.begin(a.out_f32 + lrow * (a.steps + 1));
      out.rs.put(s0);
    }
    const uint32_t need = on ? (uint32_t)a.steps : 0u;
    uint32_t cnt = 0;
    uf_drive<kUfUnroll / 2>(cnt, need, uf_cap(2 * a.steps), err, [&]() {
      float z1, z2;
      const bool a1 = q.feed(pcg_next(st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z1);
      const bool a2 = q.feed(pcg_next(st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z2);
      const float first = a1 ? z1 : z2;
      const bool two = a1 & a2, one = a1 ^ a2;
      const bool step = half ? (a1 | a2) : two;
      const float dw1 = half ? zc : z1;
      const float dz = half ? first : z2;
      if (half) {
        if (two) zc = z2;
      } else if (one) {
        zc = first;
      }
      half ^= one;
      if (step & (cnt < need)) {
        const float dw2 = fmaf(rho, dw1, rho_comp * dz);
        const float v_plus = fmaxf(v, 0.0f);
        const float sqrt_v = sqrt_approx(v_plus);
        v += fmaf(kappa_dt, theta - v_plus, xi_sdt * sqrt_v * dw2);
        lg.add(fmaf(nhalf_dt, v_plus, mu_dt) + sqrt_v * sdt * dw1);
        out.rs.put(s0 * expf(lg.value()));
        ++cnt;
      }
    });
  });
  if (err) atomicOr(a.err, err);
}

__global__ void __launch_bounds__(256, kMatMinBlocks) k_merton_rows_uf(const __grid_constant__ PathLaunch a) {
  PathOut<float, kRows> out;
  out.init(dyn_smem);
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const uint64_t thr = a.merton.jump_thr;
  const float drift = a.f32.m_drift, diffusion = a.f32.m_diff, mu_j = a.f32.m_mu_j;
  const float sigma_j = a.f32.m_sigma_j, s0 = a.f32.m_s0;
  unsigned err = 0;
  for_rows_warp(a.rows, out, [&](uint64_t lrow, bool on) {
    DevPcg st = pcg_path_state(a.ss, a.row_begin + lrow);
    ZigFeed q;
    Kahan w;
    float jumps = 0.0f, kf = 0.0f;
    bool in_jump = false;
    if (on) {
      out.begin(a.out_f32 + lrow * (a.steps + 1));
      out.rs.put(s0);
    }
    const uint32_t need = on ? (uint32_t)a.steps : 0u;
    uint32_t cnt = 0;
    uf_drive(cnt, need, uf_cap(2 * a.steps), err, [&]() {
      float z;
      if (q.feed(pcg_next(st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z) & (cnt < need)) {
        bool done = true;
        if (in_jump) {
          jumps += fmaf(sigma_j, z, mu_j);
          in_jump = false;
        } else {
          w.add(z);
          if ((pcg_next(st, a.ss.inc_lo, a.ss.inc_hi) >> 11) < thr) {
            in_jump = true;
            done = false;
          }
        }
        if (done) {
          kf += 1.0f;
          out.rs.put(s0 * expf(fmaf(kf, drift, diffusion * w.value()) + jumps));
          ++cnt;
        }
      }
    });
  });
  if (err) atomicOr(a.err, err);
}

// Materialised rows of Heston Euler and Merton go to the warp-uniform kernels
// (their counts are 32-bit).
inline bool rows_uf(const PathLaunch& L) {
  return L.steps < (1ull << 31) && (L.model == kMerton || (L.model == kHeston && L.heston.scheme == 0));
}

// Tuning table: per model kind (gbm, heston, merton, multi-GBM with 1..4
// assets) the block size, ILP, grid waves and kernel form of the fused
// launch.  Default: the warp-uniform form (ZigFeed), 256 threads, 2 waves,
// which the autotuner picks for all three models of the 1e6 x 252 workload on
// GB300 (the shapes it prefers for the other block sizes and waves lie within
// about 1 % of it).
FusedTune g_tune[kTuneSlots] = {{256, 1, 2, 2}, {256, 1, 2, 2}, {256, 1, 2, 2}, {256, 1, 2, 2},
                                {256, 1, 2, 2}, {256, 1, 2, 2}, {256, 1, 2, 2}};

const void* fused_kernel(int slot, int ilp, int variant) {
  if (variant == 0) {  // the per-path loop kernels (one path per thread at a time)
    switch (slot) {
      case 0: return (const void*)k_gbm_f32<kFused>;
      case 1: return (const void*)k_heston_euler_f32<kFused>;
      case 2: return (const void*)k_merton_f32<kFused>;
      case 3: return (const void*)k_multi_gbm_f32<1, kFused>;
      case 4: return (const void*)k_multi_gbm_f32<2, kFused>;
      case 5: return (const void*)k_multi_gbm_f32<3, kFused>;
      default: return (const void*)k_multi_gbm_f32<4, kFused>;
    }
  }
  if (variant == 2) {  // warp-uniform sampler feed (one path per thread)
    switch (slot) {
      case 0: return (const void*)k_gbm_uf<0>;
      case 1: return (const void*)k_heston_uf;
      case 2: return (const void*)k_merton_uf;
      case 3: return (const void*)k_gbm_uf<1>;
      case 4: return (const void*)k_gbm_uf<2>;
      case 5: return (const void*)k_gbm_uf<3>;
      default: return (const void*)k_gbm_uf<4>;
    }
  }
  const bool two = ilp == 2;
  switch (slot) {
    case 0: return two ? (const void*)k_gbm_fused<2> : (const void*)k_gbm_fused<1>;
    case 1: return two ? (const void*)k_heston_fused<2> : (const void*)k_heston_fused<1>;
    case 2: return two ? (const void*)k_merton_fused<2> : (const void*)k_merton_fused<1>;
    case 3: return two ? (const void*)k_multi_fused<1, 2> : (const void*)k_multi_fused<1, 1>;
    case 4: return two ? (const void*)k_multi_fused<2, 2> : (const void*)k_multi_fused<2, 1>;
    case 5: return two ? (const void*)k_multi_fused<3, 2> : (const void*)k_multi_fused<3, 1>;
    default: return two ? (const void*)k_multi_fused<4, 2> : (const void*)k_multi_fused<4, 1>;
  }
}

template <int kMode>
void launch_multi32(const PathLaunch& L, dim3 g, dim3 b, size_t sm, cudaStream_t st) {
  switch (L.multi.na) {
    case 1: k_multi_gbm_f32<1, kMode><<<g, b, sm, st>>>(L); break;
    case 2: k_multi_gbm_f32<2, kMode><<<g, b, sm, st>>>(L); break;
    case 3: k_multi_gbm_f32<3, kMode><<<g, b, sm, st>>>(L); break;
    case 4: k_multi_gbm_f32<4, kMode><<<g, b, sm, st>>>(L); break;
    default: k_multi_gbm_f32<0, kMode><<<g, b, sm, st>>>(L); break;
  }
}

// The untuned kernel of L's model in store mode kMode (occupancy query).
template <int kMode>
const void* model_kernel32(const PathLaunch& L) {
  if constexpr (kMode == kRows) {
    if (rows_uf(L)) return L.model == kMerton ? (const void*)k_merton_rows_uf : (const void*)k_heston_rows_uf;
  }
  switch (L.model) {
    case kGbm: return (const void*)k_gbm_f32<kMode>;
    case kHeston:
      return L.heston.scheme != 0 ? (const void*)k_heston_qe_f32<kMode> : (const void*)k_heston_euler_f32<kMode>;
    case kMerton: return (const void*)k_merton_f32<kMode>;
    default: return (const void*)k_multi_gbm_f32<3, kMode>;
  }
}

template <int kMode>
int launch_model32(const PathLaunch& L, dim3 G, dim3 B, size_t sm, cudaStream_t st) {
  if constexpr (kMode == kRows) {
    if (rows_uf(L)) {
      if (L.model == kMerton)
        k_merton_rows_uf<<<G, B, sm, st>>>(L);
      else
        k_heston_rows_uf<<<G, B, sm, st>>>(L);
      return 0;
    }
  }
  switch (L.model) {
    case kGbm: k_gbm_f32<kMode><<<G, B, sm, st>>>(L); break;
    case kHeston:
      if (L.heston.scheme != 0)
        k_heston_qe_f32<kMode><<<G, B, sm, st>>>(L);
      else
        k_heston_euler_f32<kMode><<<G, B, sm, st>>>(L);
      break;
    case kMerton: k_merton_f32<kMode><<<G, B, sm, st>>>(L); break;
    case kMultiGbm: launch_multi32<kMode>(L, G, B, sm, st); break;
    default: return -1;
  }
  return 0;
}

// Diagnostic: the error of the hardware logarithm (__logf) over every
// normal float x in (0, 1), against log(x) in FP64: out[0] the largest
// absolute error for x in [0.5, 1), out[1] the largest relative error for
// x < 0.5 (float bits of non-negative values order like the values).  The
// ziggurat tail test's FP32 margin is derived from these bounds.
__global__ void __launch_bounds__(256) k_debug_logf_scan(unsigned* out) {
  float a_max = 0.0f, r_max = 0.0f;
  const uint32_t lo = 0x00800000u, hi = 0x3F800000u;  // [min normal, 1.0)
  for (uint32_t b = lo + blockIdx.x * blockDim.x + threadIdx.x; b < hi; b += gridDim.x * blockDim.x) {
    const float x = __uint_as_float(b);
    const double d = (double)__logf(x) - log((double)x);
    if (x >= 0.5f)
      a_max = fmaxf(a_max, (float)fabs(d));
    else
      r_max = fmaxf(r_max, (float)(fabs(d) / -log((double)x)));
  }
  atomicMax(out, __float_as_uint(a_max));
  atomicMax(out + 1, __float_as_uint(r_max));
}

}  // namespace

int tune_slot(int model, int na) {
  if (model == kMultiGbm) return na >= 1 && na <= 4 ? 2 + na : -1;
  return model == kGbm ? 0 : model == kHeston ? 1 : model == kMerton ? 2 : -1;
}

FusedTune get_fused_tune(int slot) {
  return slot >= 0 && slot < kTuneSlots ? g_tune[slot] : FusedTune{256, 1, 2, 2};
}

int set_fused_tune(int slot, FusedTune t) {
  if (slot < 0 || slot >= kTuneSlots) return -1;
  if ((t.block != 64 && t.block != 128 && t.block != 256) || (t.ilp != 1 && t.ilp != 2) || t.waves < 1 ||
      t.waves > 2 || t.variant < 0 || t.variant > 2 || (t.variant != 1 && t.ilp != 1))
    return -1;
  g_tune[slot] = t;
  return 0;
}

int launch_paths_f32(const PathLaunch& L, cudaStream_t st) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const bool store = L.out_f32 != nullptr;
  const int slot = tune_slot(L.model, L.multi.na);
  if (!store && slot >= 0 && !(L.model == kHeston && L.heston.scheme != 0)) {
    // fused pricing: tuned block size, ILP and waves of resident blocks
    const FusedTune t = g_tune[slot];
    // the warp-uniform form counts normals in 32 bits
    const int variant = t.variant == 2 && L.steps >= (1ull << 22) ? 0 : t.variant;
    const void* fn = fused_kernel(slot, t.ilp, variant);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.block, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    uint64_t g = (L.rows + (uint64_t)t.block * t.ilp - 1) / ((uint64_t)t.block * t.ilp);
    const uint64_t cap = (uint64_t)sms * per_sm * t.waves;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    // every form but the two-path lockstep one takes its rows from the work
    // queue when the caller supplies one
    PathLaunch Lq = L;
    const bool queue = L.work != nullptr && !(variant == 1 && t.ilp == 2) && L.batch_rows >= 32 &&
                       L.batch_rows % 32 == 0;
    if (!queue) Lq.work = nullptr;
    const uint64_t records = queue ? (L.rows + L.batch_rows - 1) / L.batch_rows : g;
    if (L.max_records && records > L.max_records) return kRecordsExceeded;
    if (queue && cudaMemsetAsync(L.work, 0, sizeof(unsigned long long), st) != cudaSuccess) return -1;
    void* args[] = {(void*)&Lq};
    if (cudaLaunchKernel(fn, dim3((unsigned)g), dim3(t.block), args, 0, st) != cudaSuccess) return -1;
    return (int)records;
  }
  PathLaunch Ls = L;  // the untuned kernels below run static rows
  Ls.work = nullptr;
  const int b = 256;
  const int mode = !store ? kFused : row_store_fits(L, sizeof(float)) ? kRows : kElems;
  const size_t sm = mode == kRows ? RowStore<float>::bytes((uint32_t)b) : 0;
  // Persistent grid: exactly the blocks that are resident at once, so the
  // grid-stride loop gives every thread the same number of paths (+-1) in a
  // single wave instead of a partial second wave of blocks.
  const void* fn = mode == kRows ? model_kernel32<kRows>(L) : mode == kElems ? model_kernel32<kElems>(L)
                                                                             : model_kernel32<kFused>(L);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, b, sm) != cudaSuccess || per_sm < 1) per_sm = 2;
  uint64_t g = (L.rows + b - 1) / b;
  const uint64_t cap = (uint64_t)sms * per_sm;
  if (g > cap && !L.flat_grid) g = cap;
  if (g < 1) g = 1;
  if (!store && L.max_records && g > L.max_records) return kRecordsExceeded;
  dim3 G((unsigned)g), B(b);
  const int rc = mode == kRows ? launch_model32<kRows>(Ls, G, B, sm, st)
                 : mode == kElems ? launch_model32<kElems>(Ls, G, B, 0, st)
                                  : launch_model32<kFused>(Ls, G, B, 0, st);
  if (rc < 0) return -1;
  return cudaPeekAtLastError() == cudaSuccess ? (int)g : -1;
}

// Diagnostic: the two FP32 sampler forms on the same streams (stream i:
// path i of the launch's StreamSpec).  Form 0 calls normal_f32 n times per
// thread; form 1 runs ZigFeed warp-uniformly (32 consecutive streams a warp)
// and records a stream's generator state when its n-th normal completes.  Both
// must give the same values and states bit for bit.
__global__ void __launch_bounds__(256) k_debug_zigfeed(const __grid_constant__ DebugZig a) {
  __shared__ ZigShared zs;
  __shared__ ZigShared32 zs32;
  zig_stage(zs, a.tabs, false);
  zig_stage32(zs32, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wb < a.n_paths; wb += nthreads) {
    const uint64_t i = wb + (threadIdx.x & 31u);
    const bool ok = i < a.n_paths;
    DevPcg st = pcg_path_state(a.ss, ok ? i : wb);
    float* out = a.out + (ok ? i : 0) * a.n;
    if (a.form == 0) {
      if (ok) {
        PcgGen g{st, a.ss.inc_lo, a.ss.inc_hi};
        for (uint32_t k = 0; k < a.n; ++k) out[k] = normal_f32(g, c, zs, err);
        a.state[2 * i] = g.s.lo;
        a.state[2 * i + 1] = g.s.hi;
      }
    } else {
      ZigFeed q;
      const uint32_t need = ok ? a.n : 0u;
      uint32_t cnt = 0;
      uf_drive(cnt, need, uf_cap(a.n), err, [&]() {
        float z;
        if (q.feed(pcg_next(st, a.ss.inc_lo, a.ss.inc_hi), zs32, c, z) & (cnt < need)) {
          out[cnt] = z;
          if (++cnt == need) {
            a.state[2 * i] = st.lo;
            a.state[2 * i + 1] = st.hi;
          }
        }
      });
    }
  }
  if (err) atomicOr(a.err, err);
}

void launch_debug_zigfeed(const DebugZig& a, cudaStream_t st) {
  if (a.n_paths) k_debug_zigfeed<<<(unsigned)std::min<uint64_t>((a.n_paths + 255) / 256, 4096), 256, 0, st>>>(a);
}

void launch_debug_logf_scan(unsigned* out, cudaStream_t st) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_debug_logf_scan<<<sms * 8, 256, 0, st>>>(out);
}

}  // namespace stocha
