// FP64 path kernels: the reference's own discretisation of each model with
// its exact operation order (this translation unit is built with
// --fmad=false, so no a*b+c is contracted, as in Rust).  Each thread owns one
// output row: it derives the row's stream by jump-ahead (gbm.rs:58-59) and
// runs the model recurrence, either storing every step (materialised) or
// reducing the terminal value to a call/put payoff in registers (fused).
//
//   GBM          src/finance/gbm.rs:42-107
//   multi-GBM    src/finance/multi_gbm.rs:22-113
//   Heston       src/finance/heston.rs:44-87 (Euler), :89-174 (QE)
//   Merton       src/finance/jump_diffusion.rs:48-105
#include <cuda_runtime.h>

#include "engine.h"
#include "mc_device.cuh"
#include "reduce.cuh"
#include "row_store.cuh"

namespace stocha {
namespace {

// Staging area of the row-major stores: RowStore<double>::bytes(blockDim.x)
// bytes, passed at launch in the kRows mode.
extern __shared__ __align__(16) unsigned char dyn_smem[];

__device__ __forceinline__ double payoff_f64(double s, double k, int kind) {
  return kind == kCall ? fmax(s - k, 0.0) : fmax(k - s, 0.0);
}

// Payoff of a fused launch, including the pathwise estimators of
// greeks.rs:387-418 with the reference's expression order.
__device__ __forceinline__ double launch_payoff(const PathLaunch& a, double s) {
  const double k = a.strike;
  switch (a.payoff) {
    case kCall:
    case kPut:
      return payoff_f64(s, k, a.payoff);
    case kPwDeltaCall:
      return s > k ? 1.0 * s / a.aux[0] : 0.0;
    case kPwDeltaPut:
      return s < k ? -1.0 * s / a.aux[0] : 0.0;
    default: {
      const bool call = a.payoff == kPwVegaCall;
      if (call ? !(s > k) : !(s < k)) return 0.0;
      const double s0 = a.aux[0], r = a.aux[1], sigma = a.aux[2], t = a.aux[3];
      const double log_return = log(s / s0);
      return (call ? 1.0 : -1.0) * s * (log_return - (r + 0.5 * sigma * sigma) * t) / sigma;
    }
  }
}

// Row-major (or time-major) store of one path value.
__device__ __forceinline__ void store64(const PathLaunch& a, uint64_t lrow, uint64_t step, uint64_t width,
                                        uint64_t col, double v) {
  if (a.terminal_only) {
    if (step == a.steps) a.out_f64[lrow * width + col] = v;
    return;
  }
  if (a.time_major)
    a.out_f64[(step * width + col) * a.rows + lrow] = v;
  else
    a.out_f64[(lrow * (a.steps + 1) + step) * width + col] = v;
}

template <int kMode>
using Out64 = PathOut<double, kMode>;

template <int kMode>
__device__ __forceinline__ void emit64(Out64<kMode>& out, const PathLaunch& a, uint64_t lrow, uint64_t step,
                                       uint64_t width, uint64_t col, double v) {
  if (kMode == kRows)
    out.rs.put(v);
  else if (kMode == kElems)
    store64(a, lrow, step, width, col, v);
}

template <int kMode>
__global__ void __launch_bounds__(128) k_gbm_f64(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  double acc = 0.0, acc2 = 0.0;
  Out64<kMode> out;
  out.init(dyn_smem);
  for_rows(a.rows, out, [&](uint64_t lrow) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    // the antithetic path's -z enters only through diffusion * z, so the sign
    // goes on the coefficient once per path (exact: IEEE products are odd)
    const double drift = a.gbm.drift, diffusion = neg ? -a.gbm.diffusion : a.gbm.diffusion;
    double x = a.gbm.s0;
    if (kMode == kRows) out.begin(a.out_f64 + lrow * (a.steps + 1));
    if (kStore) emit64(out, a, lrow, 0, 1, 0, x);
    // Two steps at a time: both draws, then both exponentials (independent
    // chains the compiler interleaves), then the two dependent products.  At
    // small path counts a warp's step is latency-bound on the exponential's
    // chain; the values are those of the one-step loop.
    uint64_t k = 1;
#pragma unroll 1
    for (; k + 1 <= a.steps; k += 2) {
      const double z0 = normal_f64<false, true>(s, c, zs, err);
      const double z1 = normal_f64<false, true>(s, c, zs, err);
      const double y0 = exp_y(fma(diffusion, z0, drift), zs);
      const double y1 = exp_y(fma(diffusion, z1, drift), zs);
      x *= y0;
      if (kStore) emit64(out, a, lrow, k, 1, 0, x);
      x *= y1;
      if (kStore) emit64(out, a, lrow, k + 1, 1, 0, x);
    }
    if (k <= a.steps) {
      const double z = normal_f64<false, true>(s, c, zs, err);
      x = mul_exp(x, fma(diffusion, z, drift), zs);
      if (kStore) emit64(out, a, lrow, k, 1, 0, x);
    }
    if (!kStore) {
      double p = launch_payoff(a, x);
      acc += p;
      acc2 += p * p;
    }
  });
  if (!kStore) block_sum2_store(acc, acc2, a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

template <int NA, int kMode>
__global__ void __launch_bounds__(128) k_multi_gbm_f64(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const int na = NA > 0 ? NA : a.multi.na;
  unsigned err = 0;
  double acc[NA > 0 ? NA : kMaxAssets], acc2[NA > 0 ? NA : kMaxAssets];
  for (int i = 0; i < na; ++i) acc[i] = acc2[i] = 0.0;
  Out64<kMode> out;
  out.init(dyn_smem);
  for_rows(a.rows, out, [&](uint64_t lrow) {
    const uint64_t row = a.row_begin + lrow;
    const bool neg = row >= a.base_paths;
    PcgGen s{pcg_path_state(a.ss, neg ? row - a.base_paths : row), a.ss.inc_lo, a.ss.inc_hi};
    double sv[NA > 0 ? NA : kMaxAssets], z[NA > 0 ? NA : kMaxAssets];
    // the antithetic path's -z as a sign flip of each normal (integer XOR, exact)
    const long long zsgn = neg ? (long long)(1ull << 63) : 0ll;
    if (kMode == kRows) out.begin(a.out_f64 + lrow * (a.steps + 1) * na);
#pragma unroll
    for (int i = 0; i < na; ++i) {
      sv[i] = a.multi.s0[i];
      if (kStore) emit64(out, a, lrow, 0, na, i, sv[i]);
    }
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      // the normals' products by DMUL: with its exponent rows folded (below)
      // this kernel is bound by issue and the ALU pipe, not by the FP64 pipe
      // (49 %), so one DMUL is cheaper than the integer-pipe product
#pragma unroll
      for (int i = 0; i < na; ++i)
        z[i] = __longlong_as_double(__double_as_longlong(normal_f64<false, true>(s, c, zs, err)) ^ zsgn);
#pragma unroll
      for (int i = 0; i < na; ++i) {
        // exponent drift_i + diffusion_i (L z)_i as one DFMA chain over row i of
        // diffusion_i L, started from the drift: i + 1 FP64 operations where
        // the row sum and its scaling took i + 2 (the roundings move by an
        // ulp or so of the exponent, ~1e-18 of the price per step)
        double t = fma(a.multi.LD[i * kMaxAssets], z[0], a.multi.drift[i]);
#pragma unroll
        for (int m = 1; m <= i; ++m) t = fma(a.multi.LD[i * kMaxAssets + m], z[m], t);
        sv[i] = mul_exp(sv[i], t, zs);
        if (kStore) emit64(out, a, lrow, k, na, i, sv[i]);
      }
    }
    if (!kStore) {
#pragma unroll
      for (int i = 0; i < na; ++i) {
        double p = launch_payoff(a, sv[i]);
        acc[i] += p;
        acc2[i] += p * p;
      }
    }
  });
  if (!kStore) {
    for (int i = 0; i < na; ++i) block_sum2_store(acc[i], acc2[i], a.partials + (2 * (uint64_t)blockIdx.x) * na + 2 * i);
  }
  if (err) atomicOr(a.err, err);
}

template <int kMode>
__global__ void __launch_bounds__(128) k_heston_f64(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const HestonK& h = a.heston;
  unsigned err = 0;
  double acc = 0.0, acc2 = 0.0;
  Out64<kMode> out;
  out.init(dyn_smem);
  for_rows(a.rows, out, [&](uint64_t lrow) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    double x = h.s0, v = h.v0;
    if (kMode == kRows) out.begin(a.out_f64 + lrow * (a.steps + 1));
    if (kStore) emit64(out, a, lrow, 0, 1, 0, x);
    if (h.scheme == 0) {
      const double mu_dt = h.mu * h.dt, nhalf_dt = -0.5 * h.dt;
#pragma unroll 1
      for (uint64_t k = 1; k <= a.steps; ++k) {
        const double dw1 = normal_f64<true, true>(s, c, zs, err);  // FP64-pipe bound: integer products
        const double dz = normal_f64<true, true>(s, c, zs, err);
        const double v_plus = max0_int(v);
        // w = sqrt(v+ dt) serves both updates; sqrt(v+) is the correctly
        // rounded one, on the integer pipes
        const double w = sqrt_rn_int(v_plus) * h.sqrt_dt;
        // v += kappa (theta - v+) dt + xi sqrt(v+ dt) dW2 with dW2 = rho dW1 +
        // sqrt(1 - rho^2) dZ (heston.rs:59-70), with xi rho, xi sqrt(1 - rho^2)
        // and kappa dt formed on the host and the sums fused: 6 FP64 operations
        // instead of the reference's 11, the same quantities up to an ulp or
        // two of each term.  max(v, 0) is continuous, so such an ulp moves the
        // path by ~1e-15; only a v within ~1e-17 of zero could split a path
        // from the reference's (about 1e-16 per path-step)
        const double xdw2 = fma(h.xi_rho, dw1, h.xi_rho_comp * dz);
        v = fma(h.kdt, h.theta - v_plus, fma(w, xdw2, v));
        // the log-price increment (mu - v+/2) dt + sqrt(v+ dt) dW1, fused
        x = mul_exp(x, fma(w, dw1, fma(nhalf_dt, v_plus, mu_dt)), zs);
        if (kStore) emit64(out, a, lrow, k, 1, 0, x);
      }
    } else {
#pragma unroll 1
      for (uint64_t k = 1; k <= a.steps; ++k) {
        double v_plus = fmax(v, 0.0);
        double m = h.qe_m0 + v_plus * h.e_kdt;
        m = fmax(m, 1e-15);
        double s2 = v_plus * h.xi * h.xi * h.e_kdt * h.one_m_ekdt / h.kappa + h.qe_s2b;
        double psi = s2 / (m * m);
        double v_next;
        if (psi <= 1.5) {
          double b2 = 2.0 / psi - 1.0 + sqrt(2.0 / psi * (2.0 / psi - 1.0));
          b2 = fmax(b2, 0.0);
          double aa = m / (1.0 + b2);
          double b = sqrt(b2);
          double z = normal_f64<false, true>(s, c, zs, err);
          v_next = aa * (b + z) * (b + z);
        } else {
          double p = (psi - 1.0) / (psi + 1.0);
          double beta = (1.0 - p) / m;
          double u = u64_to_unit_f64(s.next());
          v_next = (u <= p) ? 0.0 : log((1.0 - p) / (1.0 - u)) / beta;
        }
        v_next = fmax(v_next, 0.0);
        double z1 = normal_f64<false, true>(s, c, zs, err);
        double var_term = fmax(h.k3_s * v_plus + h.k4_s * v_next, 0.0);
        double log_s = log(x) + h.k0_s + h.k1_s * v_plus + h.k2_s * v_next + sqrt(var_term) * z1;
        x = exp(fmin(fmax(log_s, -500.0), 500.0));
        v = v_next;
        if (kStore) emit64(out, a, lrow, k, 1, 0, x);
      }
    }
    if (!kStore) {
      double p = launch_payoff(a, x);
      acc += p;
      acc2 += p * p;
    }
  });
  if (!kStore) block_sum2_store(acc, acc2, a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

// 9 resident blocks in the store modes (56 registers): 2.856 -> 2.815 ms at
// 1e6 x 252 materialised on GB300 (the same cap made multi-GBM slower).
template <int kMode>
__global__ void __launch_bounds__(128, kMode == kFused ? 1 : 9) k_merton_f64(const __grid_constant__ PathLaunch a) {
  constexpr bool kStore = kMode != kFused;
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const MertonK& M = a.merton;
  unsigned err = 0;
  double acc = 0.0, acc2 = 0.0;
  Out64<kMode> out;
  out.init(dyn_smem);
  for_rows(a.rows, out, [&](uint64_t lrow) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    double x = M.s0;
    if (kMode == kRows) out.begin(a.out_f64 + lrow * (a.steps + 1));
    if (kStore) emit64(out, a, lrow, 0, 1, 0, x);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      const double z = normal_f64<false, true>(s, c, zs, err);
      double ret = fma(M.diffusion, z, M.drift);
      const uint64_t u = s.next();
      if ((u >> 11) < M.jump_thr) {  // the reference adds a zero jump return otherwise
        const double z_j = normal_f64<false, true>(s, c, zs, err);
        ret += fma(M.sigma_j, z_j, M.mu_j);
      }
      x = mul_exp<false>(x, ret, zs);  // issue-bound: the early-exit form
      if (kStore) emit64(out, a, lrow, k, 1, 0, x);
    }
    if (!kStore) {
      double p = launch_payoff(a, x);
      acc += p;
      acc2 += p * p;
    }
  });
  if (!kStore) block_sum2_store(acc, acc2, a.partials + 2 * blockIdx.x);
  if (err) atomicOr(a.err, err);
}

// Hull-White one-factor short rate by its exact Gaussian transition
// (hull_white.rs:26-57): r <- r * e + (theta/a)(1 - e) + vol * z; paths only.
template <int kMode>
__global__ void __launch_bounds__(128) k_hull_white_f64(const __grid_constant__ PathLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  const HullWhiteK& H = a.hw;
  unsigned err = 0;
  Out64<kMode> out;
  out.init(dyn_smem);
  for_rows(a.rows, out, [&](uint64_t lrow) {
    const uint64_t row = a.row_begin + lrow;
    PcgGen s{pcg_path_state(a.ss, row), a.ss.inc_lo, a.ss.inc_hi};
    double x = H.r0;
    if (kMode == kRows) out.begin(a.out_f64 + lrow * (a.steps + 1));
    emit64(out, a, lrow, 0, 1, 0, x);
#pragma unroll 1
    for (uint64_t k = 1; k <= a.steps; ++k) {
      // the exact tail value: the rate paths are bit-exact with the reference
      const double z = normal_f64<false, false>(s, c, zs, err);
      x = x * H.e + H.mean_reversion + H.vol * z;
      emit64(out, a, lrow, k, 1, 0, x);
    }
  });
  if (err) atomicOr(a.err, err);
}

// fn 0: the kernels' exponential, 1: their correctly rounded sqrt, 2 and 3:
// the normal's product m * X[L] 2^-53 (L = i mod 256) on the integer pipes and
// by DMUL, 4: the exponential's early-exit form
__global__ void k_debug_f64(int fn, const double* __restrict__ x, double* __restrict__ y, uint64_t n,
                            const ZigTables* tabs) {
  __shared__ ZigShared zs;
  zig_stage(zs, tabs, true);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    y[i] = fn == 0   ? mul_exp(1.0, x[i], zs)
           : fn == 1 ? sqrt_rn_int(x[i])
           : fn == 2 ? mul_u53_rn((uint64_t)x[i], e64_xs(zs.e64[i & 255]))
           : fn == 3 ? __dmul_rn(x[i], e64_xs(zs.e64[i & 255]))
           : fn == 5 ? tail_value_fast_f64((uint64_t)__double_as_longlong(x[i]), tabs, zs)
           : fn == 6 ? tail_value_f64((uint64_t)__double_as_longlong(x[i]), tabs->r)
                     : mul_exp<false>(1.0, x[i], zs);
}

// Block v sums value v of all records: thread t adds records t, t + 256, ...
// in order, then a shared-memory tree adds the 256 partial sums.  The order
// depends only on the record count, so the result is deterministic.
__global__ void __launch_bounds__(256) k_reduce_partials(const double* __restrict__ partials, int nblocks,
                                                         int nvals, double* __restrict__ out) {
  __shared__ double sh[256];
  const int v = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += 256) s += partials[(uint64_t)b * nvals + v];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[v] = sh[0];
}

template <int kMode>
int launch_multi(const PathLaunch& L, dim3 g, dim3 b, size_t sm, cudaStream_t st) {
  switch (L.multi.na) {
    case 1: k_multi_gbm_f64<1, kMode><<<g, b, sm, st>>>(L); break;
    case 2: k_multi_gbm_f64<2, kMode><<<g, b, sm, st>>>(L); break;
    case 3: k_multi_gbm_f64<3, kMode><<<g, b, sm, st>>>(L); break;
    case 4: k_multi_gbm_f64<4, kMode><<<g, b, sm, st>>>(L); break;
    default: k_multi_gbm_f64<0, kMode><<<g, b, sm, st>>>(L); break;
  }
  return 0;
}

template <int kMode>
int launch_model(const PathLaunch& L, dim3 G, dim3 B, size_t sm, cudaStream_t st) {
  switch (L.model) {
    case kGbm: k_gbm_f64<kMode><<<G, B, sm, st>>>(L); break;
    case kHeston: k_heston_f64<kMode><<<G, B, sm, st>>>(L); break;
    case kMerton: k_merton_f64<kMode><<<G, B, sm, st>>>(L); break;
    case kMultiGbm: launch_multi<kMode>(L, G, B, sm, st); break;
    case kHullWhite:
      if (kMode == kFused) return -1;  // rate paths have no in-kernel payoff
      k_hull_white_f64<kMode == kFused ? kElems : kMode><<<G, B, sm, st>>>(L);
      break;
    default:
      return -1;
  }
  return 0;
}

}  // namespace

// Grid: one thread per row when that fits the GPU; small row counts use
// single-warp blocks so every SM gets an equal share of warps.
static void pick_grid(uint64_t rows, int* grid, int* block) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int b = rows <= (uint64_t)sms * 1024 ? 32 : 128;
  uint64_t g = (rows + b - 1) / b;
  uint64_t cap = (uint64_t)sms * 64;  // grid-stride beyond this
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  *grid = (int)g;
  *block = b;
}

int launch_paths_f64(const PathLaunch& L, cudaStream_t st) {
  int g, b;
  pick_grid(L.rows, &g, &b);
  const bool store = L.out_f64 != nullptr;
  if (!store && L.max_records && (uint64_t)g > L.max_records) return kRecordsExceeded;
  const int mode = !store ? kFused : row_store_fits(L, sizeof(double)) ? kRows : kElems;
  const size_t sm = mode == kRows ? RowStore<double>::bytes((uint32_t)b) : 0;
  dim3 G(g), B(b);
  const int rc = mode == kRows ? launch_model<kRows>(L, G, B, sm, st)
                 : mode == kElems ? launch_model<kElems>(L, G, B, 0, st)
                                  : launch_model<kFused>(L, G, B, 0, st);
  if (rc < 0) return -1;
  return cudaPeekAtLastError() == cudaSuccess ? g : -1;
}

void launch_debug_f64(int fn, const double* x, double* y, uint64_t n, const ZigTables* tabs, cudaStream_t st) {
  k_debug_f64<<<256, 256, 0, st>>>(fn, x, y, n, tabs);
}

void launch_reduce_partials(const double* partials, int nblocks, int nvals, double* out, cudaStream_t st) {
  if (nvals > 0) k_reduce_partials<<<nvals, 256, 0, st>>>(partials, nblocks, nvals, out);
}

}  // namespace stocha
