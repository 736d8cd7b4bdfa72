// Exotic Monte Carlo payoffs on GBM paths, FP64 (the reference's arithmetic):
//   barrier   src/finance/barrier.rs:286-403 (barrier_mc, rebate_path_pv)
//   asian     src/finance/asian.rs:143-290 (asian_mc: per-path arithmetic and
//             geometric payoffs; the control-variate estimator runs as two
//             device reductions) and :292-352 (asian_mc_floating_seasoned)
//   lookback  src/finance/lookback.rs:158-210 (lookback_mc)
// Every path has its own stream, Pcg64Dxsm::new(seed) advanced by
// path * (steps + 1024) * 2, and the GBM step s *= exp(drift + diffusion * z)
// with the kernels' table-driven exponential.  The running log price of the
// geometric average is carried as a sum of the step exponents (ln s_k =
// ln s0 + sum of (drift + diffusion * z)), equal to the reference's ln(s_k)
// to rounding.  Payoffs never leave registers; per-block FP64 sums (or, for
// the Asian estimator, the per-path payoff pair) go to device memory.
#include <cuda_runtime.h>

#include "exotics_kernels.h"
#include "mc_device.cuh"
#include "reduce.cuh"

namespace stocha {
namespace {

__device__ __forceinline__ double intrinsic(double s, double k, int is_call) {
  return is_call ? fmax(s - k, 0.0) : fmax(k - s, 0.0);
}

// barrier.rs:379-403: rebate paid at the hit time (knock-out, at_hit), at
// expiry on a hit (knock-out), or at expiry without a hit (knock-in).
__device__ __forceinline__ double rebate_pv(const ExoticLaunch& a, int hit) {
  const bool knocked = hit >= 0;
  if (!a.kind_in && a.rebate_at_hit) return knocked ? a.rebate * exp(-a.r * ((double)hit * a.dt)) : 0.0;
  if (!a.kind_in) return knocked ? a.rebate * exp(-a.r * ((double)a.steps * a.dt)) : 0.0;
  return knocked ? 0.0 : a.rebate * exp(-a.r * ((double)a.steps * a.dt));
}

// a >= b for doubles known to be >= +0 (or b negative), by their bits on the
// integer pipes: for non-negative IEEE doubles the order of the bit patterns
// as signed integers is the numeric order, and any negative b compares below.
__device__ __forceinline__ bool ge_pos(double a, double b) {
  return __double_as_longlong(a) >= __double_as_longlong(b);
}

__global__ void __launch_bounds__(128) k_exotic(const __grid_constant__ ExoticLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  double sum = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    PcgGen g{pcg_path_state(a.ss, i), a.ss.inc_lo, a.ss.inc_hi};
    double s = a.s0;
    if (a.kind == kExoBarrier) {
      int hit = -1;
      if (a.already_hit) {
        hit = 0;
      } else {
        for (uint64_t st = 1; st <= a.steps; ++st) {
          const double z = normal_f64(g, c, zs, err);
          s = mul_exp<false>(s, fma(a.diffusion, z, a.drift), zs);
          // s > 0 and the barrier is validated positive
          if (a.direction == 0 ? ge_pos(s, a.barrier) : ge_pos(a.barrier, s)) {
            hit = (int)st;
            break;
          }
        }
      }
      const bool knocked = hit >= 0;
      if (knocked && a.kind_in && (uint64_t)hit < a.steps)  // drive a knocked-in path to T
        for (uint64_t st = (uint64_t)hit; st < a.steps; ++st) {
          const double z = normal_f64(g, c, zs, err);
          s = mul_exp<false>(s, fma(a.diffusion, z, a.drift), zs);
        }
      const double opt = a.kind_in ? (knocked ? intrinsic(s, a.k, a.is_call) : 0.0)
                                   : (knocked ? 0.0 : intrinsic(s, a.k, a.is_call));
      // no rebate (the common case, uniform over the launch): opt + 0 / discount
      // is opt, without the FP64 division
      sum += a.rebate == 0.0 ? opt : opt + rebate_pv(a, hit) / a.discount;
    } else if (a.kind == kExoLookback) {
      double mx = a.m0, mn = a.n0;
      for (uint64_t st = 0; st < a.steps; ++st) {
        const double z = normal_f64(g, c, zs, err);
        s = mul_exp<false>(s, fma(a.diffusion, z, a.drift), zs);
        // s > 0 and mx >= s0 > 0; mn may be any non-NaN value
        if (!ge_pos(mx, s)) mx = s;
        if (!ge_pos(s, mn)) mn = s;
      }
      sum += a.strike_fixed ? (a.is_call ? fmax(mx - a.k, 0.0) : fmax(a.k - mn, 0.0))
                            : (a.is_call ? s - mn : mx - s);
    } else {  // Asian: plain (per-path pair) or floating seasoned (block sum)
      // sum over steps of ln s_k = n ln s0 + sum_i (n - i + 1) x_i: one DFMA a
      // step with the integer weight built on the integer pipes, instead of the
      // running log and its running sum (two DADDs)
      double sum_arith = 0.0, sum_wx = 0.0;
      for (uint64_t st = 0; st < a.steps; ++st) {
        const double z = normal_f64(g, c, zs, err);
        const double x = fma(a.diffusion, z, a.drift);
        s = mul_exp<false>(s, x, zs);
        sum_arith += s;
        sum_wx = fma(u53_scaled_f64(a.steps - st, 0), x, sum_wx);  // exact for steps < 2^53 (host-checked)
      }
      const double nsteps = (double)a.steps;
      const double sum_log = fma(nsteps, a.log_s0, sum_wx);
      const double avg_a = sum_arith / nsteps;
      const double avg_g = exp(sum_log / nsteps);
      if (a.kind == kExoAsian) {
        double pa, pg;
        if (!a.strike_floating) {
          pa = intrinsic(avg_a, a.k, a.is_call);
          pg = intrinsic(avg_g, a.k, a.is_call);
        } else {
          pa = a.is_call ? fmax(s - avg_a, 0.0) : fmax(avg_a - s, 0.0);
          pg = a.is_call ? fmax(s - avg_g, 0.0) : fmax(avg_g - s, 0.0);
        }
        a.arith[i] = pa;
        a.geo[i] = pg;
      } else {  // kExoAsianSeasoned (floating strike)
        const double avg_rem = a.geometric ? avg_g : avg_a;
        const double avg_t = a.geometric ? exp(log(a.a_spent) * a.w_spent + log(avg_rem) * a.w_remain)
                                         : a.w_spent * a.a_spent + a.w_remain * avg_rem;
        sum += a.is_call ? fmax(s - avg_t, 0.0) : fmax(avg_t - s, 0.0);
      }
    }
  }
  if (a.kind != kExoAsian) block_sum2_store(sum, 0.0, a.partials + 2 * (uint64_t)blockIdx.x);
  if (err) atomicOr(a.err, err);
}

// FP32 form of k_exotic (a GB300 addition; the reference prices in FP64).
// The same streams and draws (the FP32 sampler consumes exactly the
// reference's u64s); the path is carried in log space, ls = ln(S_t / s0) as a
// plain FP32 running sum of drift + diffusion * z, so the barrier test is
// ls against ln(H / s0) and the running extremes are extremes of ls, with
// one exp per path; the Asian average takes one FP32 exp per step.  Values
// differ from the FP64 form by rounding: a barrier decision can flip only for
// a path within ~1e-7 (in log price) of the barrier at a monitoring date.
// The per-path loop form of k_exotic_f32, for step counts of 2^31 and more
// (the warp-uniform form counts normals in 32 bits).
__global__ void __launch_bounds__(128) k_exotic_f32_loop(const __grid_constant__ ExoticLaunch a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, false);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  double sum = 0.0;
  const float drift = a.f_drift, diffusion = a.f_diff, s0 = a.f_s0, k = a.f_k;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    PcgGen g{pcg_path_state(a.ss, i), a.ss.inc_lo, a.ss.inc_hi};
    float ls = 0.0f;
    if (a.kind == kExoBarrier) {
      const float lb = a.f_lb;
      int hit = -1;
      if (a.already_hit) {
        hit = 0;
      } else {
        for (uint64_t st = 1; st <= a.steps; ++st) {
          ls += fmaf(diffusion, normal_f32(g, c, zs, err), drift);
          if (a.direction == 0 ? ls >= lb : ls <= lb) {
            hit = (int)st;
            break;
          }
        }
      }
      const bool knocked = hit >= 0;
      if (knocked && a.kind_in && (uint64_t)hit < a.steps)
        for (uint64_t st = (uint64_t)hit; st < a.steps; ++st) ls += fmaf(diffusion, normal_f32(g, c, zs, err), drift);
      const float sT = s0 * expf(ls);
      const float iv = a.is_call ? fmaxf(sT - k, 0.0f) : fmaxf(k - sT, 0.0f);
      const float opt = a.kind_in ? (knocked ? iv : 0.0f) : (knocked ? 0.0f : iv);
      sum += a.rebate == 0.0 ? (double)opt : (double)opt + rebate_pv(a, hit) / a.discount;
    } else if (a.kind == kExoLookback) {
      float lmx = a.f_lm0, lmn = a.f_ln0;
      for (uint64_t st = 0; st < a.steps; ++st) {
        ls += fmaf(diffusion, normal_f32(g, c, zs, err), drift);
        lmx = fmaxf(lmx, ls);
        lmn = fminf(lmn, ls);
      }
      const float s = s0 * expf(ls), mx = s0 * expf(lmx), mn = s0 * expf(lmn);
      sum += a.strike_fixed ? (a.is_call ? fmaxf(mx - k, 0.0f) : fmaxf(k - mn, 0.0f))
                            : (a.is_call ? s - mn : mx - s);
    } else {  // Asian: plain (per-path pair) or floating seasoned (block sum)
      float sum_arith = 0.0f, sum_log = 0.0f;
      for (uint64_t st = 0; st < a.steps; ++st) {
        ls += fmaf(diffusion, normal_f32(g, c, zs, err), drift);
        sum_arith += expf(ls);
        sum_log += ls;
      }
      const double nsteps = (double)a.steps;
      const double s = (double)s0 * exp((double)ls);
      const double avg_a = a.s0 * (double)sum_arith / nsteps;
      const double avg_g = a.s0 * exp((double)sum_log / nsteps);
      if (a.kind == kExoAsian) {
        double pa, pg;
        if (!a.strike_floating) {
          pa = intrinsic(avg_a, a.k, a.is_call);
          pg = intrinsic(avg_g, a.k, a.is_call);
        } else {
          pa = a.is_call ? fmax(s - avg_a, 0.0) : fmax(avg_a - s, 0.0);
          pg = a.is_call ? fmax(s - avg_g, 0.0) : fmax(avg_g - s, 0.0);
        }
        a.arith[i] = pa;
        a.geo[i] = pg;
      } else {  // kExoAsianSeasoned (floating strike)
        const double avg_rem = a.geometric ? avg_g : avg_a;
        const double avg_t = a.geometric ? exp(log(a.a_spent) * a.w_spent + log(avg_rem) * a.w_remain)
                                         : a.w_spent * a.a_spent + a.w_remain * avg_rem;
        sum += a.is_call ? fmax(s - avg_t, 0.0) : fmax(avg_t - s, 0.0);
      }
    }
  }
  if (a.kind != kExoAsian) block_sum2_store(sum, 0.0, a.partials + 2 * (uint64_t)blockIdx.x);
  if (err) atomicOr(a.err, err);
}

// Sums over the Asian payoff pairs: mode 0 {sum a, sum g}; mode 1, with the
// means m = {ma, mg}: {sum (a - ma)(g - mg), sum (g - mg)^2} (asian.rs:270-281).
__global__ void __launch_bounds__(256) k_asian_sums(const double* __restrict__ arith, const double* __restrict__ geo,
                                                    uint64_t n, int mode, const double* __restrict__ means,
                                                    double* __restrict__ partials) {
  double s0 = 0.0, s1 = 0.0;
  const double ma = mode ? means[0] : 0.0, mg = mode ? means[1] : 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    if (mode == 0) {
      s0 += arith[i];
      s1 += geo[i];
    } else {
      const double dg = geo[i] - mg;
      s0 += (arith[i] - ma) * dg;
      s1 += dg * dg;
    }
  }
  block_sum2_store(s0, s1, partials + 2 * (uint64_t)blockIdx.x);
}

// One thread: the means of the mode-0 totals (means[i] = totals[i] / n).
__global__ void k_asian_means(const double* __restrict__ totals, uint64_t n, double* __restrict__ means) {
  if (threadIdx.x == 0) {
    means[0] = totals[0] / (double)n;
    means[1] = totals[1] / (double)n;
  }
}

// FP32 exotic Monte Carlo on the warp-uniform sampler feed (ZigFeed): a warp
// simulates 32 paths together, every lane stepping its generator each
// iteration, and only wedge tests and tail draws diverge.  Each thread takes
// the paths of the per-path loop form (path i on thread i mod the grid's
// threads), and the normals, their order and every per-path update are the
// loop form's, so the per-thread sums and the block totals are the same bits.
// A knocked-out barrier path stops drawing (its lane needs no more normals);
// a knock-in path draws to maturity.
__global__ void __launch_bounds__(128, 8) k_exotic_f32(const __grid_constant__ ExoticLaunch a) {
  __shared__ ZigShared32 zs;
  zig_stage32(zs, a.tabs);
  const SamplerCtx c{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  double sum = 0.0;
  const float drift = a.f_drift, diffusion = a.f_diff, s0 = a.f_s0, k = a.f_k, lb = a.f_lb;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint32_t steps = (uint32_t)a.steps;
  for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wb < a.n; wb += stride) {
    const uint64_t i = wb + (threadIdx.x & 31u);
    const bool on = i < a.n;
    DevPcg st = pcg_path_state(a.ss, on ? i : wb);
    ZigFeed q;
    float ls = 0.0f;
    int hit = -1;  // barrier: the monitoring step of the first crossing
    float lmx = a.f_lm0, lmn = a.f_ln0;  // lookback
    float sum_arith = 0.0f, sum_log = 0.0f;  // Asian
    uint32_t need = on ? steps : 0u;
    if (a.kind == kExoBarrier && a.already_hit) {
      hit = 0;
      if (!a.kind_in) need = 0;  // knocked out before the first step: nothing to draw
    }
    uint32_t cnt = 0;
    uf_drive(cnt, need, uf_cap(a.steps), err, [&]() {
      float z;
      if (q.feed(pcg_next(st, a.ss.inc_lo, a.ss.inc_hi), zs, c, z) & (cnt < need)) {
        ls += fmaf(diffusion, z, drift);
        ++cnt;
        if (a.kind == kExoBarrier) {
          if (hit < 0 && (a.direction == 0 ? ls >= lb : ls <= lb)) {
            hit = (int)cnt;
            if (!a.kind_in) need = cnt;  // knocked out: stop drawing
          }
        } else if (a.kind == kExoLookback) {
          lmx = fmaxf(lmx, ls);
          lmn = fminf(lmn, ls);
        } else {
          sum_arith += expf(ls);
          sum_log += ls;
        }
      }
    });
    if (!on) continue;
    if (a.kind == kExoBarrier) {
      const bool knocked = hit >= 0;
      const float sT = s0 * expf(ls);
      const float iv = a.is_call ? fmaxf(sT - k, 0.0f) : fmaxf(k - sT, 0.0f);
      const float opt = a.kind_in ? (knocked ? iv : 0.0f) : (knocked ? 0.0f : iv);
      sum += a.rebate == 0.0 ? (double)opt : (double)opt + rebate_pv(a, hit) / a.discount;
    } else if (a.kind == kExoLookback) {
      const float s = s0 * expf(ls), mx = s0 * expf(lmx), mn = s0 * expf(lmn);
      sum += a.strike_fixed ? (a.is_call ? fmaxf(mx - k, 0.0f) : fmaxf(k - mn, 0.0f))
                            : (a.is_call ? s - mn : mx - s);
    } else {  // Asian: plain (per-path pair) or floating seasoned (block sum)
      const double nsteps = (double)a.steps;
      const double s = (double)s0 * exp((double)ls);
      const double avg_a = a.s0 * (double)sum_arith / nsteps;
      const double avg_g = a.s0 * exp((double)sum_log / nsteps);
      if (a.kind == kExoAsian) {
        double pa, pg;
        if (!a.strike_floating) {
          pa = intrinsic(avg_a, a.k, a.is_call);
          pg = intrinsic(avg_g, a.k, a.is_call);
        } else {
          pa = a.is_call ? fmax(s - avg_a, 0.0) : fmax(avg_a - s, 0.0);
          pg = a.is_call ? fmax(s - avg_g, 0.0) : fmax(avg_g - s, 0.0);
        }
        a.arith[i] = pa;
        a.geo[i] = pg;
      } else {  // kExoAsianSeasoned (floating strike)
        const double avg_rem = a.geometric ? avg_g : avg_a;
        const double avg_t = a.geometric ? exp(log(a.a_spent) * a.w_spent + log(avg_rem) * a.w_remain)
                                         : a.w_spent * a.a_spent + a.w_remain * avg_rem;
        sum += a.is_call ? fmax(s - avg_t, 0.0) : fmax(avg_t - s, 0.0);
      }
    }
  }
  if (a.kind != kExoAsian) block_sum2_store(sum, 0.0, a.partials + 2 * (uint64_t)blockIdx.x);
  if (err) atomicOr(a.err, err);
}

}  // namespace

int exotic_grid(uint64_t n, int sms) {
  const uint64_t want = (n + 127) / 128;
  const uint64_t cap = (uint64_t)sms * 32;
  return (int)(want < cap ? (want ? want : 1) : cap);
}

void launch_exotic(const ExoticLaunch& a, int grid, cudaStream_t st) {
  if (a.f32) {
    // converted here rather than in the kernel, where the compiler may redo a
    // conversion (an FP64-pipe instruction) inside the path loop
    ExoticLaunch b = a;
    b.f_drift = (float)a.drift;
    b.f_diff = (float)a.diffusion;
    b.f_s0 = (float)a.s0;
    b.f_k = (float)a.k;
    b.f_lb = (float)a.lbarrier;
    b.f_lm0 = (float)a.lm0;
    b.f_ln0 = (float)a.ln0;
    if (a.steps < (1ull << 31))
      k_exotic_f32<<<grid, 128, 0, st>>>(b);
    else
      k_exotic_f32_loop<<<grid, 128, 0, st>>>(b);
  } else
    k_exotic<<<grid, 128, 0, st>>>(a);
}

void launch_asian_sums(const double* arith, const double* geo, uint64_t n, int mode, const double* means,
                       double* partials, int grid, cudaStream_t st) {
  k_asian_sums<<<grid, 256, 0, st>>>(arith, geo, n, mode, means, partials);
}

void launch_asian_means(const double* totals, uint64_t n, double* means, cudaStream_t st) {
  k_asian_means<<<1, 32, 0, st>>>(totals, n, means);
}

}  // namespace stocha
