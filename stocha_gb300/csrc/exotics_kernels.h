// Exotic Monte Carlo launch description (exotics.cu), used by exotics_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_types.h"

namespace stocha {

enum ExoticKind : int { kExoBarrier = 0, kExoAsian = 1, kExoLookback = 2, kExoAsianSeasoned = 3 };

struct ExoticLaunch {
  StreamSpec ss;
  const ZigTables* tabs;
  unsigned* err;
  double* partials;      // per block {sum, 0} (barrier, lookback, seasoned Asian)
  double* arith;         // Asian: per-path arithmetic payoff
  double* geo;           // Asian: per-path geometric payoff
  int kind;
  int is_call;
  // barrier
  int direction;         // 0 up, 1 down
  int kind_in;           // 1 knock-in, 0 knock-out
  int rebate_at_hit;
  int already_hit;
  // Asian / lookback
  int strike_floating;   // Asian
  int strike_fixed;      // lookback
  int geometric;         // seasoned Asian
  int f32;               // 1: the FP32 form (log-space paths, FP32 sampler)
  uint64_t n, steps;
  double s0, k, drift, diffusion, discount, dt, r;
  double barrier, rebate;
  double log_s0;                  // Asian: ln(s0)
  double m0, n0;                  // lookback: initial running max / min
  double a_spent, w_spent, w_remain;  // seasoned Asian
  double lbarrier, lm0, ln0;          // FP32 form: ln(barrier / s0), ln(m0 / s0), ln(n0 / s0)
  // FP32 form: the constants it reads, rounded once on the host (launch_exotic)
  float f_drift, f_diff, f_s0, f_k, f_lb, f_lm0, f_ln0;
};

int exotic_grid(uint64_t n, int sms);
void launch_exotic(const ExoticLaunch& a, int grid, cudaStream_t st);
void launch_asian_sums(const double* arith, const double* geo, uint64_t n, int mode, const double* means,
                       double* partials, int grid, cudaStream_t st);
void launch_asian_means(const double* totals, uint64_t n, double* means, cudaStream_t st);

}  // namespace stocha
