// LSMC backward-sweep launch description (lsmc.cu), used by lsmc_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace stocha {

// Per-step regression state, resident on the device.
struct LsmcStep {
  double m, mean, std, inv_std;
  double coef[5];
  int skip;
  int pad;
};

struct LsmcLaunch {
  const void* spot;  // time-major spot[(steps+1) * n], double or float
  int spot_f32;
  double* cf;        // n cash flows
  double* part;      // grid * 14 partials
  LsmcStep* step_params;  // steps entries
  double* result;    // [0] mean of discounted cash flows, [1] sum of squared deviations
  uint64_t n, steps;
  double k, disc;
  int is_put, deg, grid;
};

void lsmc_sweep(const LsmcLaunch& a, cudaStream_t st);

}  // namespace stocha
