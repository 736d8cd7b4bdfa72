// Batched bump-and-revalue Greeks with common random numbers (greeks.rs:322-358
// for one instance; many instances per launch here).  Shared by greeks.cu and
// greeks_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_types.h"

namespace stocha {

// Per-path sums accumulated for one instance (FP32 per thread, FP64 per block):
//   0 P0    payoff at the base parameters
//   1 P0sq  its square (standard error)
//   2 Ds    pay(S0+h) - pay(S0-h)             (delta)
//   3 Gs    pay(S0+h) - 2 pay(S0) + pay(S0-h) (gamma)
//   4 Dv    pay(sigma+h) - pay(sigma-h)       (vega; Heston: v0 +- h)
//   5 DT    pay(T-h) - pay(T)                 (theta)
//   6 PT    pay(T-h)
//   7 Dr    pay(r+h) - pay(r-h)               (rho; same-path drift shift)
//   8 Prm   pay(r-h)
constexpr int kGreekAcc = 9;

// Trajectory index of the scenario constants.
enum : int { kTrBase = 0, kTrSigUp = 1, kTrSigDn = 2, kTrTDn = 3 };

struct GInst {
  StreamSpec ss;
  int model;   // kGbm / kHeston / kMerton
  int payoff;  // kCall / kPut
  int theta_pass;  // Merton: run the T-h scenario as a second pass
  int price_only;  // only sums 0 and 1 (the others are written as zero)
  uint64_t steps, n_paths, item_begin, chunk;
  uint64_t jthr[2];  // Merton jump thresholds at T and T-h
  float K, s0, u;    // s0 bump ratio u = h_s0 / s0
  float erp, erm, sh2;  // exp(h_r T), exp(-h_r T), 2 sinh(h_r T)
  // GBM / Merton: log S_T = kdrift + diff * sum(z) (+ jumps) per trajectory
  float kdrift[4], diff[4];
  float mu_j, sigma_j;
  // Heston full-truncation Euler per trajectory (v0, dt) variants
  float hv0[4], hkdt[4], hxsdt[4], hnhdt[4], hmudt[4], hsdt[4];
  float hrho, hrho_comp, htheta;
};

struct GreeksLaunch {
  const GInst* inst;           // device array
  const uint32_t* item_inst;   // item -> instance (NULL: found from the instances' item_begin)
  uint64_t total_items;
  unsigned long long* counter; // work-queue head (zeroed before launch; unused when direct)
  int direct;                  // 1: one block per item, grid = total_items
  double* item_part;           // total_items * kGreekAcc
  double* inst_sums;           // n_inst * kGreekAcc
  int n_inst;
  const ZigTables* tabs;
  unsigned* err;
};

void launch_greeks_batch(const GreeksLaunch& g, cudaStream_t st);

}  // namespace stocha
