// Internal interface between the C-ABI host code (api.cpp) and the kernel
// translation units.  Nothing here is exported from the shared library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_types.h"

namespace stocha {

constexpr int kMaxAssets = 16;

enum Model : int { kGbm = 0, kHeston = 1, kMerton = 2, kMultiGbm = 3, kHullWhite = 4 };
// In-kernel payoffs of the fused FP64 kernels.  kPw*: the pathwise (IPA)
// estimators of greeks.rs:387-418 (aux = s0, r, sigma, t).
enum Payoff : int { kCall = 0, kPut = 1, kPwDeltaCall = 2, kPwDeltaPut = 3, kPwVegaCall = 4, kPwVegaPut = 5 };

// Model constants, computed on the host with the reference's expression order
// so that every double the kernels start from equals the reference's.
struct GbmK {  // gbm.rs:43-45
  double s0, drift, diffusion;
};
struct HestonK {  // heston.rs:45-48 (Euler), :92-97,143-150 (QE)
  double s0, v0, mu, kappa, theta, xi, rho;
  double dt, sqrt_dt, rho_comp;
  double e_kdt, k1, qe_m0, qe_s2b, one_m_ekdt;
  double k0_s, k1_s, k2_s, k3_s, k4_s;
  double kdt, xi_rho, xi_rho_comp;  // kappa dt, xi rho, xi sqrt(1 - rho^2) (FP64 Euler kernel)
  int scheme;  // 0 euler, 1 qe
};
struct MertonK {  // jump_diffusion.rs:49-64
  double s0, drift, diffusion, mu_j, sigma_j;
  uint64_t jump_thr;  // u < jump_prob  <=>  (u64 >> 11) < jump_thr
};
struct MultiK {  // multi_gbm.rs:22-40
  int na;
  double s0[kMaxAssets], drift[kMaxAssets], diffusion[kMaxAssets];
  double L[kMaxAssets * kMaxAssets];   // lower Cholesky factor, row-major
  double LD[kMaxAssets * kMaxAssets];  // diffusion[i] * L[i][j] (the FP64 kernel's exponent rows)
};

struct HullWhiteK {  // hull_white.rs:26-30: exact transition constants
  double r0, e, mean_reversion, vol;
};

// FP32 constants of the FP32 kernels, rounded once on the host: a double
// operation or a double->float conversion inside a kernel runs on the FP64
// pipe (1/64 of the FP32 rate on GB300), which these kernels avoid entirely.
struct F32K {
  float strike;
  float g_s0, g_kdrift, g_diff, g_drift;  // GBM: kdrift = steps * drift
  float m_s0, m_kdrift, m_diff, m_drift, m_mu_j, m_sigma_j;  // Merton
  float h_s0, h_v0, h_rho, h_rho_comp, h_kdt, h_theta, h_xsdt, h_nhdt, h_mudt, h_sdt;  // Heston Euler
  // Heston QE: m = m0 + v+ e_kdt, s2 = cs2 v+ + s2b, log-price coefficients
  // k0..k4 (heston.rs:112-150), log s0
  float q_ekdt, q_m0, q_cs2, q_s2b, q_k0, q_k1, q_k2, q_k3, q_k4, q_ls0;
  float a_s0[kMaxAssets], a_kdrift[kMaxAssets], a_diff[kMaxAssets], a_drift[kMaxAssets];
  float a_L[kMaxAssets * kMaxAssets];
};

// One launch of a path kernel over output rows [row_begin, row_begin+rows).
struct PathLaunch {
  StreamSpec ss;
  const ZigTables* tabs;
  unsigned* err;
  // materialised mode: row-major rows of `row_len` values (out_f64 or out_f32)
  double* out_f64;
  float* out_f32;
  int time_major;     // 1: out[step * rows + row] (internal consumers, e.g. LSMC)
  int terminal_only;  // 1: out[row] = S_T only (terminal prices, greeks.rs:165-166)
  // fused mode: per-block partial sums {sum payoff, sum payoff^2} per asset
  double* partials;
  // fused FP32 mode with a work queue (work != nullptr): warps take batches
  // of batch_rows consecutive rows (a multiple of 32) from the counter *work,
  // which the launcher zeroes, and write one partial record per batch
  unsigned long long* work;
  uint32_t batch_rows;
  // fused mode: when non-zero, the launcher returns kRecordsExceeded without
  // launching if its grid would write more partial records than this (callers
  // whose record buffer has a fixed size)
  uint64_t max_records;
  double strike;
  int payoff;
  double aux[4];  // payoff parameters (pathwise estimators: s0, r, sigma, t)
  uint64_t row_begin, rows, steps, base_paths;
  int model;
  int flat_grid;  // FP32 kernels: one row per thread and no grid cap (blocks retire
                  // early, so work on higher-priority streams gets SMs sooner)
  GbmK gbm;
  HestonK heston;
  MertonK merton;
  MultiK multi;
  HullWhiteK hw;
  F32K f32;
};

// Launch shape of the fused FP32 pricing kernels, per model kind (tuning
// slot: 0 gbm, 1 heston, 2 merton, 3..6 multi-GBM with 1..4 assets).
struct FusedTune {
  int block;    // threads per block: 64, 128 or 256
  int ilp;      // paths per thread in lockstep: 1 or 2 (lockstep form)
  int waves;    // grid = waves * resident blocks (1 or 2)
  int variant;  // 0: per-path loop kernel (ilp 1); 1: lockstep kernel; 2: warp-uniform sampler feed (ilp 1)
};
constexpr int kTuneSlots = 7;
int tune_slot(int model, int na);  // -1: no fused FP32 kernel for this model
FusedTune get_fused_tune(int slot);
int set_fused_tune(int slot, FusedTune t);  // 0, or -1 for an invalid slot or shape

// Whether the staged sector writer takes L's rows: row-major output of at
// least two 32-byte sectors a row (the first and last sectors of a row are
// then distinct) and below 2^31 elements (its offsets are 32-bit).
inline bool row_store_fits(const PathLaunch& L, uint64_t elem) {
  if (L.time_major || L.terminal_only) return false;
  const uint64_t width = L.model == kMultiGbm ? (uint64_t)L.multi.na : 1;
  const uint64_t row_len = (L.steps + 1) * width;
  return row_len >= 2 * (32 / elem) && row_len < (1ull << 31);
}

// Rounds the FP32 constants of L (after the model constants are set).
void fill_f32_constants(PathLaunch* L);

// Launch helpers (paths_f64.cu / paths_f32.cu).  Return the number of
// partial records written in fused mode (blocks launched, or batches in the
// work-queue mode), -1 on error, or kRecordsExceeded (nothing launched) when
// that number would exceed L.max_records.
constexpr int kRecordsExceeded = -2;
int launch_paths_f64(const PathLaunch& L, cudaStream_t st);
int launch_paths_f32(const PathLaunch& L, cudaStream_t st);
// y[i] = exp(x[i]) by the kernels' table-driven exponential (diagnostic).
void launch_debug_f64(int fn, const double* x, double* y, uint64_t n, const ZigTables* tabs, cudaStream_t st);
// out[0..1] (zeroed by the caller): float bits of the largest absolute error
// of __logf on [0.5, 1) and of its largest relative error below 0.5.
void launch_debug_logf_scan(unsigned* out, cudaStream_t st);

// Diagnostic: n normals for each of n_paths streams from one of the FP32
// samplers, and each stream's generator state after its last consumed draw.
struct DebugZig {
  StreamSpec ss;
  const ZigTables* tabs;
  unsigned* err;
  float* out;         // [n_paths][n]
  uint64_t* state;    // [n_paths][2]: lo, hi
  uint64_t n_paths;
  uint32_t n;
  int form;           // 0: normal_f32 one normal after another; 1: ZigFeed, warp-uniform
};
void launch_debug_zigfeed(const DebugZig& a, cudaStream_t st);
// Sum per-block partials (deterministic order) into out[nvals].
void launch_reduce_partials(const double* partials, int nblocks, int nvals, double* out, cudaStream_t st);

}  // namespace stocha
