// Types shared by the host side and the kernels of the Monte Carlo engine.
#pragma once
#include <stdint.h>

namespace stocha {

// rand_pcg Lcg128CmDxsm64 multiplier ("cheap multiplier", 64-bit).
constexpr uint64_t kPcgMul = 0xda942042e4dd58b5ULL;

// A PCG state jump: state' = mul * state + add (mod 2^128), as (lo, hi) words.
struct PcgJump {
  uint64_t mul_lo, mul_hi, add_lo, add_hi;
};

// The streams of one launch: every path i starts from `base` advanced by
// i * block draws (gbm.rs:58-59).  jump[j] advances by block * 2^j.
constexpr int kMaxJumpBits = 48;
struct StreamSpec {
  uint64_t base_lo, base_hi;  // state of Pcg64Dxsm::new(seed)
  uint64_t inc_lo, inc_hi;    // LCG increment (odd), shared by all paths
  PcgJump jump[kMaxJumpBits];
};

// Ziggurat tables as the kernels read them (filled once per context).
//   thr[L]   : fast path taken iff (u >> 11) < thr[L]; equivalent to the
//              reference's  (u>>11)*2^-53*X[L] < X[L+1]  (normal.rs:25-27).
//   xs[L]    : X[L] * 2^-53 (exact), so x = (double)(u>>11) * xs[L] rounds
//              exactly like the reference's u_frac * X[L].
//   y[257]   : Y table (wedge test, normal.rs:38-42).
//   x32/y32  : float copies for the FP32 kernels.
struct ZigTables {
  uint64_t thr[256];
  double xs[256];
  double x[257];
  double y[257];
  float x32[257];
  float y32[257];
  double r;
  float r32;
  float nrinv32;  // -1/R rounded to float (the FP32 tail test's x = ln(u1) * nrinv32)
  double nrinv;   // -1/R (the path kernels' FP64 tail value)
  uint64_t exp2q[256];  // 2^(j/256) * 2^63 (integer-pipe exponential)
};

// Device error bits (ORed into a per-context word).
enum : unsigned {
  kErrZigAttempts = 1u,  // a normal draw exceeded the rejection-attempt cap
  kErrTailIters = 2u,    // a ziggurat tail draw exceeded its iteration cap
  kErrQueue = 4u,        // persistent work queue inconsistency
  kErrGammaIters = 8u,   // a gamma draw exceeded its rejection cap
};

// Iteration caps for rejection loops.  The reference loops without bound; the
// probability of reaching these caps with a correct table is below 1e-300.
constexpr int kZigMaxAttempts = 4096;
constexpr int kZigMaxTail = 4096;
constexpr int kGammaMaxIters = 1 << 20;

}  // namespace stocha
