// Batched FP32 bump-and-revalue Greeks with common random numbers.
//
// One persistent launch serves a queue of work items (instance, chunk of
// paths) drawn from many instances with different models, path counts and
// step counts.  A block takes the next item from a global counter, its
// threads simulate the item's paths, and the block writes the item's partial
// sums; a final pass adds each instance's items in a fixed order.
//
// Common random numbers (greeks.rs:322-358 prices every scenario with the
// same seed): every path's draws are generated once and drive all scenarios.
//   * s0 bumps: S_T is linear in s0 in all three models, so S_T(s0 +- h) =
//     S_T * (1 +- h/s0); the payoff differences are formed per path by case
//     analysis at the strike (no cancellation for tiny h).
//   * drift (rho) bumps: S_T(mu +- h) = S_T * exp(+-h T) (the drift enters
//     the log price as steps*dt*mu); same per-path differences.
//   * sigma bumps (Heston: v0) and the T-h scenario: separate trajectories
//     driven by the same normals (GBM and Merton in closed form from the sum
//     of the normals; Heston as extra (v, log S) recurrences).  Merton's T-h
//     scenario changes the jump probability and therefore the draws it
//     consumes (jump_diffusion.rs:60,79-80): it runs as a second pass over
//     the same stream.
#include <cuda_runtime.h>

#include "engine.h"
#include "greeks_kernels.h"
#include "mc_device.cuh"
#include "reduce.cuh"

namespace stocha {
namespace {

struct K32 {
  float s, c;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

__device__ __forceinline__ float pay(float s, float k, int call) { return call ? fmaxf(s - k, 0.0f) : fmaxf(k - s, 0.0f); }

// First and second payoff differences for  up = S*ru, base = S, dn = S*rd
// (ru > 1 > rd) with  up - dn = S * dud  and  up - 2 S + dn = S * d2
// supplied exactly by the caller.
__device__ __forceinline__ void diffs(float S, float up, float dn, float dud, float d2, float K, int call,
                                      float* d1_out, float* g_out) {
  float d1, g;
  if (call) {
    if (dn >= K) {
      d1 = S * dud;
      g = S * d2;
    } else if (up <= K) {
      d1 = 0.0f;
      g = 0.0f;
    } else {
      d1 = up - K;
      g = S <= K ? up - K : (up - K) - 2.0f * (S - K);
    }
  } else {
    if (up <= K) {
      d1 = -S * dud;
      g = -S * d2;
    } else if (dn >= K) {
      d1 = 0.0f;
      g = 0.0f;
    } else {
      d1 = -(K - dn);
      g = S >= K ? K - dn : (K - dn) - 2.0f * (K - S);
    }
  }
  *d1_out = d1;
  *g_out = g;
}

// Per-path contributions from the terminal values of the trajectories (PO:
// price only, the first two sums).
template <bool PO>
__device__ __forceinline__ void contribute(const GInst& I, float S, float S_sp, float S_sm, float S_tm, K32* acc) {
  const int call = I.payoff == kCall;
  const float p0 = pay(S, I.K, call);
  acc[0].add(p0);
  acc[1].add(p0 * p0);
  if constexpr (PO) return;
  float d1, g;
  diffs(S, S * (1.0f + I.u), S * (1.0f - I.u), 2.0f * I.u, 0.0f, I.K, call, &d1, &g);
  acc[2].add(d1);
  acc[3].add(g);
  acc[4].add(pay(S_sp, I.K, call) - pay(S_sm, I.K, call));
  const float pt = pay(S_tm, I.K, call);
  acc[5].add(pt - p0);
  acc[6].add(pt);
  const float sp = S * I.erp, sm = S * I.erm;
  float dr, gr;
  diffs(S, sp, sm, I.sh2, 0.0f, I.K, call, &dr, &gr);
  acc[7].add(dr);
  acc[8].add(pay(sm, I.K, call));
}

// Draws per warp vote in the feed loops.  This kernel holds the three models,
// each in a price-only and a Greeks form; with 8 draws a vote its code outgrew
// the instruction cache (ncu: instruction fetch the top stall).  Measured on
// GB300, 512-instance batch: 8 draws 77.7 ms, 4 draws 66.1 ms, 2 draws 67.6 ms.
constexpr int kGreeksUnroll = 4;

// The paths of a warp are 32 consecutive ones (base + lane), simulated with
// the warp-uniform sampler feed (ZigFeed): every lane steps its generator in
// the same instruction each iteration and only wedge tests and the tail
// diverge.  Draws and FP32 values are those of normal_f32 one normal after
// another, and every per-path sum adds them in the same order, so the results
// are those of a per-thread loop over normal_f32.  A lane past the chunk end
// (ok false) runs on a valid stream and contributes nothing.
template <bool PO>
__device__ void path_gbm(const GInst& I, uint64_t p, bool ok, const SamplerCtx& c, const ZigShared32& zs,
                         unsigned& err, K32* acc) {
  DevPcg st = pcg_path_state(I.ss, p);
  ZigFeed q;
  // plain FP32 sum of the normals: every scenario of the path is a closed
  // form of the same W, so its rounding (~5e-6 over 252 steps) moves them
  // together and cancels in the bump differences
  float W = 0.0f;
  const uint32_t need = ok ? (uint32_t)I.steps : 0u;
  uint32_t cnt = 0;
  uf_drive<kGreeksUnroll>(cnt, need, uf_cap(I.steps), err, [&]() {
    float z;
    if (q.feed(pcg_next(st, I.ss.inc_lo, I.ss.inc_hi), zs, c, z) & (cnt < need)) {
      W += z;
      ++cnt;
    }
  });
  if (!ok) return;
  constexpr int NT = PO ? 1 : 4;
  float S[4];
#pragma unroll
  for (int t = 0; t < NT; ++t) S[t] = I.s0 * expf(fmaf(I.diff[t], W, I.kdrift[t]));
  contribute<PO>(I, S[0], S[PO ? 0 : 1], S[PO ? 0 : 2], S[PO ? 0 : 3], acc);
}

// Merton: after the diffusion normal of a step the lane takes the jump
// uniform at once (a second generator step in the same iteration); on a jump
// its next normal is the jump size.
__device__ void merton_pass(const GInst& I, uint64_t p, bool ok, uint64_t thr, const SamplerCtx& c,
                            const ZigShared32& zs, unsigned& err, float* W, float* J) {
  DevPcg st = pcg_path_state(I.ss, p);
  ZigFeed q;
  float w = 0.0f;  // plain sum, as for GBM
  float jumps = 0.0f;
  bool in_jump = false;
  const uint32_t need = ok ? (uint32_t)I.steps : 0u;
  uint32_t cnt = 0;
  uf_drive<kGreeksUnroll>(cnt, need, uf_cap(2 * I.steps), err, [&]() {
    float z;
    if (q.feed(pcg_next(st, I.ss.inc_lo, I.ss.inc_hi), zs, c, z) & (cnt < need)) {
      if (in_jump) {
        jumps += fmaf(I.sigma_j, z, I.mu_j);
        in_jump = false;
        ++cnt;
      } else {
        w += z;
        if ((pcg_next(st, I.ss.inc_lo, I.ss.inc_hi) >> 11) < thr)
          in_jump = true;
        else
          ++cnt;
      }
    }
  });
  *W = w;
  *J = jumps;
}

template <bool PO>
__device__ void path_merton(const GInst& I, uint64_t p, bool ok, const SamplerCtx& c, const ZigShared32& zs,
                            unsigned& err, K32* acc) {
  float W, J;
  merton_pass(I, p, ok, I.jthr[0], c, zs, err, &W, &J);
  float S[4];
  if constexpr (PO) {
    if (!ok) return;
    S[0] = I.s0 * expf(fmaf(I.diff[0], W, I.kdrift[0]) + J);
    contribute<true>(I, S[0], S[0], S[0], S[0], acc);
  } else {
#pragma unroll
    for (int t = 0; t < 3; ++t) S[t] = I.s0 * expf(fmaf(I.diff[t], W, I.kdrift[t]) + J);
    if (I.theta_pass) {
      float W2, J2;
      merton_pass(I, p, ok, I.jthr[1], c, zs, err, &W2, &J2);
      S[3] = I.s0 * expf(fmaf(I.diff[3], W2, I.kdrift[3]) + J2);
    } else {
      S[3] = S[0];
    }
    if (!ok) return;
    contribute<false>(I, S[0], S[1], S[2], S[3], acc);
  }
}

// Heston: two draws a call and at most one step a call, its normals picked by
// the lane's phase (as in the fused pricing kernel): the steps' arithmetic,
// four scenarios of it for the Greeks, issues once per two draws.
template <bool PO>
__device__ void path_heston(const GInst& I, uint64_t p, bool ok, const SamplerCtx& c, const ZigShared32& zs,
                            unsigned& err, K32* acc) {
  constexpr int NT = PO ? 1 : 4;
  DevPcg st = pcg_path_state(I.ss, p);
  ZigFeed q;
  float v[4];
  K32 lg[4];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    v[t] = I.hv0[t];
    lg[t] = K32{0.0f, 0.0f};
  }
  float zc = 0.0f;
  bool half = false;
  const uint32_t need = ok ? (uint32_t)I.steps : 0u;
  uint32_t cnt = 0;
  uf_drive<kGreeksUnroll / 2>(cnt, need, uf_cap(2 * I.steps), err, [&]() {
    float z1, z2;
    const bool a1 = q.feed(pcg_next(st, I.ss.inc_lo, I.ss.inc_hi), zs, c, z1);
    const bool a2 = q.feed(pcg_next(st, I.ss.inc_lo, I.ss.inc_hi), zs, c, z2);
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
      const float dw2 = fmaf(I.hrho, dw1, I.hrho_comp * dz);
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const float vp = fmaxf(v[t], 0.0f);
        const float sv = sqrt_approx(vp);
        v[t] += fmaf(I.hkdt[t], I.htheta - vp, I.hxsdt[t] * sv * dw2);
        lg[t].add(fmaf(I.hnhdt[t], vp, I.hmudt[t]) + sv * I.hsdt[t] * dw1);
      }
      ++cnt;
    }
  });
  if (!ok) return;
  float S[4];
#pragma unroll
  for (int t = 0; t < NT; ++t) S[t] = I.s0 * expf(lg[t].s - lg[t].c);
  contribute<PO>(I, S[0], S[PO ? 0 : 1], S[PO ? 0 : 2], S[PO ? 0 : 3], acc);
}

// Paths [lo, hi) of one instance, one per thread in turn, then the item's
// block totals (compensated FP32 per thread and per warp, FP64 across warps).
template <bool PO>
__device__ __forceinline__ void run_item(const GInst& I, uint64_t lo, uint64_t hi, const SamplerCtx& c,
                                         const ZigShared32& zs, unsigned& err, double* out) {
  constexpr int NA = PO ? 2 : kGreekAcc;
  K32 acc[kGreekAcc];
#pragma unroll
  for (int j = 0; j < kGreekAcc; ++j) acc[j] = K32{0.0f, 0.0f};
  // warp-uniform loop: the sampler feed votes across all 32 lanes
  for (uint64_t b = lo + (threadIdx.x & ~31u); b < hi; b += blockDim.x) {
    const uint64_t p = b + (threadIdx.x & 31u);
    const bool ok = p < hi;
    const uint64_t pp = ok ? p : b;
    if (I.model == kGbm)
      path_gbm<PO>(I, pp, ok, c, zs, err, acc);
    else if (I.model == kHeston)
      path_heston<PO>(I, pp, ok, c, zs, err, acc);
    else
      path_merton<PO>(I, pp, ok, c, zs, err, acc);
  }
  float s[NA], cc[NA];
#pragma unroll
  for (int j = 0; j < NA; ++j) {
    s[j] = acc[j].s;
    cc[j] = acc[j].c;
  }
  block_sum_kahan_store<NA>(s, cc, out);
  if (PO && (int)threadIdx.x >= 2 && (int)threadIdx.x < kGreekAcc) out[threadIdx.x] = 0.0;
}

// Instance of an item: from the item map, or the last instance whose first
// item is <= item (binary search over the ordered item_begin).
__device__ __forceinline__ uint32_t inst_of_item(const GreeksLaunch& g, unsigned long long item) {
  if (g.item_inst) return g.item_inst[item];
  int lo = 0, hi = g.n_inst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.inst[mid].item_begin <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return (uint32_t)lo;
}

// A block serves items: the next from the queue counter (persistent grid) or
// item blockIdx.x (direct: one block per item, so blocks retire after one
// chunk and work on higher-priority streams gets SMs between them).
// 3 resident blocks per SM (80 registers instead of 124): the kernel is
// issue-bound like the fused pricing kernels, and the extra warps hide more
// of the generator's latency (512-instance batch 90 -> 84 ms on GB300).
__global__ void __launch_bounds__(256, 3) k_greeks(const GreeksLaunch g) {
  __shared__ ZigShared32 zs;
  __shared__ unsigned long long item_s;
  zig_stage32(zs, g.tabs);
  const SamplerCtx c{g.tabs, g.tabs->r32, g.tabs->r};
  unsigned err = 0;
  for (unsigned long long round = 0;; ++round) {
    unsigned long long item;
    if (g.direct) {
      if (round > 0) break;
      item = blockIdx.x;
    } else {
      if (threadIdx.x == 0) item_s = atomicAdd(g.counter, 1ull);
      __syncthreads();
      item = item_s;
      __syncthreads();  // item_s is rewritten next round
    }
    if (item >= g.total_items) break;
    const GInst& I = g.inst[inst_of_item(g, item)];
    const uint64_t lo = (item - I.item_begin) * I.chunk;
    uint64_t hi = lo + I.chunk;
    if (hi > I.n_paths) hi = I.n_paths;
    double* out = g.item_part + item * kGreekAcc;
    if (I.price_only)
      run_item<true>(I, lo, hi, c, zs, err, out);
    else
      run_item<false>(I, lo, hi, c, zs, err, out);
  }
  if (err) atomicOr(g.err, err);
}

// One block per instance: thread j adds the instance's items j, j + 256, ...
// in order, then a fixed block tree; the totals depend only on the
// instance's own items, never on what else is in the launch.
__global__ void __launch_bounds__(256) k_greeks_finish(const GreeksLaunch g) {
  const int i = blockIdx.x;
  if (i >= g.n_inst) return;
  const GInst& I = g.inst[i];
  const uint64_t items = (I.n_paths + I.chunk - 1) / I.chunk;
  double s[kGreekAcc];
#pragma unroll
  for (int j = 0; j < kGreekAcc; ++j) s[j] = 0.0;
  for (uint64_t it = threadIdx.x; it < items; it += blockDim.x) {
    const double* p = g.item_part + (I.item_begin + it) * kGreekAcc;
#pragma unroll
    for (int j = 0; j < kGreekAcc; ++j) s[j] += p[j];
  }
  block_sum_n_store<kGreekAcc>(s, g.inst_sums + (uint64_t)i * kGreekAcc);
}

}  // namespace

void launch_greeks_batch(const GreeksLaunch& g, cudaStream_t st) {
  int dev = 0, sms = 152, per_sm = 2;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_greeks, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 2;
  uint64_t blocks = (uint64_t)sms * per_sm;
  if (blocks > g.total_items || g.direct) blocks = g.total_items ? g.total_items : 1;
  if (!g.direct) cudaMemsetAsync(g.counter, 0, sizeof(unsigned long long), st);
  k_greeks<<<(unsigned)blocks, 256, 0, st>>>(g);
  if (g.n_inst > 0) k_greeks_finish<<<g.n_inst, 256, 0, st>>>(g);
}

}  // namespace stocha
