// Longstaff-Schwartz backward sweep (src/finance/lsmc.rs:25-115) on the GPU.
//
// Paths come from the GBM path kernel in time-major layout, spot[step][path],
// so every pass reads contiguous step columns.  The reference's per-step work
//   discount all cash flows                          lsmc.rs:52-54
//   ITM set, mean and std of its spots               lsmc.rs:57-71
//   least squares of discounted cash flow on powers  lsmc.rs:73-84
//   exercise where intrinsic > max(continuation, 0)  lsmc.rs:88-98
// is pipelined so that one pass over the paths serves a whole step: pass t
// does, per path, the exercise decision of step t+1 (coefficients solved at
// the end of the previous pass), the regression sums of step t (ITM
// statistics from the previous pass) and the ITM statistics of step t-1.
// Block partial sums are then combined in a fixed order, step t's normal
// equations are solved in FP64 (Hankel matrix of the power sums
// p_j = sum x^j, right-hand side q_j = sum x^j y, Cholesky) and step t-1's
// sums become its mean and std.  Passes: init (terminal cash flows,
// statistics of step steps-1), one per step, the mean and the variance of the
// discounted cash flows (lsmc.rs:100-112).
//
// Two launch forms of the same passes:
//   * multi-launch (large n): one grid-wide launch per pass; the last block
//     to finish (a counter, no waiting) combines the partials and solves.
//   * cluster (small and medium n): ONE launch of one thread-block cluster
//     runs every pass; blocks exchange partials through distributed shared
//     memory at the hardware cluster barrier and each block combines and
//     solves redundantly (same inputs, same order, same result).  No launch
//     per step, and the rest of the GPU stays free for other work.
//
// FP64 form (the plain method): all arithmetic in FP64 and cash flows
// discounted one step at a time as the reference does.
// FP32 form: spots, regression sums (per thread; FP64 from warp totals on) and
// decisions in FP32; a path carries its undiscounted exercise payoff and
// exercise step, and its value at step t is payoff * disc^(tau - t) with
// disc^j rounded once from FP64 (no compounding of FP32 roundings).  The solve,
// the estimator and the standard error stay in FP64.
//
// The reference solves by Householder QR (faer); the normal equations give
// the same coefficients to ~cond^2 * 1e-16, so exercise decisions differ only
// at near-ties.  Partials are combined in a fixed order: results are the same
// run to run and independent of other work on the device.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "lsmc_kernels.h"
#include "reduce.cuh"

namespace stocha {
namespace {

namespace cg = cooperative_groups;

constexpr int kThreads = 256;         // multi-launch blocks
constexpr int kClusterThreads = 512;  // cluster blocks
constexpr int kU = 4;                 // paths per thread whose loads are issued together
enum Mode : int { kInit = 0, kStep = 1, kFinal = 2, kVar = 3 };

__device__ __forceinline__ float mx(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double mx(double a, double b) { return fmax(a, b); }

template <typename T>
__device__ __forceinline__ T intrinsic(T s, T k, int is_put) {  // lsmc.rs:117-123
  return is_put ? mx(k - s, T(0)) : mx(s - k, T(0));
}

__device__ __forceinline__ float warp_sum_t(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_t(double v) { return warp_sum(v); }

// Cash flow of one path: FP64 form, the discounted value; FP32 form, the
// undiscounted payoff (bits) and its exercise step.
template <typename T>
struct Cf;
template <>
struct Cf<double> {
  using type = double;
};
template <>
struct Cf<float> {
  using type = uint2;
};

template <typename T>
struct StepView {
  T mean, inv, c[5];
  int skip;
};

template <typename T>
__device__ __forceinline__ StepView<T> view(const LsmcStep& s);
template <>
__device__ __forceinline__ StepView<double> view<double>(const LsmcStep& s) {
  StepView<double> v;
  v.mean = s.mean;
  v.inv = s.inv_std;
#pragma unroll
  for (int j = 0; j < 5; ++j) v.c[j] = s.coef[j];
  v.skip = s.skip;
  return v;
}
template <>
__device__ __forceinline__ StepView<float> view<float>(const LsmcStep& s) {
  StepView<float> v;
  v.mean = s.mean_f;
  v.inv = s.inv_f;
#pragma unroll
  for (int j = 0; j < 5; ++j) v.c[j] = s.coef_f[j];
  v.skip = s.skip;
  return v;
}

template <typename T>
__device__ __forceinline__ StepView<T> no_step() {
  StepView<T> v;
  v.mean = T(0);
  v.inv = T(0);
#pragma unroll
  for (int j = 0; j < 5; ++j) v.c[j] = T(0);
  v.skip = 1;
  return v;
}

// Continuation value sum_j c_j x^j (lsmc.rs:91-93).
template <typename T, int DEG>
__device__ __forceinline__ T continuation(const StepView<T>& P, T x) {
  T cont = P.c[0], xp = T(1);
#pragma unroll
  for (int j = 1; j <= DEG; ++j) {
    xp *= x;
    cont += P.c[j] * xp;
  }
  return cont;
}

// Exercise decision of one path at a step with regression P: ITM and the
// intrinsic value above max(continuation, 0) (lsmc.rs:88-98).
template <typename T, int DEG>
__device__ __forceinline__ bool decide(const StepView<T>& P, T s, T k, int is_put, T* ex_out) {
  if (P.skip) return false;
  const T ex = intrinsic(s, k, is_put);
  if (!(ex > T(0))) return false;
  const T x = (s - P.mean) * P.inv;
  *ex_out = ex;
  return ex > mx(continuation<T, DEG>(P, x), T(0));
}

// Value at step t of a cash flow (FP64: already discounted to t).
__device__ __forceinline__ double value_at(double c, uint64_t, const float*) { return c; }
__device__ __forceinline__ float value_at(uint2 c, uint64_t t, const float* dpow) {
  return __uint_as_float(c.x) * dpow[c.y - (unsigned)t];
}

// Applies the decision of step `ustep` to cash flow c (FP64: then one discount).
template <typename T, int DEG>
__device__ __forceinline__ bool apply_decision(typename Cf<T>::type& c, const StepView<T>& P1, T s1, T k,
                                               int is_put, double disc, unsigned ustep) {
  T ex = T(0);
  const bool exer = decide<T, DEG>(P1, s1, k, is_put, &ex);
  if constexpr (sizeof(T) == 8) {
    c = (exer ? ex : c) * disc;
    return true;  // always rewritten (discount)
  } else {
    if (exer) c = make_uint2(__float_as_uint(ex), ustep);
    return exer;
  }
}

// Init pass (step = steps) or step pass t over paths i0, i0 + stride, ...:
// cash-flow init or the decision of step t+1, regression sums of step t into
// vals[0..13], ITM statistics of step u (u >= 1) into vals[14..16].
template <typename T, int DEG>
__device__ __forceinline__ void step_paths(const LsmcLaunch& a, uint64_t t, bool init, bool dec,
                                           const StepView<T>& P1, const StepView<T>& P, uint64_t u,
                                           const float* dpow, uint64_t i0, uint64_t stride, T* vals) {
  using C = typename Cf<T>::type;
  const T* spot = (const T*)a.spot;
  C* cf = (C*)a.cf;
  const uint64_t n = a.n;
  const T k = (T)a.k;
  const int is_put = a.is_put;
  const T* col_a = spot + (init ? a.steps : t + 1) * n;  // terminal column, or step t+1
  const T* col_t = spot + t * n;
  const T* col_u = spot + u * n;
  const bool reg = !init && !P.skip;
  const bool stats = u >= 1;
  for (uint64_t base = i0; base < n; base += stride * kU) {
    C c[kU];
    T s1[kU], s[kU], su[kU];
#pragma unroll
    for (int q = 0; q < kU; ++q) {  // all loads of the batch before any store
      const uint64_t i = base + q * stride;
      if constexpr (sizeof(T) == 8)
        c[q] = 0.0;
      else
        c[q] = make_uint2(0u, 0u);
      s1[q] = s[q] = su[q] = T(0);
      if (i < n) {
        if (!init) c[q] = cf[i];
        if (init || dec) s1[q] = col_a[i];
        if (reg) s[q] = col_t[i];
        if (stats) su[q] = col_u[i];
      }
    }
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      const uint64_t i = base + q * stride;
      if (i < n) {
        if (init) {
          const T ex = intrinsic(s1[q], k, is_put);
          if constexpr (sizeof(T) == 8)
            cf[i] = ex * a.disc;  // lsmc.rs:44-47, then the first discount (:52-54)
          else
            cf[i] = make_uint2(__float_as_uint(ex), (unsigned)a.steps);
        } else if (dec) {
          if (apply_decision<T, DEG>(c[q], P1, s1[q], k, is_put, a.disc, (unsigned)(t + 1))) cf[i] = c[q];
        }
        if (reg && intrinsic(s[q], k, is_put) > T(0)) {
          const T x = (s[q] - P.mean) * P.inv;
          const T y = value_at(c[q], t, dpow);
          T xp = T(1);
#pragma unroll
          for (int j = 0; j <= 2 * DEG; ++j) {
            vals[j] += xp;
            if (j <= DEG) vals[9 + j] += xp * y;
            xp *= x;
          }
        }
        if (stats && intrinsic(su[q], k, is_put) > T(0)) {
          const T d = su[q] - k;
          vals[14] += T(1);
          vals[15] += d;
          vals[16] += d * d;
        }
      }
    }
  }
}

// Final passes: with `dec`, the decision of step 1 (and the last discount)
// then the sum of the values at time 0; with `var`, the sum of squared
// deviations from `mean` (lsmc.rs:100-112).
template <typename T, int DEG>
__device__ __forceinline__ double final_paths(const LsmcLaunch& a, bool var, double mean, bool dec,
                                              const StepView<T>& P1, const float* dpow, uint64_t i0,
                                              uint64_t stride) {
  using C = typename Cf<T>::type;
  const T* col1 = (const T*)a.spot + a.n;
  C* cf = (C*)a.cf;
  const uint64_t n = a.n;
  const T k = (T)a.k;
  double s = 0.0;
  for (uint64_t base = i0; base < n; base += stride * kU) {
    C c[kU];
    T s1[kU];
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      const uint64_t i = base + q * stride;
      if constexpr (sizeof(T) == 8)
        c[q] = 0.0;
      else
        c[q] = make_uint2(0u, 0u);
      s1[q] = T(0);
      if (i < n) {
        c[q] = cf[i];
        if (dec) s1[q] = col1[i];
      }
    }
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      const uint64_t i = base + q * stride;
      if (i < n) {
        if (dec && apply_decision<T, DEG>(c[q], P1, s1[q], k, a.is_put, a.disc, 1u)) cf[i] = c[q];
        const double v = (double)value_at(c[q], 0, dpow);
        if (var)
          s = fma(v - mean, v - mean, s);
        else
          s += v;
      }
    }
  }
  return s;
}

// Block totals of vals[0..NV) into out[0..NV) (threads < NV write).  FP32
// values are summed in FP32 within the block (warp tree, then the warps in
// order) and converted once: FP64 instructions issue at 1/64 of the FP32 rate
// on this GPU, so a conversion per warp and value would dominate the pass.
// Every thread of the block must call it.
template <typename T, int NV>
__device__ __forceinline__ void block_reduce(const T* vals, double* out) {
  __shared__ T red[32][kLsmcValues];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // a previous call's readers of red are done
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const T w = warp_sum_t(vals[v]);
    if (lane == 0) red[wid][v] = w;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    T s = T(0);
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    out[threadIdx.x] = (double)s;
  }
}

// tot[v] = sum over rows r < nrows of row(r, v), v < NV, in a fixed order:
// four lanes per value (rows r = j, j+4, ... for lane j of the group), then
// the four in order.  Threads below 4*NV rounded up to whole warps take
// part (the block has at least that many); ends with a barrier.
template <int NV, typename Row>
__device__ __forceinline__ void combine_rows(Row row, int nrows, double* tot) {
  const int v = threadIdx.x >> 2, j = threadIdx.x & 3;
  if ((int)threadIdx.x < ((4 * NV + 31) & ~31)) {  // whole warps
    double s = 0.0;
    if (v < NV)
      for (int r = j; r < nrows; r += 4) s += row(r, v);
    s += __shfl_down_sync(0xffffffffu, s, 1, 4);
    s += __shfl_down_sync(0xffffffffu, s, 2, 4);
    if (v < NV && j == 0) tot[v] = s;
  }
  __syncthreads();
}

// Multi-launch: counts one finished cluster; true in the last one, which then
// sees every cluster's row.  Called by the whole rank-0 block.
__device__ __forceinline__ bool arrive_last(unsigned* counter, unsigned nclusters, bool* last_s) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *last_s = atomicAdd(counter, 1u) == nclusters - 1;
  __syncthreads();
  if (*last_s) __threadfence();
  return *last_s;
}

// Mean and std of step u's ITM spots from (count, sum(s-k), sum(s-k)^2):
// ITM spots lie on one side of the strike, so the shifted one-pass moments
// lose nothing to cancellation (lsmc.rs:61-71).
__device__ void finish_stats(const double* tot, int ncols, double k, LsmcStep* st) {
  const double m = tot[14];
  st->m = m;
  st->skip = m < (double)(ncols + 1);  // lsmc.rs:62-64
  const double d = m > 0.0 ? tot[15] / m : 0.0;
  st->mean = k + d;
  const double var = m > 0.0 ? fmax(tot[16] / m - d * d, 0.0) : 0.0;
  st->std = fmax(sqrt(var), 1e-12);  // lsmc.rs:68-71
  st->inv_std = 1.0 / st->std;
  st->mean_f = (float)st->mean;
  st->inv_f = (float)st->inv_std;
}

// FP64 Cholesky solve of Hankel(p) c = q, (deg+1) unknowns; one division per
// pivot (reciprocal of the diagonal).
__device__ void solve_normal(const double* tot, int deg, LsmcStep* st) {
  const int nc = deg + 1;
  double L[25] = {0}, inv[5], w[5], c[5];
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = tot[i + j];
      for (int kk = 0; kk < j; ++kk) s -= L[i * 5 + kk] * L[j * 5 + kk];
      if (i == j) {
        const double d = sqrt(s);
        L[i * 5 + i] = d;
        inv[i] = 1.0 / d;
      } else {
        L[i * 5 + j] = s * inv[j];
      }
    }
  for (int i = 0; i < nc; ++i) {
    double s = tot[9 + i];
    for (int kk = 0; kk < i; ++kk) s -= L[i * 5 + kk] * w[kk];
    w[i] = s * inv[i];
  }
  for (int i = nc - 1; i >= 0; --i) {
    double s = w[i];
    for (int kk = i + 1; kk < nc; ++kk) s -= L[kk * 5 + i] * c[kk];
    c[i] = s * inv[i];
  }
  for (int i = 0; i < 5; ++i) {
    st->coef[i] = i < nc ? c[i] : 0.0;
    st->coef_f[i] = (float)st->coef[i];
  }
}

// Solve of step t (warp 0) and statistics of step u (warp 1), in parallel.
__device__ __forceinline__ void finish_pass(const double* tot, bool solve, LsmcStep* ps, bool stats, LsmcStep* pu,
                                            int deg, double k) {
  if (solve && threadIdx.x == 0) solve_normal(tot, deg, ps);
  if (stats && threadIdx.x == 32) finish_stats(tot, deg + 1, k, pu);
}

// ------------------------------------------------------------ multi-launch ---
// Launched in clusters of kMultiCluster blocks: rank 0 of each cluster adds
// its blocks' totals (distributed shared memory, rank order) into one row,
// and the last cluster to finish adds the rows, so the final FP64 combine
// runs over gridDim/kMultiCluster rows instead of gridDim.
constexpr int kMultiCluster = 8;

template <typename T, int DEG>
__global__ void __launch_bounds__(kThreads) k_lsmc(const LsmcLaunch* __restrict__ ap, uint64_t t, int mode) {
  const LsmcLaunch& a = *ap;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank(), csz = cluster.num_blocks();
  const unsigned cid = blockIdx.x / csz, ncl = gridDim.x / csz;
  __shared__ double bsum[kLsmcValues];
  __shared__ double tot[kLsmcValues];
  __shared__ bool last;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool fin = mode == kFinal || mode == kVar;
  const bool init = mode == kInit;
  const uint64_t u = init ? a.steps - 1 : (fin ? 0 : t - 1);  // statistics of step u (u >= 1)
  StepView<T> P = no_step<T>();
  if (fin) {
    const bool dec = mode == kFinal && a.steps >= 2;
    const StepView<T> P1 = dec ? view<T>(a.step_params[1]) : no_step<T>();
    const double mean = mode == kVar ? __ldcg(a.result) : 0.0;
    const double s = final_paths<T, DEG>(a, mode == kVar, mean, dec, P1, a.dpow, i0, stride);
    block_reduce<double, 1>(&s, bsum);
  } else {
    const bool dec = !init && t + 1 <= a.steps - 1;
    const StepView<T> P1 = dec ? view<T>(a.step_params[t + 1]) : no_step<T>();
    if (!init) P = view<T>(a.step_params[t]);
    if constexpr (sizeof(T) == 4) {
      if (init)
        for (uint64_t j = i0; j <= a.steps; j += stride) a.dpow[j] = (float)exp(a.log_disc * (double)j);
    }
    T vals[kLsmcValues];
#pragma unroll
    for (int v = 0; v < kLsmcValues; ++v) vals[v] = T(0);
    step_paths<T, DEG>(a, init ? a.steps : t, init, dec, P1, P, u, a.dpow, i0, stride, vals);
    block_reduce<T, kLsmcValues>(vals, bsum);
  }
  const int nv = fin ? 1 : kLsmcValues;
  cluster.sync();
  if (rank == 0 && (int)threadIdx.x < nv) {
    double s = 0.0;
    for (unsigned r = 0; r < csz; ++r) s += cluster.map_shared_rank(bsum, r)[threadIdx.x];
    a.part[(uint64_t)cid * kLsmcValues + threadIdx.x] = s;
  }
  cluster.sync();  // remote reads done before any block of the cluster leaves
  if (rank != 0) return;
  if (!arrive_last(a.counter, ncl, &last)) return;
  const double* part = a.part;
  auto row = [part](int r, int v) { return __ldcg(part + (uint64_t)r * kLsmcValues + v); };
  if (fin) {
    combine_rows<1>(row, (int)ncl, tot);
    if (threadIdx.x == 0) {
      if (mode == kFinal)
        a.result[0] = tot[0] / (double)a.n;
      else
        a.result[1] = tot[0];
      *a.counter = 0;
    }
    return;
  }
  combine_rows<kLsmcValues>(row, (int)ncl, tot);
  finish_pass(tot, !init && !P.skip, a.step_params + t, u >= 1, a.step_params + u, DEG, a.k);
  if (threadIdx.x == 0) *a.counter = 0;
}

// ----------------------------------------------------------------- cluster ---
// The grid is exactly one cluster.  Step parameters rotate through three
// shared slots (step s in slot s % 3); partials are double-buffered so that a
// block never overwrites values another block may still be reading.
template <typename T, int DEG>
__global__ void __launch_bounds__(kClusterThreads, 1) k_lsmc_cluster(const __grid_constant__ LsmcLaunch a) {
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned C = gridDim.x;
  extern __shared__ float dpow_s[];  // FP32 form: disc^j, j = 0..steps
  __shared__ double part[2][kLsmcValues];
  __shared__ double tot[kLsmcValues];
  __shared__ LsmcStep prm[3];
  const uint64_t steps = a.steps;
  const uint64_t stride = (uint64_t)C * blockDim.x;
  const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float* dpow = nullptr;
  if constexpr (sizeof(T) == 4) {
    for (uint64_t j = threadIdx.x; j <= steps; j += blockDim.x) dpow_s[j] = (float)exp(a.log_disc * (double)j);
    dpow = dpow_s;
  }
  int buf = 0;
  // tot[0..NV) = sum over cluster ranks (in rank order) of part[buf]
  auto combine = [&](auto nv_tag) {
    constexpr int NV = decltype(nv_tag)::value;
    cluster.sync();
    const double* mine = &part[buf][0];
    auto row = [&cluster, mine](int r, int v) { return cluster.map_shared_rank(mine, (unsigned)r)[v]; };
    combine_rows<NV>(row, (int)C, tot);
  };
  using All = std::integral_constant<int, kLsmcValues>;
  using One = std::integral_constant<int, 1>;

  {  // init pass
    T vals[kLsmcValues];
#pragma unroll
    for (int v = 0; v < kLsmcValues; ++v) vals[v] = T(0);
    const StepView<T> none = no_step<T>();
    step_paths<T, DEG>(a, steps, true, false, none, none, steps - 1, dpow, i0, stride, vals);
    block_reduce<T, kLsmcValues>(vals, part[buf]);
    combine(All{});
    finish_pass(tot, false, nullptr, steps >= 2, &prm[(steps - 1) % 3], DEG, a.k);
    __syncthreads();
    buf ^= 1;
  }
  for (uint64_t t = steps - 1; t >= 1; --t) {
    T vals[kLsmcValues];
#pragma unroll
    for (int v = 0; v < kLsmcValues; ++v) vals[v] = T(0);
    const bool dec = t + 1 <= steps - 1;
    const StepView<T> P1 = dec ? view<T>(prm[(t + 1) % 3]) : no_step<T>();
    const StepView<T> P = view<T>(prm[t % 3]);
    step_paths<T, DEG>(a, t, false, dec, P1, P, t - 1, dpow, i0, stride, vals);
    block_reduce<T, kLsmcValues>(vals, part[buf]);
    combine(All{});
    finish_pass(tot, !P.skip, &prm[t % 3], t >= 2, &prm[(t - 1) % 3], DEG, a.k);
    __syncthreads();
    buf ^= 1;
  }
  double mean;
  {  // decision of step 1, last discount, mean
    const bool dec = steps >= 2;
    const StepView<T> P1 = dec ? view<T>(prm[1 % 3]) : no_step<T>();
    const double s = final_paths<T, DEG>(a, false, 0.0, dec, P1, dpow, i0, stride);
    block_reduce<double, 1>(&s, part[buf]);
    combine(One{});
    mean = tot[0] / (double)a.n;
    buf ^= 1;
  }
  {  // sum of squared deviations
    const double s = final_paths<T, DEG>(a, true, mean, false, no_step<T>(), dpow, i0, stride);
    block_reduce<double, 1>(&s, part[buf]);
    combine(One{});
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.result[0] = mean;
      a.result[1] = tot[0];
    }
  }
  cluster.sync();  // no block leaves while another may still read its shared memory
}

cudaLaunchConfig_t cluster_config(unsigned grid, unsigned block, size_t smem, unsigned csize, cudaStream_t st,
                                  cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// Multi-launch passes as one instantiated graph per shape (see LsmcGraphs).
template <typename T, int DEG>
cudaError_t sweep_multi(const LsmcLaunch& a0, cudaStream_t st, LsmcGraphs* G) {
  if (!G) return cudaErrorInvalidValue;
  // one wave of whole clusters: no more than are resident at once (a.grid
  // sized the partial rows; fewer clusters use fewer of them)
  auto fn = k_lsmc<T, DEG>;
  cudaLaunchAttribute attr[1];
  static int max_clusters = 0;
  if (max_clusters == 0) {
    cudaLaunchConfig_t probe = cluster_config(kMultiCluster, kThreads, 0, kMultiCluster, st, attr);
    int v = 0;
    if (cudaOccupancyMaxActiveClusters(&v, fn, &probe) != cudaSuccess || v < 1) v = 1;
    cudaGetLastError();
    max_clusters = v;
  }
  uint64_t want = ((uint64_t)a0.grid + kMultiCluster - 1) / kMultiCluster;
  if (want > (uint64_t)max_clusters) want = max_clusters;
  if (want < 1) want = 1;
  const unsigned g = (unsigned)want * kMultiCluster;

  LsmcLaunch a = a0;
  a.counter = (unsigned*)(G->d_params + 1);
  *G->h_params = a;  // read by the graph's first node when it runs
  const int f32 = sizeof(T) == 4;
  for (int i = 0; i < G->n_cache; ++i) {
    const LsmcGraphs::Entry& e = G->cache[i];
    if (e.steps == a.steps && e.deg == DEG && e.f32 == f32 && e.grid == (int)g) return cudaGraphLaunch(e.exec, st);
  }
  // params upload, counter reset, steps + 2 passes
  auto enqueue = [&](cudaStream_t s) {
    cudaMemcpyAsync(G->d_params, G->h_params, sizeof(LsmcLaunch), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(a.counter, 0, sizeof(unsigned), s);
    cudaLaunchConfig_t cfg = cluster_config(g, kThreads, 0, kMultiCluster, s, attr);
    const LsmcLaunch* ap = G->d_params;
    cudaLaunchKernelEx(&cfg, fn, ap, (uint64_t)a.steps, (int)kInit);
    for (uint64_t t = a.steps - 1; t >= 1; --t) cudaLaunchKernelEx(&cfg, fn, ap, t, (int)kStep);
    cudaLaunchKernelEx(&cfg, fn, ap, (uint64_t)0, (int)kFinal);
    cudaLaunchKernelEx(&cfg, fn, ap, (uint64_t)0, (int)kVar);
  };
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();  // a stream that cannot be captured (the legacy default stream): plain launches
    enqueue(st);
    return cudaGetLastError();
  }
  enqueue(st);
  cudaGraph_t graph = nullptr;
  cudaError_t err = cudaStreamEndCapture(st, &graph);
  if (err) return err;
  cudaGraphExec_t exec = nullptr;
  err = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (err) return err;
  int slot;
  if (G->n_cache < 8) {
    slot = G->n_cache++;
  } else {  // replace the oldest (an exec still running is freed when it completes)
    slot = G->next;
    G->next = (G->next + 1) % 8;
    cudaGraphExecDestroy(G->cache[slot].exec);
  }
  G->cache[slot] = LsmcGraphs::Entry{a.steps, DEG, f32, (int)g, exec};
  return cudaGraphLaunch(exec, st);
}

template <typename T, int DEG>
cudaError_t sweep_cluster(const LsmcLaunch& a, cudaStream_t st) {
  auto fn = k_lsmc_cluster<T, DEG>;
  const size_t smem = sizeof(T) == 4 ? (a.steps + 1) * sizeof(float) : 0;
  cudaError_t e;
  if (a.cluster > 8 && (e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)))
    return e;
  if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config((unsigned)a.cluster, kClusterThreads, smem, (unsigned)a.cluster, st, attr);
  return cudaLaunchKernelEx(&cfg, fn, a);
}

template <typename T, int DEG>
cudaError_t sweep(const LsmcLaunch& a, cudaStream_t st, LsmcGraphs* G) {
  return a.cluster > 0 ? sweep_cluster<T, DEG>(a, st) : sweep_multi<T, DEG>(a, st, G);
}

template <typename T>
cudaError_t sweep_deg(const LsmcLaunch& a, cudaStream_t st, LsmcGraphs* G) {
  switch (a.deg) {
    case 1: return sweep<T, 1>(a, st, G);
    case 2: return sweep<T, 2>(a, st, G);
    case 3: return sweep<T, 3>(a, st, G);
    default: return sweep<T, 4>(a, st, G);
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

int lsmc_grid(uint64_t n, int sms) {
  // one wave: 4 blocks of 256 threads per SM (<= 64 registers a thread)
  const uint64_t want = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)sms * 4;
  return (int)(want < cap ? (want ? want : 1) : cap);
}

int lsmc_cluster_size(uint64_t n, uint64_t steps, int f32) {
  // FP64 arithmetic issues at 1/64 of the FP32 rate: the FP64 form uses the
  // whole GPU sooner
  const uint64_t max_paths = f32 ? kLsmcClusterMaxPaths : kLsmcClusterMaxPaths / 32;
  if (n > max_paths || steps + 1 > kLsmcClusterMaxSteps) return 0;
  static int size = -1;  // 16 where the device schedules 16-block clusters, else 8
  if (size < 0) {
    int s = 8;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(16, kClusterThreads, kLsmcClusterMaxSteps * sizeof(float), 16, 0, attr);
    auto fn = k_lsmc_cluster<float, 4>;
    int clusters = 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kLsmcClusterMaxSteps * sizeof(float))) == cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess && clusters >= 1)
      s = 16;
    cudaGetLastError();
    size = s;
  }
  return size;
}

size_t lsmc_scratch_bytes(uint64_t n, uint64_t steps, int grid) {
  return align256(n * 8) + align256((size_t)grid * kLsmcValues * 8) + align256((steps + 1) * sizeof(LsmcStep)) +
         align256((steps + 1) * 4) + 256 + 256;
}

void lsmc_bind_scratch(LsmcLaunch* a, void* scratch) {
  char* p = (char*)scratch;
  a->cf = p;
  p += align256(a->n * 8);
  a->part = (double*)p;
  p += align256((size_t)a->grid * kLsmcValues * 8);
  a->step_params = (LsmcStep*)p;
  p += align256((a->steps + 1) * sizeof(LsmcStep));
  a->dpow = (float*)p;
  p += align256((a->steps + 1) * 4);
  a->counter = (unsigned*)p;
  p += 256;
  a->result = (double*)p;
}

cudaError_t lsmc_graphs_create(LsmcGraphs** out) {
  LsmcGraphs* g = new LsmcGraphs();
  cudaError_t e;
  if ((e = cudaMalloc((void**)&g->d_params, sizeof(LsmcLaunch) + 256)) ||
      (e = cudaMallocHost((void**)&g->h_params, sizeof(LsmcLaunch)))) {
    lsmc_graphs_destroy(g);
    *out = nullptr;
    return e;
  }
  *out = g;
  return cudaSuccess;
}

void lsmc_graphs_destroy(LsmcGraphs* g) {
  if (!g) return;
  for (int i = 0; i < g->n_cache; ++i)
    if (g->cache[i].exec) cudaGraphExecDestroy(g->cache[i].exec);
  if (g->d_params) cudaFree(g->d_params);
  if (g->h_params) cudaFreeHost(g->h_params);
  delete g;
}

cudaError_t lsmc_sweep(const LsmcLaunch& a, cudaStream_t st, LsmcGraphs* graphs) {
  return a.spot_f32 ? sweep_deg<float>(a, st, graphs) : sweep_deg<double>(a, st, graphs);
}

}  // namespace stocha
