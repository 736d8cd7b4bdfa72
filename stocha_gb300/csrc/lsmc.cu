// Longstaff-Schwartz backward sweep (src/finance/lsmc.rs:25-115) on the GPU.
//
// Paths come from the GBM path kernel in time-major layout, spot[step][path],
// so every pass below reads one contiguous step column (at 4e6 paths a column
// plus the cash flows fit in L2).  Per backward step k:
//   k_stats   ITM count and strike-shifted sums of spot[k]   lsmc.rs:57-71
//   k_merge3  one thread: fixed-order totals -> mean, std, skip flag
//             (#ITM < ncols + 1)                             lsmc.rs:61-71
//   k_gram    power sums p_j = sum x^j (j <= 2*deg) and q_j = sum x^j y over
//             ITM paths, x = (s - mean)/std: the normal equations of the
//             reference's regression (X^T X = Hankel(p), X^T y = q)
//   k_solve   one thread: FP64 Cholesky solve of the (deg+1)^2 system
//   k_update  exercise where intrinsic > max(continuation, 0), then the
//             next step's discount                          lsmc.rs:91-98,52-54
// The reference solves by Householder QR (faer); the normal equations give
// the same coefficients to ~cond^2 * 1e-16, so exercise decisions differ
// only at near-ties.  All step parameters stay on the device: the sweep is
// a fixed sequence of launches with no host round trip.
#include <cuda_runtime.h>

#include "lsmc_kernels.h"
#include "reduce.cuh"

namespace stocha {
namespace {

__device__ __forceinline__ double intrinsic(double s, double k, int is_put) {  // lsmc.rs:117-123
  return is_put ? fmax(k - s, 0.0) : fmax(s - k, 0.0);
}

template <typename T>
__global__ void __launch_bounds__(256) k_init(const T* __restrict__ spot_T, uint64_t n, double k, int is_put,
                                              double disc, double* __restrict__ cf) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    cf[i] = intrinsic((double)spot_T[i], k, is_put) * disc;
}

// ITM count and sums of (s - k), (s - k)^2: ITM spots lie on one side of
// the strike, so the shifted one-pass moments lose nothing to cancellation.
template <typename T>
__global__ void __launch_bounds__(256) k_stats(const T* __restrict__ spot, uint64_t n, double k, int is_put,
                                               double* __restrict__ part) {
  double cn = 0.0, s1 = 0.0, s2 = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double s = (double)spot[i];
    if (intrinsic(s, k, is_put) > 0.0) {
      const double d = s - k;
      cn += 1.0;
      s1 += d;
      s2 = fma(d, d, s2);
    }
  }
  __shared__ double red[32][3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  cn = warp_sum(cn);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    red[wid][0] = cn;
    red[wid][1] = s1;
    red[wid][2] = s2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
    part[3 * (uint64_t)blockIdx.x + threadIdx.x] = t;
  }
}

__global__ void k_merge3(const double* __restrict__ part, int nb, int ncols, double k, LsmcStep* __restrict__ st) {
  if (threadIdx.x != 0) return;
  double m = 0.0, s1 = 0.0, s2 = 0.0;
  for (int i = 0; i < nb; ++i) {
    m += part[3 * i];
    s1 += part[3 * i + 1];
    s2 += part[3 * i + 2];
  }
  st->skip = m < (double)(ncols + 1);  // lsmc.rs:62-64
  st->m = m;
  const double d = m > 0.0 ? s1 / m : 0.0;
  st->mean = k + d;
  const double var = m > 0.0 ? fmax(s2 / m - d * d, 0.0) : 0.0;
  st->std = fmax(sqrt(var), 1e-12);  // lsmc.rs:68-71
  st->inv_std = 1.0 / st->std;
}

template <typename T>
__global__ void __launch_bounds__(256) k_gram(const T* __restrict__ spot, const double* __restrict__ cf, uint64_t n,
                                              double k, int is_put, int deg, const LsmcStep* __restrict__ st,
                                              double* __restrict__ part) {
  if (st->skip) return;
  const double mean = st->mean, inv = st->inv_std;
  double p[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, q[5] = {0, 0, 0, 0, 0};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double s = (double)spot[i];
    if (intrinsic(s, k, is_put) > 0.0) {
      const double x = (s - mean) * inv;
      const double y = cf[i];
      double xp = 1.0;
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        if (j <= 2 * deg) p[j] += xp;
        if (j <= deg) q[j] += xp * y;
        xp *= x;
      }
    }
  }
  // block reduce 14 values (fixed order)
  __shared__ double red[32][14];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 14; ++j) {
    double v = j < 9 ? p[j] : q[j - 9];
    v = warp_sum(v);
    if (lane == 0) red[wid][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 14) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    part[14 * (uint64_t)blockIdx.x + threadIdx.x] = s;
  }
}

__global__ void k_solve(const double* __restrict__ part, int nb, int deg, LsmcStep* __restrict__ st) {
  __shared__ double tot[14];
  if (threadIdx.x < 14) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[14 * (uint64_t)b + threadIdx.x];
    tot[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0 || st->skip) return;
  const int nc = deg + 1;
  double G[25], L[25] = {0}, w[5], c[5];
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j) G[i * 5 + j] = tot[i + j];
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = G[i * 5 + j];
      for (int kk = 0; kk < j; ++kk) s -= L[i * 5 + kk] * L[j * 5 + kk];
      L[i * 5 + j] = (i == j) ? sqrt(s) : s / L[j * 5 + j];
    }
  for (int i = 0; i < nc; ++i) {
    double s = tot[9 + i];
    for (int kk = 0; kk < i; ++kk) s -= L[i * 5 + kk] * w[kk];
    w[i] = s / L[i * 5 + i];
  }
  for (int i = nc - 1; i >= 0; --i) {
    double s = w[i];
    for (int kk = i + 1; kk < nc; ++kk) s -= L[kk * 5 + i] * c[kk];
    c[i] = s / L[i * 5 + i];
  }
  for (int i = 0; i < 5; ++i) st->coef[i] = i < nc ? c[i] : 0.0;
}

template <typename T>
__global__ void __launch_bounds__(256) k_update(const T* __restrict__ spot, double* __restrict__ cf, uint64_t n,
                                                double k, int is_put, int deg, double disc,
                                                const LsmcStep* __restrict__ st) {
  const bool skip = st->skip;
  const double mean = st->mean, inv = st->inv_std;
  double c[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) c[j] = st->coef[j];
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    double v = cf[i];
    if (!skip) {
      const double s = (double)spot[i];
      const double ex = intrinsic(s, k, is_put);
      if (ex > 0.0) {
        const double x = (s - mean) * inv;
        double cont = 0.0, xp = 1.0;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          if (j <= deg) cont += c[j] * xp;
          xp *= x;
        }
        if (ex > fmax(cont, 0.0)) v = ex;
      }
    }
    cf[i] = v * disc;
  }
}

// sum (mode 0) or sum of (c - mean)^2 (mode 1) of the cash flows
__global__ void __launch_bounds__(256) k_cf_sum(const double* __restrict__ cf, uint64_t n, int mode,
                                                const double* __restrict__ mean_p, double* __restrict__ part) {
  const double mean = mode ? *mean_p : 0.0;
  double s = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double d = cf[i] - mean;
    s += mode ? d * d : cf[i];
  }
  block_sum2_store(s, 0.0, part + 2 * (uint64_t)blockIdx.x);
}

// one block: total of partials[2*b] -> out[0] = total / n (mode 0) or total (mode 1)
__global__ void k_cf_total(const double* __restrict__ part, int nb, uint64_t n, int mode, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[2 * b];
  out[mode] = mode ? s : s / (double)n;
}

}  // namespace

template <typename T>
void lsmc_sweep_impl(const LsmcLaunch& a, cudaStream_t st) {
  const T* spot = (const T*)a.spot;
  const int g = a.grid;
  k_init<T><<<g, 256, 0, st>>>(spot + (uint64_t)a.steps * a.n, a.n, a.k, a.is_put, a.disc, a.cf);
  for (uint64_t step = a.steps - 1; step >= 1; --step) {
    const T* col = spot + step * a.n;
    LsmcStep* sp = a.step_params + step;
    k_stats<T><<<g, 256, 0, st>>>(col, a.n, a.k, a.is_put, a.part);
    k_merge3<<<1, 32, 0, st>>>(a.part, g, a.deg + 1, a.k, sp);
    k_gram<T><<<g, 256, 0, st>>>(col, a.cf, a.n, a.k, a.is_put, a.deg, sp, a.part);
    k_solve<<<1, 32, 0, st>>>(a.part, g, a.deg, sp);
    k_update<T><<<g, 256, 0, st>>>(col, a.cf, a.n, a.k, a.is_put, a.deg, a.disc, sp);
  }
  k_cf_sum<<<g, 256, 0, st>>>(a.cf, a.n, 0, nullptr, a.part);
  k_cf_total<<<1, 32, 0, st>>>(a.part, g, a.n, 0, a.result);
  k_cf_sum<<<g, 256, 0, st>>>(a.cf, a.n, 1, a.result, a.part);
  k_cf_total<<<1, 32, 0, st>>>(a.part, g, a.n, 1, a.result);
}

void lsmc_sweep(const LsmcLaunch& a, cudaStream_t st) {
  if (a.spot_f32)
    lsmc_sweep_impl<float>(a, st);
  else
    lsmc_sweep_impl<double>(a, st);
}

}  // namespace stocha
