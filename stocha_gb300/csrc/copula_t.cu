// Student-t copula (src/copula/student_t.rs:93-170) from ONE sequential
// stream, Pcg64Dxsm::new(seed), in parallel.
//
// A sample consumes a variable number of draws: chi-square(nu) by
// Marsaglia-Tsang's gamma sampler (student_t.rs:93-124: normal, cube,
// uniform, squeeze or log test, repeat on rejection), then `dim` normals.
// Its consumption depends only on the draws, so the stream is cut into
// chunks of C draws and each chunk is parsed from E candidate entry offsets
// at once (k_tparse: samples starting in the chunk, and where the last one
// ends).  The true entries are then chained through groups of chunks
// (k_tcompose, k_ttop, k_tfill; a chunk whose entry lies beyond the
// candidates is parsed where it is met), k_temit re-parses every chunk from
// its true entry and stores each sample's chi-square and normals, and k_tcdf
// forms the uniforms u = T_nu((L z)_j * sqrt(nu / chi2)) with the
// reference's Student-t CDF (regularized incomplete beta by the
// modified-Lentz continued fraction, Lanczos log-gamma formed on the host;
// student_t.rs:6-91).  Every accept/reject decision uses the reference's FP64
// values (exact normals; ln in the gamma test from the device libm); the CDF
// differs from the reference's by rounding only (Newton reciprocals, host
// coefficients).
#include <cuda_runtime.h>

#include <algorithm>

#include "copula_t_kernels.h"
#include "mc_device.cuh"

namespace stocha {
namespace {

template <class G>
__device__ __forceinline__ double next_f64(G& g) { return u64_to_unit_f64(g.next()); }  // pcg64.rs:37-39

// student_t.rs:93-119 (shape >= 1: nu > 2 is enforced)
template <class G>
__device__ double sample_gamma(G& g, double d, double c, const SamplerCtx& sc, const ZigShared& zs, unsigned& err,
                               int max_iter = kGammaMaxIters) {
#pragma unroll 1
  for (int it = 0; it < max_iter; ++it) {
    const double x = normal_f64(g, sc, zs, err);
    const double v_inner = 1.0 + c * x;
    if (v_inner <= 0.0) continue;
    const double v = v_inner * v_inner * v_inner;
    const double u = next_f64(g);
    if (u < 1.0 - 0.0331 * (x * x) * (x * x)) return d * v;
    if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return d * v;
  }
  err |= kErrGammaIters;
  return d;
}

// One sample: chi-square (2 * gamma(nu / 2), student_t.rs:121-124) and dim
// normals.  With z null only the consumption matters: the normals are then
// drawn by the FP32 sampler, which consumes exactly the same draws without
// FP64 work (the gamma's own normal keeps its exact FP64 value, which steers
// the accept test).
__device__ __forceinline__ double sample_one(CountingGen& g, const TParse& a, const SamplerCtx& sc,
                                             const ZigShared& zs, unsigned& err, double* z) {
  const double chi = 2.0 * sample_gamma(g, a.d, a.c, sc, zs, err);
  for (int j = 0; j < a.dim; ++j) {
    if (z)
      z[j] = normal_f64(g, sc, zs, err);
    else
      (void)normal_f32(g, sc, zs, err);
  }
  return chi;
}

__device__ __forceinline__ CountingGen gen_at(const TParse& a, uint64_t pos) {
  return CountingGen{pcg_path_state(a.ss, pos), a.ss.inc_lo, a.ss.inc_hi, pos};
}

// Parses the samples that start in [lo, hi) from a sample start at pos;
// returns the end of the last one and counts them.
__device__ uint64_t parse_span(const TParse& a, uint64_t pos, uint64_t hi, const SamplerCtx& sc, const ZigShared& zs,
                               unsigned& err, uint32_t* count) {
  CountingGen g = gen_at(a, pos);
  uint32_t n = 0;
  while (g.pos < hi) {
    sample_one(g, a, sc, zs, err, nullptr);
    ++n;
  }
  *count = n;
  return g.pos;
}

__global__ void __launch_bounds__(128) k_tparse(const __grid_constant__ TParse a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const uint64_t total = a.nchunks * (uint64_t)a.E;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t chunk = t / a.E, e = t - chunk * a.E;
    const uint64_t lo = chunk * a.C, hi = lo + a.C;
    uint32_t cnt = 0;
    const uint64_t end = parse_span(a, lo + e, hi, sc, zs, err, &cnt);
    a.exits[t] = end - hi;
    a.counts[t] = cnt;
  }
  if (err) atomicOr(a.err, err);
}

// Carries (entry, count) through chunk c: the candidate table, a chunk that a
// sample spans entirely, or a parse when the entry lies beyond the candidates.
__device__ __forceinline__ void chunk_step(const TParse& a, uint64_t c, uint64_t& entry, uint64_t& count,
                                           const SamplerCtx& sc, const ZigShared& zs, unsigned& err) {
  if (entry >= a.C) {
    entry -= a.C;
    return;
  }
  if (entry < (uint64_t)a.E) {
    count += a.counts[c * a.E + entry];
    entry = a.exits[c * a.E + entry];
    return;
  }
  const uint64_t lo = c * a.C;
  uint32_t n;
  entry = parse_span(a, lo + entry, lo + a.C, sc, zs, err, &n) - (lo + a.C);
  count += n;
}

// The stitch runs in three passes over groups of G chunks, so that no thread
// follows more than ~sqrt(chunks) dependent lookups:
//   compose: per (group, candidate entry) the group's exit and sample count;
//   top:     one thread chains the groups from entry 0 until n samples;
//   fill:    per group, the true entry and first sample of each of its chunks.
__global__ void __launch_bounds__(128) k_tcompose(const __grid_constant__ TParse a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < a.ngroups * a.E) {
    const uint64_t g = t / a.E;
    uint64_t entry = t - g * a.E, count = 0;
    const uint64_t c1 = min(a.nchunks, (g + 1) * a.G);
    for (uint64_t c = g * a.G; c < c1; ++c) chunk_step(a, c, entry, count, sc, zs, err);
    a.gexit[t] = entry;
    a.gcount[t] = count;
  }
  if (err) atomicOr(a.err, err);
}

__global__ void k_ttop(const __grid_constant__ TParse a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  if (threadIdx.x != 0) return;
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  uint64_t entry = 0, base = 0, g = 0;
  for (; g < a.ngroups && base < a.n; ++g) {
    a.gentry[g] = entry;
    a.gfirst[g] = base;
    if (entry < (uint64_t)a.E) {
      base += a.gcount[g * a.E + entry];
      entry = a.gexit[g * a.E + entry];
    } else {
      const uint64_t c1 = min(a.nchunks, (g + 1) * a.G);
      for (uint64_t c = g * a.G; c < c1; ++c) chunk_step(a, c, entry, base, sc, zs, err);
    }
  }
  a.status[0] = min(a.nchunks, g * a.G);
  a.status[1] = base;
  a.status[2] = g;
  if (err) atomicOr(a.err, err);
}

__global__ void __launch_bounds__(128) k_tfill(const __grid_constant__ TParse a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < a.status[2]) {
    uint64_t entry = a.gentry[g], base = a.gfirst[g];
    const uint64_t c1 = min(a.nchunks, (g + 1) * a.G);
    for (uint64_t c = g * a.G; c < c1; ++c) {
      a.entry[c] = entry;
      a.first[c] = base;
      chunk_step(a, c, entry, base, sc, zs, err);
    }
  }
  if (err) atomicOr(a.err, err);
}

// One thread per chunk: the chunk's samples from its true entry.
__global__ void __launch_bounds__(128) k_temit(const __grid_constant__ TParse a, const uint64_t* __restrict__ status) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  const uint64_t used = status[0];
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < used; c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = c * a.C, hi = lo + a.C;
    CountingGen g = gen_at(a, lo + a.entry[c]);
    uint64_t s = a.first[c];
    while (g.pos < hi && s < a.n) {
      double* row = a.raw + s * (uint64_t)(a.dim + 1);
      row[0] = sample_one(g, a, sc, zs, err, row + 1);
      ++s;
    }
  }
  if (err) atomicOr(a.err, err);
}

// ---- Student-t CDF (student_t.rs:6-91) ----
// Modified Lentz continued fraction of the incomplete beta (student_t.rs:40-72).
// The even and odd partial numerators are x times coefficients of m alone
// (cf[2(m-1)], cf[2(m-1)+1]), formed once per call on the host.
// Each half step needs 1/d' (the new d) and, for the next half step, 1/c:
// both come from one reciprocal of the product d' c.
__device__ double beta_cf(double x, double a, double b, const double* __restrict__ cf) {
  const double EPS = 3e-7, FPMIN = 1e-30;
  const double qab = a + b, qap = a + 1.0;
  double c = 1.0, rc = 1.0;  // c and 1/c
  double d = fmax(1.0 - qab * x / qap, FPMIN);
  d = recip_nr(d);
  double h = d;
  for (int m = 1; m <= 200; ++m) {
    double aa = __ldg(cf + 2 * (m - 1)) * x;
    double dp = fmax(fabs(1.0 + aa * d), FPMIN);
    c = fmax(fabs(1.0 + aa * rc), FPMIN);
    double r = recip_nr(dp * c);
    d = r * c;
    rc = r * dp;
    h *= d * c;
    aa = __ldg(cf + 2 * (m - 1) + 1) * x;
    dp = fmax(fabs(1.0 + aa * d), FPMIN);
    c = fmax(fabs(1.0 + aa * rc), FPMIN);
    r = recip_nr(dp * c);
    d = r * c;
    rc = r * dp;
    const double del = d * c;
    h *= del;
    if (fabs(del - 1.0) < EPS) break;
  }
  return h;
}

// student_t.rs:19-31.  log_beta = lgamma(a) + lgamma(b) - lgamma(a + b) is
// the same for (a, b) and the flipped (b, a) (IEEE addition commutes), so the
// host forms it once per call with the reference's Lanczos log-gamma.
// cf holds the continued-fraction coefficients for (a, b) and, 400 doubles
// on, for the flipped (b, a).
__device__ double ibeta(double x, double a, double b, double log_beta, const double* __restrict__ cf) {
  if (x <= 0.0) return 0.0;
  if (x >= 1.0) return 1.0;
  bool flip = false;
  if (x > (a + 1.0) / (a + b + 2.0)) {
    flip = true;
    x = 1.0 - x;
    const double t = a;
    a = b;
    b = t;
    cf += 400;
  }
  const double front = exp(a * log(x) + b * log(1.0 - x) - log_beta) / a;
  const double v = front * beta_cf(x, a, b, cf);
  return flip ? 1.0 - v : v;
}

__global__ void __launch_bounds__(256) k_tcdf(const double* __restrict__ raw, const double* __restrict__ L,
                                              uint64_t n, int dim, double nu, double log_beta,
                                              const double* __restrict__ cf, double* __restrict__ u) {
  const uint64_t total = n * (uint64_t)dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / (uint64_t)dim;
    const int j = (int)(e - i * (uint64_t)dim);
    const double* row = raw + i * (uint64_t)(dim + 1);
    const double scale = sqrt(nu / row[0]);  // student_t.rs:157
    double x = 0.0;
    for (int k = 0; k <= j; ++k) x += L[j * dim + k] * row[1 + k];
    const double xs = x * scale;
    const double z = nu / (nu + xs * xs);
    const double ib = ibeta(z, nu / 2.0, 0.5, log_beta, cf);
    u[e] = xs >= 0.0 ? 1.0 - 0.5 * ib : 0.5 * ib;
  }
}

__global__ void __launch_bounds__(256) k_debug_capped(const __grid_constant__ DebugCapped a) {
  __shared__ ZigShared zs;
  zig_stage(zs, a.tabs, true);
  const SamplerCtx sc{a.tabs, a.tabs->r32, a.tabs->r};
  unsigned err = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x) {
    PcgGen g{pcg_path_state(a.ss, i), a.ss.inc_lo, a.ss.inc_hi};
    double v;
    switch (a.sampler) {
      case 0: v = normal_f64(g, sc, zs, err, a.cap, kZigMaxTail); break;
      case 1: v = normal_f64(g, sc, zs, err, kZigMaxAttempts, a.cap); break;
      case 2: v = normal_f32(g, sc, zs, err, nullptr, a.cap, kZigMaxTail); break;
      case 3: v = normal_f32(g, sc, zs, err, nullptr, kZigMaxAttempts, a.cap); break;
      default: v = sample_gamma(g, a.d, a.c, sc, zs, err, a.cap); break;
    }
    a.out[i] = v;
  }
  if (err) atomicOr(a.err, err);
}

}  // namespace

void launch_tparse(const TParse& a, cudaStream_t st) {
  const uint64_t total = a.nchunks * (uint64_t)a.E;
  uint64_t g = (total + 127) / 128;
  if (g > 152ull * 64) g = 152ull * 64;
  k_tparse<<<(unsigned)(g ? g : 1), 128, 0, st>>>(a);
}

void launch_tstitch(const TParse& a, cudaStream_t st) {
  const uint64_t threads = a.ngroups * (uint64_t)a.E;
  k_tcompose<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(a);
  k_ttop<<<1, 32, 0, st>>>(a);
  k_tfill<<<(unsigned)((a.ngroups + 127) / 128), 128, 0, st>>>(a);
}

void launch_temit(const TParse& a, const uint64_t* status, cudaStream_t st) {
  uint64_t g = (a.nchunks + 127) / 128;
  k_temit<<<(unsigned)(g ? g : 1), 128, 0, st>>>(a, status);
}

void launch_tcdf(const double* raw, const double* L, uint64_t n, int dim, double nu, double log_beta,
                 const double* cf, double* u, cudaStream_t st) {
  const uint64_t total = n * (uint64_t)dim;
  uint64_t g = (total + 255) / 256;
  if (g > 152ull * 32) g = 152ull * 32;
  k_tcdf<<<(unsigned)(g ? g : 1), 256, 0, st>>>(raw, L, n, dim, nu, log_beta, cf, u);
}

void launch_debug_capped(const DebugCapped& a, cudaStream_t st) {
  if (a.n) k_debug_capped<<<(unsigned)std::min<uint64_t>((a.n + 255) / 256, 4096), 256, 0, st>>>(a);
}

}  // namespace stocha
