// RNG surface (src/lib.rs:74-184): draws of ONE sequential PCG64DXSM stream,
// generated in parallel.
//
// uniform / raw: draw i is DXSM(state advanced by i); thread t starts at
// position t by jump-ahead and strides by the thread count.
//
// standard_normal / normal: a normal consumes a variable number of draws
// (normal.rs:18-67), so position of normal j is unknown until every earlier
// normal is drawn.  The stream is cut into chunks of C draws:
//   1. k_parse   every chunk is parsed (consumption only, FP32 decisions that
//                match the reference's FP64 ones) from each candidate entry
//                offset e < kEntries: normals started inside the chunk and the
//                offset at which the next normal starts in the next chunk.
//   2. k_stitch  one block resolves each chunk's true entry (chunk 0 enters at
//                0; a chunk whose parses all exit at the same offset fixes its
//                successor's entry without knowing its own), re-parses the rare
//                chunk entered beyond kEntries, and prefix-sums the counts.
//   3. k_emit    every chunk re-parses from its true entry and writes its
//                normals' exact FP64 values at their global index.
// Parses from different entries meet after a few draws, so step 2 almost
// never follows a chain longer than one chunk.
#include <cuda_runtime.h>

#include "engine.h"
#include "mc_device.cuh"
#include "rng_kernels.h"

namespace stocha {
namespace {

__device__ __forceinline__ uint64_t dxsm(uint64_t lo, uint64_t hi) {
  uint64_t o = hi ^ (hi >> 32);
  o *= kPcgMul;
  o ^= o >> 48;
  return o * (lo | 1ull);
}

// kind 0: raw u64, 1: uniform f64 (next_f64)
__global__ void __launch_bounds__(256) k_rng_raw(const __grid_constant__ StreamSpec ss, PcgJump stride,
                                                 uint64_t n, int kind, void* out) {
  const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  DevPcg s = pcg_path_state(ss, t);
  for (uint64_t i = t; i < n; i += T) {
    uint64_t u = dxsm(s.lo, s.hi);
    if (kind == 0)
      ((uint64_t*)out)[i] = u;
    else
      ((double*)out)[i] = u64_to_unit_f64(u);
    u128_mul_add(s.lo, s.hi, stride.mul_lo, stride.mul_hi, stride.add_lo, stride.add_hi);
  }
}

// Parse one chunk [c*C, (c+1)*C) from position c*C + e.
struct ParseResult {
  uint32_t count;
  uint32_t exit;  // next normal starts at (c+1)*C + exit
};

__device__ __forceinline__ ParseResult parse_chunk(const StreamSpec& ss, uint64_t c, uint32_t C, uint32_t e,
                                                   const SamplerCtx& sc, const ZigShared& zs, unsigned& err) {
  const uint64_t start = c * C + e, end = (c + 1) * C;
  CountingGen g{pcg_path_state(ss, start), ss.inc_lo, ss.inc_hi, start};
  uint32_t cnt = 0;
#pragma unroll 1
  while (g.pos < end) {
    (void)normal_f32(g, sc, zs, err);
    ++cnt;
  }
  return ParseResult{cnt, (uint32_t)(g.pos - end)};
}

__global__ void __launch_bounds__(128) k_parse(const __grid_constant__ StreamSpec ss, const ZigTables* tabs,
                                               uint64_t nchunks, uint32_t C, uint32_t* counts, uint32_t* exits,
                                               unsigned* err_out) {
  __shared__ ZigShared zs;
  zig_stage(zs, tabs, false);
  const SamplerCtx sc{tabs, tabs->r32, tabs->r};
  unsigned err = 0;
  const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id < nchunks * kRngEntries) {
    const uint64_t c = id / kRngEntries;
    const uint32_t e = (uint32_t)(id % kRngEntries);
    ParseResult r = parse_chunk(ss, c, C, e, sc, zs, err);
    counts[id] = r.count;
    exits[id] = r.exit;
  }
  if (err) atomicOr(err_out, err);
}

// One block.  entry[c], offset[c] (exclusive prefix of counts); total.
__global__ void __launch_bounds__(1024) k_stitch(const __grid_constant__ StreamSpec ss, const ZigTables* tabs,
                                                 uint64_t nchunks, uint32_t C, const uint32_t* counts,
                                                 const uint32_t* exits, uint32_t* entry, uint32_t* cnt_out,
                                                 uint64_t* offset, uint64_t* total, unsigned* err_out) {
  __shared__ ZigShared zs;
  __shared__ uint64_t warp_tot[32];
  __shared__ uint64_t carry;
  zig_stage(zs, tabs, false);
  const SamplerCtx sc{tabs, tabs->r32, tabs->r};
  unsigned err = 0;
  // (a) entries: chase back to chunk 0 or to a chunk whose exits all agree.
  for (uint64_t c = threadIdx.x; c < nchunks; c += blockDim.x) {
    uint64_t j = c;
    while (j > 0) {
      const uint32_t* ex = exits + (j - 1) * kRngEntries;
      bool conv = true;
      for (int e = 1; e < kRngEntries; ++e) conv &= ex[e] == ex[0];
      if (conv) break;
      --j;
    }
    uint32_t e = 0;
    if (j > 0) e = exits[(j - 1) * kRngEntries];
    // walk forward from chunk j (entry e) to chunk c
    for (uint64_t k = j; k < c; ++k) {
      if (e < kRngEntries) {
        e = exits[k * kRngEntries + e];
      } else {
        ParseResult r = parse_chunk(ss, k, C, e, sc, zs, err);
        e = r.exit;
      }
    }
    entry[c] = e;
    if (e < kRngEntries) {
      cnt_out[c] = counts[c * kRngEntries + e];
    } else {
      ParseResult r = parse_chunk(ss, c, C, e, sc, zs, err);
      cnt_out[c] = r.count;
    }
  }
  __syncthreads();
  // (b) exclusive prefix sum of cnt_out in fixed-size tiles of blockDim.x
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint64_t base = 0; base < nchunks; base += blockDim.x) {
    uint64_t c = base + threadIdx.x;
    uint64_t v = c < nchunks ? cnt_out[c] : 0;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint64_t w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    uint64_t before = carry + (wid > 0 ? warp_tot[wid - 1] : 0) + x - v;
    if (c < nchunks) offset[c] = before;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
  if (err) atomicOr(err_out, err);
}

// kind 1: standard normal; 2: loc + scale * z (normal.rs:77-79).
__global__ void __launch_bounds__(128) k_emit(const __grid_constant__ StreamSpec ss, const ZigTables* tabs,
                                              uint64_t nchunks, uint32_t C, const uint32_t* entry,
                                              const uint32_t* cnt, const uint64_t* offset, uint64_t n, int kind,
                                              double loc, double scale, double* out, uint64_t* final_pos,
                                              unsigned* err_out) {
  __shared__ ZigShared zs;
  zig_stage(zs, tabs, true);
  const SamplerCtx sc{tabs, tabs->r32, tabs->r};
  unsigned err = 0;
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nchunks && offset[c] < n) {
    const uint64_t start = c * C + entry[c];
    CountingGen g{pcg_path_state(ss, start), ss.inc_lo, ss.inc_hi, start};
    uint64_t idx = offset[c];
    const uint32_t k_end = cnt[c];
#pragma unroll 1
    for (uint32_t k = 0; k < k_end && idx < n; ++k, ++idx) {
      double z = normal_f64(g, sc, zs, err);
      out[idx] = kind == 2 ? loc + scale * z : z;
      if (idx == n - 1) *final_pos = g.pos;
    }
  }
  if (err) atomicOr(err_out, err);
}

}  // namespace

void launch_rng_raw(const StreamSpec& ss, const PcgJump& stride, uint64_t threads, uint64_t n, int kind,
                    void* out, cudaStream_t st) {
  const uint64_t b = 256;
  uint64_t g = (threads + b - 1) / b;
  if (g == 0) g = 1;
  k_rng_raw<<<(unsigned)g, (unsigned)b, 0, st>>>(ss, stride, n, kind, out);
}

void launch_rng_parse(const StreamSpec& ss, const ZigTables* tabs, uint64_t nchunks, uint32_t C, uint32_t* counts,
                      uint32_t* exits, uint32_t* entry, uint32_t* cnt, uint64_t* offset, uint64_t* total,
                      unsigned* err, cudaStream_t st) {
  const uint64_t items = nchunks * kRngEntries;
  k_parse<<<(unsigned)((items + 127) / 128), 128, 0, st>>>(ss, tabs, nchunks, C, counts, exits, err);
  k_stitch<<<1, 1024, 0, st>>>(ss, tabs, nchunks, C, counts, exits, entry, cnt, offset, total, err);
}

void launch_rng_emit(const StreamSpec& ss, const ZigTables* tabs, uint64_t nchunks, uint32_t C,
                     const uint32_t* entry, const uint32_t* cnt, const uint64_t* offset, uint64_t n, int kind,
                     double loc, double scale, double* out, uint64_t* final_pos, unsigned* err, cudaStream_t st) {
  k_emit<<<(unsigned)((nchunks + 127) / 128), 128, 0, st>>>(ss, tabs, nchunks, C, entry, cnt, offset, n, kind,
                                                             loc, scale, out, final_pos, err);
}

// One thread per output element (i, j): the reference's running sum
// x_j = sum_{k<=j} L[j,k] z_k in k order (gaussian.rs:60-66; this unit is
// compiled without FMA contraction), then its normal CDF
// (dist/normal_cdf.rs:3-22, Abramowitz-Stegun 26.2.17).  The CDF's FP64
// division and exp (GB300 runs FP64 at 1/64 of the FP32 rate) are the
// Newton reciprocal and the table-driven exponential: pdf = exp(-x^2/2) /
// sqrt(2 pi) becomes (1 / sqrt(2 pi)) * exp(-x^2/2), within ~3 ulp of it.
__global__ void __launch_bounds__(256) k_copula_gaussian(const double* __restrict__ z, const double* __restrict__ L,
                                                         uint64_t n, int dim, const ZigTables* __restrict__ tabs,
                                                         double inv_sqrt_2pi, double* __restrict__ u) {
  __shared__ ZigShared zs;
  zig_stage(zs, tabs, true);
  const uint64_t total = n * (uint64_t)dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / (uint64_t)dim;
    const int j = (int)(e - i * (uint64_t)dim);
    const double* zi = z + i * (uint64_t)dim;
    double x = 0.0;
    for (int k = 0; k <= j; ++k) x += L[j * dim + k] * zi[k];
    const double t = recip_nr(1.0 + 0.2316419 * fabs(x));
    const double poly =
        t * (0.319381530 + t * (-0.356563782 + t * (1.781477937 + t * (-1.821255978 + t * 1.330274429))));
    const double pdf = mul_exp(inv_sqrt_2pi, -0.5 * x * x, zs);
    const double cdf_pos = 1.0 - pdf * poly;
    u[e] = x >= 0.0 ? cdf_pos : 1.0 - cdf_pos;
  }
}

void launch_copula_gaussian(const double* z, const double* L, uint64_t n, int dim, const ZigTables* tabs,
                            double inv_sqrt_2pi, double* u, cudaStream_t st) {
  const uint64_t total = n * (uint64_t)dim;
  uint64_t g = (total + 255) / 256;
  if (g > 152ull * 32) g = 152ull * 32;
  if (g < 1) g = 1;
  k_copula_gaussian<<<(unsigned)g, 256, 0, st>>>(z, L, n, dim, tabs, inv_sqrt_2pi, u);
}

}  // namespace stocha
