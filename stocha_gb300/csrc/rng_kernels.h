// Launchers of the RNG-surface kernels (rng.cu), used by rng_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_types.h"

namespace stocha {

constexpr int kRngEntries = 4;        // candidate entry offsets parsed per chunk
constexpr uint32_t kRngChunk = 512;   // draws per chunk

void launch_rng_raw(const StreamSpec& ss, const PcgJump& stride, uint64_t threads, uint64_t n, int kind,
                    void* out, cudaStream_t st);
void launch_rng_parse(const StreamSpec& ss, const ZigTables* tabs, uint64_t nchunks, uint32_t C, uint32_t* counts,
                      uint32_t* exits, uint32_t* entry, uint32_t* cnt, uint64_t* offset, uint64_t* total,
                      unsigned* err, cudaStream_t st);
void launch_rng_emit(const StreamSpec& ss, const ZigTables* tabs, uint64_t nchunks, uint32_t C,
                     const uint32_t* entry, const uint32_t* cnt, const uint64_t* offset, uint64_t n, int kind,
                     double loc, double scale, double* out, uint64_t* final_pos, unsigned* err, cudaStream_t st);

// Gaussian copula rows: u[i, j] = Phi(sum_{k<=j} L[j, k] z[i, k]) with the
// reference's normal CDF (dist/normal_cdf.rs, A&S 26.2.17); inv_sqrt_2pi is
// 1 / the host's sqrt(2 pi); tabs supplies the exponential's table.
void launch_copula_gaussian(const double* z, const double* L, uint64_t n, int dim, const ZigTables* tabs,
                            double inv_sqrt_2pi, double* u, cudaStream_t st);

}  // namespace stocha
