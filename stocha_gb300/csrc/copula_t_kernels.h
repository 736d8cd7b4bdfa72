// Student-t copula kernels (copula_t.cu), used by rng_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_types.h"

namespace stocha {

struct TParse {
  StreamSpec ss;  // the sequential stream, jump table by draw index
  const ZigTables* tabs;
  unsigned* err;
  uint64_t nchunks, n;  // chunks parsed; samples wanted
  uint32_t C;           // draws per chunk
  int E;                // candidate entry offsets per chunk
  int dim;
  int pad;
  double d, c;          // Marsaglia-Tsang constants of shape nu / 2
  uint64_t* exits;      // nchunks * E: end of the last sample minus the chunk end
  uint32_t* counts;     // nchunks * E: samples starting in the chunk
  uint64_t* entry;      // nchunks: true entry offset
  uint64_t* first;      // nchunks: index of the chunk's first sample
  uint64_t* status;     // [0] chunks used, [1] samples covered, [2] groups used
  double* raw;          // n * (dim + 1): chi-square, then the dim normals
  // groups of G consecutive chunks, composed per candidate entry
  uint64_t G, ngroups;
  uint64_t* gexit;      // ngroups * E: exit of the group's last chunk
  uint64_t* gcount;     // ngroups * E: samples starting in the group
  uint64_t* gentry;     // ngroups: true entry offset of the group's first chunk
  uint64_t* gfirst;     // ngroups: index of the group's first sample
};

// Diagnostic: thread i < n draws once from path i's stream (ss: block-split
// streams) with the engine's samplers and a lowered iteration cap, so that
// the caps' error path can be driven: sampler 0 FP64 normal (attempt cap),
// 1 FP64 normal (tail cap), 2 FP32 normal (attempt cap), 3 FP32 normal (tail
// cap), 4 gamma of shape nu / 2 with constants (d, c) (rejection cap).
struct DebugCapped {
  StreamSpec ss;
  const ZigTables* tabs;
  unsigned* err;
  double* out;
  uint64_t n;
  int sampler, cap;
  double d, c;
};
void launch_debug_capped(const DebugCapped& a, cudaStream_t st);

void launch_tparse(const TParse& a, cudaStream_t st);
void launch_tstitch(const TParse& a, cudaStream_t st);
void launch_temit(const TParse& a, const uint64_t* status, cudaStream_t st);
// cf: 800 doubles, the continued-fraction coefficients of the incomplete
// beta for (nu/2, 1/2) then (1/2, nu/2): per m = 1..200 the even and odd
// partial numerators divided by x.
void launch_tcdf(const double* raw, const double* L, uint64_t n, int dim, double nu, double log_beta,
                 const double* cf, double* u, cudaStream_t st);

}  // namespace stocha
