// VaR / CVaR kernels (risk.cu), used by risk_host.cpp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace stocha {

// Radix-select state, device resident.  Before the first pass: rank = idx,
// everything else zero.  After the eighth: prefix = the key of rank idx,
// less = keys below it, equal = keys equal to it.
struct SelectState {
  uint64_t prefix, mask, rank, less, equal;
};

// 8 select passes; the first sets *bad if a return is NaN or infinite.
void launch_select(const double* r, uint64_t n, SelectState* state, unsigned long long* hist, unsigned* bad,
                   int grid, cudaStream_t st);
void launch_tail_sum(const double* r, uint64_t n, const SelectState* state, double* part, int grid, cudaStream_t st);

}  // namespace stocha
