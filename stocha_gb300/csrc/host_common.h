// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/stocha_gpu.h"
#include "engine.h"

typedef unsigned __int128 u128;

namespace stocha {

// Grow-only device buffer owned by a context.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace stocha

struct stocha_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  stocha::ZigTables* d_tabs = nullptr;
  unsigned* d_err = nullptr;
  unsigned* h_err = nullptr;  // pinned
  double* h_small = nullptr;  // pinned, 4096 doubles for small results
  stocha::DevBuf out, partials, small, aux, starts;
  std::recursive_mutex mu;
};

namespace stocha {

int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);
#define STOCHA_CUDA(call)                                     \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::stocha::cuda_error(e_, #call); \
  } while (0)

// Resolves NULL to the default context; creates it on first use.
int resolve_ctx(stocha_ctx** ctx);
int ensure_buf(stocha_ctx* c, DevBuf& b, size_t bytes);
// Clears the device error word before a launch / reads it after a sync.
int begin_call(stocha_ctx* c);
int finish_call(stocha_ctx* c);  // synchronises the stream

// Stream of Pcg64Dxsm::new(seed) split into blocks of `block` draws.
void make_stream_spec(u128 seed, u128 block, StreamSpec* ss);
// Same from an explicit (state, inc) (the RNG surface's current position).
void make_stream_spec_state(u128 state, u128 inc, u128 block, StreamSpec* ss);
// Host restatement of Pcg64Dxsm::new (prng/pcg64.rs:23-30).
void pcg_seed(u128 seed, u128* state, u128* inc);
void pcg_advance(u128* state, u128 inc, u128 delta);

// The ziggurat tables as the kernels read them (thresholds derived on the host).
void fill_zig_tables(ZigTables* t);

// u < p for u = (draw >> 11) * 2^-53  <=>  (draw >> 11) < unit_threshold(p)
uint64_t unit_threshold(double p);

// Peak-rate microbenchmarks (peaks.cu).
double measure_peak(int kind, cudaStream_t st);

// Rust f64 Display (shortest round-trip digits, no exponent).
std::string rust_f64(double v);

// Model validation with the reference's messages (check=false skips the
// range checks, as greeks_fd does, lib.rs:958-1040); fills the launch
// constants.
int prepare_model(const stocha_model* m, PathLaunch* L, uint64_t* row_len, u128* block, bool check = true);
// Enqueues a fused pricing launch: sums_dev receives {sum, sum of squares}
// of the payoff per asset.  aux4: payoff parameters (pathwise estimators).
int price_launch(stocha_ctx* c, const stocha_model* m, uint64_t seed, int precision, int payoff, double strike,
                 const double* aux4, bool check, double* sums_dev, int* nvals);
// Enqueues a launch writing the terminal price of every path (FP64).
int terminal_launch(stocha_ctx* c, const stocha_model* m, uint64_t seed, double* out_dev);

}  // namespace stocha
