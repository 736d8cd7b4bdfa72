// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include <mutex>
#include <string>

#include "../../include/stocha_gpu.h"
#include "engine.h"

typedef unsigned __int128 u128;

namespace stocha {

// A named range on the NVTX timeline (Nsight Systems, Nsight Compute) for
// the duration of one C-ABI call; without an attached tool it costs a
// pointer test.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define STOCHA_RANGE(name) ::stocha::NvtxRange stocha_nvtx_range_(name)

struct LsmcGraphs;

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
  stocha::LsmcGraphs* lsmc_graphs = nullptr;  // LSMC sweep graphs for this context's stream
  // overlap of materialised results' device-to-host copies with their compute
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t chunk_done[32] = {};
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
// Enqueues the copy of a large device result into fresh pageable host memory
// after the work already on st: the destination's pages are populated by host
// threads in the meantime and the copy goes out in chunks as they are ready
// (hostcopy.cpp).  Returns after the last chunk is enqueued.
int copy_to_host_populated(cudaStream_t st, void* dst, const void* src, size_t bytes);
// Whether [dst, dst + bytes) is a host result-cache buffer whose pages exist
// (a copy into it runs at the link's rate with no population pass).
bool host_dst_cached(const void* dst, size_t bytes);
// Enqueues a launch writing the terminal price of every path (FP64).
int terminal_launch(stocha_ctx* c, const stocha_model* m, uint64_t seed, double* out_dev);

struct GInst;
// One instance of the batched FP32 Greeks kernel (greeks_kernels.h) for a
// call or put on GBM, Heston (Euler) or Merton; price_only: only the price
// and its standard error.
void greeks_make_inst(const stocha_model& m, int payoff, double strike, double bump_size, uint64_t seed,
                      bool price_only, GInst* I);
// Price, standard error and the five Greeks (delta gamma vega theta rho) of
// one instance from its FP64 totals of the per-path sums.
void greeks_from_sums(const stocha_model& m, double bump_size, const double* S, double* price, double* se,
                      double* g);
stocha_model greeks_model_of(const stocha_greeks_instance& x);

// One LSMC American option (lsmc.rs:4-14) as a job over caller-owned device
// buffers: the path array and the sweep scratch.
struct LsmcJob {
  double s0, k, r, sigma, t;
  uint64_t steps, n_paths, deg, seed;
  int is_put, precision;
};
// Argument checks with the reference's messages (lib.rs:885-903).
int lsmc_validate(const LsmcJob& j);
void lsmc_footprint(const LsmcJob& j, int sms, size_t* path_bytes, size_t* scratch_bytes);
// Enqueues paths and sweep on st; *result_dev receives the device address of
// {mean of discounted cash flows, sum of squared deviations}.  flat: path
// launch with one path per thread (see PathLaunch::flat_grid).  graphs: the
// stream's sweep graphs (lsmc_kernels.h), used by one job at a time.
int lsmc_enqueue(const LsmcJob& j, int sms, void* paths, void* scratch, const ZigTables* tabs, unsigned* err,
                 bool flat, cudaStream_t st, LsmcGraphs* graphs, const double** result_dev);
void lsmc_graphs_release(LsmcGraphs* g);
// Price and standard error from the two device results (lsmc.rs:100-114).
void lsmc_estimate(const LsmcJob& j, const double* res2, double* price, double* std_err);

}  // namespace stocha
