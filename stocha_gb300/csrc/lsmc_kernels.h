// LSMC backward-sweep launch description (lsmc.cu), used by lsmc_host.cpp and
// the serving loop.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace stocha {

// Per-step regression state, resident on the device.
struct LsmcStep {
  double m, mean, std, inv_std;  // ITM count and statistics of the step's spots (lsmc.rs:61-71)
  double coef[5];                // regression coefficients (lsmc.rs:83-84)
  float mean_f, inv_f, coef_f[5];
  int skip;  // fewer ITM paths than ncols + 1: no regression, no exercise (lsmc.rs:62-64)
};

struct LsmcLaunch {
  const void* spot;  // time-major spot[(steps+1) * n], double (FP64 form) or float (FP32 form)
  int spot_f32;
  void* cf;            // FP64 form: n discounted cash flows; FP32 form: n {payoff, exercise step} pairs
  double* part;        // grid * kLsmcValues block partials
  unsigned* counter;   // blocks finished in the current launch (zero before the sweep)
  LsmcStep* step_params;  // steps + 1 entries
  float* dpow;         // FP32 form: disc^j, j = 0..steps
  double* result;      // [0] mean of discounted cash flows, [1] sum of squared deviations
  uint64_t n, steps;
  double k, disc, log_disc;
  int is_put, deg, grid;
  int cluster;  // > 0: the whole sweep as one launch of one cluster of this many blocks
};

constexpr int kLsmcValues = 17;  // p[0..8] | q[0..4] | ITM count, sum(s-k), sum(s-k)^2

// Largest problems the one-cluster sweep takes (paths; steps + 1 entries of
// the FP32 discount table in shared memory).
constexpr uint64_t kLsmcClusterMaxPaths = 1u << 19;
constexpr uint64_t kLsmcClusterMaxSteps = 8192;

// Blocks of every multi-launch sweep launch for n paths on `sms` SMs.
int lsmc_grid(uint64_t n, int sms);
// Cluster size for the one-cluster sweep of (n, steps) in the FP32 (f32 = 1)
// or FP64 form, or 0 for the multi-launch sweep.
int lsmc_cluster_size(uint64_t n, uint64_t steps, int f32);
// Device scratch of one sweep (everything but the path array), and the
// binding of a LsmcLaunch's scratch pointers into it (256-byte aligned base).
size_t lsmc_scratch_bytes(uint64_t n, uint64_t steps, int grid);
void lsmc_bind_scratch(LsmcLaunch* a, void* scratch);
// Instantiated CUDA graphs of the multi-launch sweep for one stream.  The
// multi-launch kernels read their LsmcLaunch from device memory (params), so
// one graph per shape (steps, degree, precision, grid) serves every job: a
// graph launch copies the job's LsmcLaunch from the pinned staging, zeroes
// the block counter and runs the steps + 2 passes.  The staging is read when
// the graph runs: one job at a time per LsmcGraphs (a stream's jobs are in
// order, and the host writes the staging only after the previous job ended).
struct LsmcGraphs {
  LsmcLaunch* d_params = nullptr;  // device: the launch description, then the block counter
  LsmcLaunch* h_params = nullptr;  // pinned host staging
  struct Entry {
    uint64_t steps;
    int deg, f32, grid;
    cudaGraphExec_t exec;
  };
  Entry cache[8];
  int n_cache = 0, next = 0;
};
cudaError_t lsmc_graphs_create(LsmcGraphs** out);
void lsmc_graphs_destroy(LsmcGraphs* g);

// Enqueues the whole sweep on `st` with no host round trip: one cluster
// launch, or one graph launch of the multi-launch passes (graphs required).
cudaError_t lsmc_sweep(const LsmcLaunch& a, cudaStream_t st, LsmcGraphs* graphs);

}  // namespace stocha
