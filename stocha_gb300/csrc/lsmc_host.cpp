// Host side of the LSMC American option (src/lib.rs:854-918,
// src/finance/lsmc.rs:25-115): validation, GBM paths in time-major layout,
// the device backward sweep, and the estimator.
#include <cmath>
#include <cstring>

#include "host_common.h"
#include "lsmc_kernels.h"

using namespace stocha;

namespace stocha {

int lsmc_validate(const LsmcJob& j) {  // lib.rs:885-903
  if (j.s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
  if (j.k <= 0.0) return set_error(STOCHA_ERR_VALUE, "k must be positive");
  if (j.sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (j.t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  if (j.steps == 0 || j.n_paths == 0) return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
  if (j.n_paths < 2) return set_error(STOCHA_ERR_VALUE, "n_paths must be at least 2");
  if (j.deg == 0 || j.deg > 4) return set_error(STOCHA_ERR_VALUE, "poly_degree must be in [1, 4]");
  return STOCHA_OK;
}

void lsmc_footprint(const LsmcJob& j, int sms, size_t* path_bytes, size_t* scratch_bytes) {
  const size_t esz = j.precision == STOCHA_FP32 ? 4 : 8;
  *path_bytes = (((size_t)j.n_paths * (j.steps + 1) * esz) + 255) & ~(size_t)255;
  *scratch_bytes = lsmc_scratch_bytes(j.n_paths, j.steps, lsmc_grid(j.n_paths, sms));
}

void lsmc_graphs_release(LsmcGraphs* g) { lsmc_graphs_destroy(g); }

int lsmc_enqueue(const LsmcJob& j, int sms, void* paths, void* scratch, const ZigTables* tabs, unsigned* err,
                 bool flat, cudaStream_t st, LsmcGraphs* graphs, const double** result_dev) {
  // GBM paths under the risk-neutral drift (lsmc.rs:29-39)
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_GBM;
  m.s0 = j.s0;
  m.mu = j.r;
  m.sigma = j.sigma;
  m.q = 0.0;
  m.t = j.t;
  m.steps = j.steps;
  m.n_paths = j.n_paths;
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(&m, &L, &row_len, &block);
  if (rc) return rc;
  make_stream_spec((u128)j.seed, block, &L.ss);
  fill_f32_constants(&L);
  L.tabs = tabs;
  L.err = err;
  L.time_major = 1;
  L.flat_grid = flat ? 1 : 0;
  const bool f32 = j.precision == STOCHA_FP32;
  if (f32)
    L.out_f32 = (float*)paths;
  else
    L.out_f64 = (double*)paths;

  LsmcLaunch a;
  std::memset(&a, 0, sizeof a);
  a.spot = paths;
  a.spot_f32 = f32;
  a.n = j.n_paths;
  a.steps = j.steps;
  a.k = j.k;
  const double dt = j.t / (double)j.steps;
  a.log_disc = -j.r * dt;
  a.disc = std::exp(a.log_disc);  // lsmc.rs:26-27
  a.is_put = j.is_put ? 1 : 0;
  a.deg = (int)j.deg;
  a.grid = lsmc_grid(j.n_paths, sms);
  a.cluster = lsmc_cluster_size(j.n_paths, j.steps, f32 ? 1 : 0);
  lsmc_bind_scratch(&a, scratch);

  const int g = f32 ? launch_paths_f32(L, st) : launch_paths_f64(L, st);
  if (g < 0) return cuda_error(cudaGetLastError(), "LSMC path launch");
  STOCHA_CUDA(lsmc_sweep(a, st, graphs));
  STOCHA_CUDA(cudaGetLastError());
  *result_dev = a.result;
  return STOCHA_OK;
}

void lsmc_estimate(const LsmcJob& j, const double* res2, double* price, double* std_err) {
  const double n = (double)j.n_paths;
  *price = res2[0];
  *std_err = std::sqrt(res2[1] / (n - 1.0) / n);  // lsmc.rs:106-112
}

}  // namespace stocha

namespace {

int lsmc_run(stocha_ctx* ctx, const LsmcJob& j, double* price, double* std_err) {
  int rc = lsmc_validate(j);
  if (rc) return rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const size_t esz = j.precision == STOCHA_FP32 ? 4 : 8;
  if (j.n_paths > (SIZE_MAX / esz) / (j.steps + 1)) return set_error(STOCHA_ERR_NOMEM, "path array too large");
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  size_t path_bytes = 0, scratch_bytes = 0;
  lsmc_footprint(j, sms, &path_bytes, &scratch_bytes);
  if ((rc = ensure_buf(ctx, ctx->out, path_bytes))) return rc;
  if ((rc = ensure_buf(ctx, ctx->aux, scratch_bytes))) return rc;
  if (!ctx->lsmc_graphs) STOCHA_CUDA(lsmc_graphs_create(&ctx->lsmc_graphs));
  if ((rc = begin_call(ctx))) return rc;
  const double* res = nullptr;
  if ((rc = lsmc_enqueue(j, sms, ctx->out.ptr, ctx->aux.ptr, ctx->d_tabs, ctx->d_err, false, ctx->stream,
                         ctx->lsmc_graphs, &res)))
    return rc;
  STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if ((rc = finish_call(ctx))) return rc;
  lsmc_estimate(j, ctx->h_small, price, std_err);
  return STOCHA_OK;
}

LsmcJob make_job(double s0, double k, double r, double sigma, double t, uint64_t steps, uint64_t n_paths,
                 int32_t is_put, uint64_t deg, uint64_t seed, int precision) {
  LsmcJob j;
  j.s0 = s0;
  j.k = k;
  j.r = r;
  j.sigma = sigma;
  j.t = t;
  j.steps = steps;
  j.n_paths = n_paths;
  j.deg = deg;
  j.seed = seed;
  j.is_put = is_put ? 1 : 0;
  j.precision = precision;
  return j;
}

}  // namespace

extern "C" {

int stocha_lsmc_american_option(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t,
                                uint64_t steps, uint64_t n_paths, int32_t is_put, uint64_t poly_degree,
                                uint64_t seed, double* price, double* std_err) {
  return lsmc_run(ctx, make_job(s0, k, r, sigma, t, steps, n_paths, is_put, poly_degree, seed, STOCHA_FP64), price,
                  std_err);
}

int stocha_lsmc(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t, uint64_t steps,
                uint64_t n_paths, int32_t is_put, uint64_t poly_degree, uint64_t seed, int32_t precision,
                double* price, double* std_err) {
  STOCHA_RANGE("stocha_lsmc");
  return lsmc_run(ctx, make_job(s0, k, r, sigma, t, steps, n_paths, is_put, poly_degree, seed, precision), price,
                  std_err);
}

}  // extern "C"
