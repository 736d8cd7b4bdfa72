// Host side of the LSMC American option (src/lib.rs:854-918,
// src/finance/lsmc.rs:25-115): validation, GBM paths in time-major layout,
// the device backward sweep, and the estimator.
#include <cmath>
#include <cstring>

#include "host_common.h"
#include "lsmc_kernels.h"

using namespace stocha;

namespace {

int lsmc_validate(double s0, double k, double sigma, double t, uint64_t steps, uint64_t n_paths, uint64_t deg) {
  if (s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
  if (k <= 0.0) return set_error(STOCHA_ERR_VALUE, "k must be positive");
  if (sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  if (steps == 0 || n_paths == 0) return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
  if (n_paths < 2) return set_error(STOCHA_ERR_VALUE, "n_paths must be at least 2");
  if (deg == 0 || deg > 4) return set_error(STOCHA_ERR_VALUE, "poly_degree must be in [1, 4]");
  return STOCHA_OK;
}

int lsmc_run(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t, uint64_t steps,
             uint64_t n_paths, int is_put, uint64_t deg, uint64_t seed, int precision, double* price,
             double* std_err) {
  int rc = lsmc_validate(s0, k, sigma, t, steps, n_paths, deg);
  if (rc) return rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  // GBM paths under the risk-neutral drift (lsmc.rs:29-39)
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_GBM;
  m.s0 = s0;
  m.mu = r;
  m.sigma = sigma;
  m.q = 0.0;
  m.t = t;
  m.steps = steps;
  m.n_paths = n_paths;
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  if ((rc = prepare_model(&m, &L, &row_len, &block))) return rc;
  make_stream_spec((u128)seed, block, &L.ss);
  fill_f32_constants(&L);
  L.tabs = ctx->d_tabs;
  L.err = ctx->d_err;
  L.time_major = 1;
  const size_t esz = precision == STOCHA_FP32 ? 4 : 8;
  if (n_paths > (SIZE_MAX / esz) / (steps + 1)) return set_error(STOCHA_ERR_NOMEM, "path array too large");
  if ((rc = ensure_buf(ctx, ctx->out, (size_t)n_paths * (steps + 1) * esz))) return rc;
  if (precision == STOCHA_FP32)
    L.out_f32 = (float*)ctx->out.ptr;
  else
    L.out_f64 = (double*)ctx->out.ptr;

  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const uint64_t want = (n_paths + 255) / 256;
  const int grid = (int)(want < (uint64_t)sms * 8 ? want : (uint64_t)sms * 8);
  // scratch: cf[n] | part[grid*14] | step params[steps] | result[2]
  const size_t off_part = (size_t)n_paths * 8;
  const size_t off_steps = off_part + (size_t)grid * 14 * 8;
  const size_t off_res = off_steps + ((steps * sizeof(LsmcStep) + 15) & ~(size_t)15);
  if ((rc = ensure_buf(ctx, ctx->aux, off_res + 16))) return rc;
  char* aux = (char*)ctx->aux.ptr;

  LsmcLaunch a;
  std::memset(&a, 0, sizeof a);
  a.spot = ctx->out.ptr;
  a.spot_f32 = precision == STOCHA_FP32;
  a.cf = (double*)aux;
  a.part = (double*)(aux + off_part);
  a.step_params = (LsmcStep*)(aux + off_steps);
  a.result = (double*)(aux + off_res);
  a.n = n_paths;
  a.steps = steps;
  a.k = k;
  const double dt = t / (double)steps;
  a.disc = std::exp(-r * dt);  // lsmc.rs:26-27
  a.is_put = is_put ? 1 : 0;
  a.deg = (int)deg;
  a.grid = grid;

  if ((rc = begin_call(ctx))) return rc;
  int g = precision == STOCHA_FP32 ? launch_paths_f32(L, ctx->stream) : launch_paths_f64(L, ctx->stream);
  if (g < 0) return cuda_error(cudaGetLastError(), "LSMC path launch");
  lsmc_sweep(a, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, a.result, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if ((rc = finish_call(ctx))) return rc;
  const double mean = ctx->h_small[0];
  const double n = (double)n_paths;
  const double var = ctx->h_small[1] / (n - 1.0);  // lsmc.rs:106-112
  *price = mean;
  *std_err = std::sqrt(var / n);
  return STOCHA_OK;
}

}  // namespace

extern "C" {

int stocha_lsmc_american_option(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t,
                                uint64_t steps, uint64_t n_paths, int32_t is_put, uint64_t poly_degree,
                                uint64_t seed, double* price, double* std_err) {
  return lsmc_run(ctx, s0, k, r, sigma, t, steps, n_paths, is_put, poly_degree, seed, STOCHA_FP64, price,
                  std_err);
}

int stocha_lsmc(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t, uint64_t steps,
                uint64_t n_paths, int32_t is_put, uint64_t poly_degree, uint64_t seed, int32_t precision,
                double* price, double* std_err) {
  return lsmc_run(ctx, s0, k, r, sigma, t, steps, n_paths, is_put, poly_degree, seed, precision, price, std_err);
}

}  // extern "C"
