/*
 * stocha_gpu.h — C ABI of the GB300 Monte Carlo engine behind stocha's API.
 *
 * Plain C: pointers, sizes and scalars only.  Every call returns STOCHA_OK (0)
 * or an error code; the message of the last failure on the calling thread is
 * available from stocha_last_error().  Messages of STOCHA_ERR_VALUE are the
 * reference's ValueError texts (src/lib.rs), so a binding can raise them as
 * they are.
 *
 * Contexts: a NULL ctx means the process-wide default context on device 0.
 * Calls on one context are serialised by the context; distinct contexts may
 * be used from distinct threads concurrently.
 *
 * Host-buffer calls (stocha_gbm, ...) block until the result is in the
 * caller's memory, like the reference's functions.  *_device calls take
 * device pointers and are asynchronous on the context's stream.
 */
#ifndef STOCHA_GPU_H
#define STOCHA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STOCHA_OK 0
#define STOCHA_ERR_VALUE 1    /* invalid argument: the reference raises ValueError */
#define STOCHA_ERR_CUDA 2     /* CUDA runtime failure */
#define STOCHA_ERR_NOMEM 3    /* device or pinned host allocation failed */
#define STOCHA_ERR_DEVICE 4   /* a kernel's own check failed (iteration cap) */
#define STOCHA_ERR_CALLBACK 5 /* a user payoff callback reported failure */
#define STOCHA_ERR_BUSY 6     /* serving: admission refused (memory budget) */
#define STOCHA_ERR_TIMEOUT 7  /* serving: a wait ended before the request finished */
#define STOCHA_ERR_CANCELLED 8 /* serving: the request was cancelled before it was admitted */

#define STOCHA_FP64 0 /* the reference's algorithm in FP64: paths within 1e-12 of its output */
#define STOCHA_FP32 1 /* FP32 paths, FP64 reductions */

#define STOCHA_MODEL_GBM 0
#define STOCHA_MODEL_HESTON 1
#define STOCHA_MODEL_MERTON 2
#define STOCHA_MODEL_MULTI_GBM 3
#define STOCHA_MODEL_HULL_WHITE 4 /* r0 in s0, a in kappa, theta, sigma (FP64 paths only) */

#define STOCHA_PAYOFF_CALL 0
#define STOCHA_PAYOFF_PUT 1

typedef struct stocha_ctx stocha_ctx;

/* Model description used by the pricing, batching and serving calls.
 * Fields a model does not use are ignored.  Heston scheme: 0 euler, 1 qe. */
typedef struct stocha_model {
  int32_t kind;
  int32_t scheme;
  double s0, mu, sigma, q, t;
  double v0, kappa, theta, xi, rho;
  double lambda_, mu_j, sigma_j;
  uint64_t steps, n_paths;
  int32_t antithetic;
  int32_t n_assets;      /* multi-GBM only */
  const double* s0_v;    /* [n_assets] */
  const double* mu_v;    /* [n_assets] */
  const double* sigma_v; /* [n_assets] */
  const double* corr;    /* [n_assets * n_assets], row-major */
} stocha_model;

/* ---------------------------------------------------------------- context */
int stocha_ctx_create(int device, stocha_ctx** out);
void stocha_ctx_destroy(stocha_ctx* ctx);
/* The cudaStream_t the context launches on (as void*). */
void* stocha_ctx_stream(stocha_ctx* ctx);
/* Launch on a caller-owned stream from now on (NULL: the context's own). */
int stocha_ctx_set_stream(stocha_ctx* ctx, void* cuda_stream);
/* Waits for the context's stream; reports device-side check failures of
 * earlier asynchronous (*_device) calls and clears them. */
int stocha_ctx_sync(stocha_ctx* ctx);
const char* stocha_last_error(void);
const char* stocha_version(void);

/* ------------------------------------------------------ host result cache
 * No counterpart in the reference (its functions return fresh NumPy arrays).
 * Delivering a large result into fresh host memory is bound by faulting its
 * pages in (~30 GB/s on a Grace host), while a copy into pages that already
 * exist runs at the chip-to-chip link's rate (~190 GB/s on GB300, the same as
 * pinned memory).  A binding that allocates its result arrays here gets back,
 * for later results of a similar size, buffers whose pages already exist.
 *   acquire: a buffer of at least `bytes` (page-aligned), a cached one of
 *     capacity bytes..bytes*5/4 when there is one, else fresh memory.
 *   release: hands a buffer from acquire back; it stays cached while the
 *     cached total is within the cap, else the oldest are unmapped.
 * The cap is STOCHA_HOST_CACHE_BYTES (bytes; 0 disables caching) or, by
 * default, an eighth of physical memory up to 64 GiB.  The host-buffer calls
 * (stocha_gbm, ...) skip the page population for a cached buffer. */
int stocha_host_buffer_acquire(size_t bytes, void** out);
int stocha_host_buffer_release(void* ptr);
/* Bytes now cached (released and kept) and the cap; either pointer may be NULL. */
int stocha_host_cache_stats(size_t* cached_bytes, size_t* cap_bytes);
/* Diagnostic (no counterpart in the reference): the 256 integer thresholds
 * of the ziggurat fast path; (u >> 11) < thr[u & 0xFF] is the reference's
 * test  (u >> 11) * 2^-53 * X[L] < X[L+1]  (src/dist/normal.rs:25-27). */
int stocha_debug_zig_thresholds(uint64_t* thr256);
/* Diagnostic (no counterpart in the reference): y[i] = exp(x[i]) by the
 * FP64 kernels' exponential, evaluated on the integer pipes (host buffers). */
int stocha_debug_exp(stocha_ctx* ctx, const double* x, double* y, uint64_t n);
/* Diagnostic (no counterpart in the reference): y[i] = sqrt(x[i]) by the FP64
 * kernels' correctly rounded integer-pipe square root (host buffers). */
int stocha_debug_sqrt(stocha_ctx* ctx, const double* x, double* y, uint64_t n);
/* Diagnostic (no counterpart in the reference): the FP64 kernels' helpers by
 * number: 0 exp (as stocha_debug_exp), 1 sqrt (as stocha_debug_sqrt), 2 the
 * normal's product (uint64)x[i] * X[L] 2^-53 with L = i mod 256 on the integer
 * pipes, 3 the same product by the FP64 pipe (they must agree bit for bit),
 * 4 exp in the early-exit form (bit for bit the same as 0), 5 the path
 * kernels' ziggurat tail value -ln(u1)/R + R for the draw whose 64 bits are
 * those of x[i] (u1 = (draw >> 11) 2^-53, draw >> 11 >= 1), 6 the same value
 * as the RNG's normals compute it (FP64 log and division). */
int stocha_debug_f64(stocha_ctx* ctx, int32_t fn, const double* x, double* y, uint64_t n);
/* Diagnostic (no counterpart in the reference): the error of the device's
 * hardware logarithm __logf over every normal float x in (0, 1), against
 * log(x) in FP64: the largest absolute error for x in [0.5, 1) and the
 * largest relative error for x < 0.5.  The FP32 ziggurat tail test's decision
 * margin rests on these bounds (an exhaustive scan, about a second). */
int stocha_debug_fast_log_error(stocha_ctx* ctx, double* abs_err_half_to_one, double* rel_err_below_half);
/* Diagnostic (no counterpart in the reference): the device samplers' iteration
 * caps.  Thread i < n draws once from the stream of path i (seed advanced by
 * i * 2050 draws, as a one-step gbm) into out[i] (host buffer), with one cap
 * lowered to `cap`: sampler 0 FP64 normal attempts, 1 FP64 normal tail
 * iterations, 2 FP32 normal attempts, 3 FP32 normal tail iterations, 4 gamma
 * (shape 2.5) rejections.  The reference's loops have no cap
 * (src/dist/normal.rs:54-67, src/copula/student_t.rs:93-119); the engine's
 * stop at 4096 (normals) and 2^20 (gamma), set an error bit and return.  A
 * draw that reaches the cap makes the call return STOCHA_ERR_DEVICE with the
 * cap named in stocha_last_error(); the next call starts clean. */
int stocha_debug_capped_draws(stocha_ctx* ctx, int32_t sampler, int32_t cap, uint64_t seed, uint64_t n,
                              double* out);
/* Diagnostic (no counterpart in the reference): the two FP32 samplers of the
 * engine on the same streams.  Stream i < n_paths is the seed's stream
 * advanced by i * (n + 1024) * 2 draws (gbm.rs:55-59); out[i * n + k] is its
 * k-th normal and state[2 i], state[2 i + 1] the generator state (low, high
 * words) after the last draw those n normals consumed (host buffers).
 * form 0: the per-path loop sampler (normal_f32); form 1: the warp-uniform
 * feed of the fused kernels (ZigFeed).  Both consume exactly the reference's
 * draws (src/dist/normal.rs:18-67), so they must agree bit for bit.
 * n_paths * n at most 2^36. */
int stocha_debug_zigfeed(stocha_ctx* ctx, int32_t form, uint64_t seed, uint64_t n_paths, uint32_t n, float* out,
                         uint64_t* state);
/* Diagnostic (no counterpart in the reference): measured peak rate of one
 * pipe for roofline denominators.  kind 0: FP32 FFMA flop/s, 1: FP64 DFMA
 * flop/s, 2: 32-bit IMAD op/s, 3: PCG64DXSM draws/s (generator alone). */
int stocha_measure_peak(stocha_ctx* ctx, int32_t kind, double* ops_per_s);

/* ------------------------------------------------------------ path models
 * Output: C-order float64, (n_paths, steps+1) or (n_paths, steps+1, n_assets);
 * the caller owns `out` (host memory). */

/* replaces #[pyfunction] gbm, src/lib.rs:205-252 -> finance/gbm.rs:42 gbm_paths */
int stocha_gbm(stocha_ctx* ctx, double s0, double mu, double sigma, double t, uint64_t steps, uint64_t n_paths,
               uint64_t seed, int32_t antithetic, double q, double* out);

/* replaces #[pyfunction] heston, src/lib.rs:327-408 -> finance/heston.rs:33
 * heston_paths_with_scheme; scheme "euler" or "qe" */
int stocha_heston(stocha_ctx* ctx, double s0, double v0, double mu, double kappa, double theta, double xi,
                  double rho, double t, uint64_t steps, uint64_t n_paths, uint64_t seed, const char* scheme,
                  double* out);

/* replaces #[pyfunction] merton_jump_diffusion, src/lib.rs:430-489 ->
 * finance/jump_diffusion.rs:48 merton_paths */
int stocha_merton_jump_diffusion(stocha_ctx* ctx, double s0, double mu, double sigma, double lambda_, double mu_j,
                                 double sigma_j, double t, uint64_t steps, uint64_t n_paths, uint64_t seed,
                                 double* out);

/* gaussian_copula (lib.rs:522-549, copula/gaussian.rs:15-99): n_samples x dim
 * uniforms from ONE sequential stream Pcg64Dxsm::new(seed) (normals drawn by
 * the parallel stream parse, bit-exact), out[n_samples * dim]. */
int stocha_gaussian_copula(stocha_ctx* ctx, const double* corr, size_t rows, size_t cols, uint64_t n_samples,
                           uint64_t seed, double* out);
/* student_t_copula (lib.rs:551-578, copula/student_t.rs:93-170): n_samples x dim
 * uniforms from ONE sequential stream; a sample's chi-square (Marsaglia-Tsang
 * gamma) and normals are found by a speculative parallel parse of the stream
 * (exact consumption), out[n_samples * dim]. */
int stocha_student_t_copula(stocha_ctx* ctx, const double* corr, size_t rows, size_t cols, double nu,
                            uint64_t n_samples, uint64_t seed, double* out);
/* hull_white (lib.rs:604-649, finance/hull_white.rs:26-57): short-rate paths
 * by the exact transition, out[n_paths * (steps+1)] (FP64). */
int stocha_hull_white(stocha_ctx* ctx, double r0, double a, double theta, double sigma, double t, uint64_t steps,
                      uint64_t n_paths, uint64_t seed, double* out);
/* replaces #[pyfunction] multi_gbm, src/lib.rs:759-827 ->
 * finance/multi_gbm.rs:22 multi_gbm_paths (+ copula/gaussian.rs:76 cholesky).
 * corr is row-major corr_rows x corr_cols. */
int stocha_multi_gbm(stocha_ctx* ctx, size_t n_assets, const double* s0, const double* mu, const double* sigma,
                     const double* corr, size_t corr_rows, size_t corr_cols, double t, uint64_t steps,
                     uint64_t n_paths, uint64_t seed, int32_t antithetic, double* out);

/* Device-resident form of the four calls above: paths of `m` written to the
 * device buffer out_dev (float64 for STOCHA_FP64, float32 for STOCHA_FP32),
 * asynchronously on the context's stream.  Same layout as the host calls. */
int stocha_paths_device(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, void* out_dev);

/* --------------------------------------------------------- fused pricing
 * European payoff of the terminal value, reduced in-kernel (no path array).
 * out[2*a], out[2*a+1] = discounted price and standard error for asset a
 * (one asset unless multi-GBM).  discount = exp(-rate * t).
 * No counterpart function in the reference: it replaces the reference
 * workflow "paths = gbm(...); price = exp(-rT) * mean(payoff(paths[:, -1]))"
 * (the same reduction greeks.rs:313-320 mc_price performs). */
int stocha_price(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff,
                 double strike, double rate, double* out);
/* Asynchronous form: out_dev is a device buffer of 2*n_assets doubles.
 * FP32: the result is the same bits run to run and for every launch shape
 * of a kernel form (rows are priced in 32-row batches from a work queue and
 * each batch's sums are added in a fixed order). */
int stocha_price_device(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff,
                        double strike, double rate, double* out_dev);

/* Fused pricing without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc: a host application
 * that owns all device memory, or a request path that must never reach the
 * allocator.  Same kernels as stocha_price_device (out_dev: 2 * n_assets
 * doubles of raw payoff sums, caller-owned device memory), on the caller's
 * cudaStream_t; scratch, tables and status live in static device arrays of
 * the library (1 MiB of scratch: at most 4 assets, 16384 partial records).
 * The sums are bit-equal to stocha_price_device's for FP64, and for FP32 up
 * to 524,288 rows; above that the FP32 work-queue batches grow past 32 rows
 * to fit the records, the sums are grouped differently and agree to FP32
 * rounding.  A launch that would need more records is refused (value error)
 * before anything runs.  Synchronous:
 * waits for `stream` and reports device-check failures.  The first call on a
 * device sets up its arrays (make it before any stream capture); calls that
 * overlap on the GPU share the arrays and race. */
int stocha_price_noalloc(const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff, double strike,
                         double* sums_dev, void* stream);

/* ----------------------------------------------------------------- LSMC */
/* replaces #[pyfunction] lsmc_american_option, src/lib.rs:854-918 ->
 * finance/lsmc.rs:25 lsmc_american_option.  FP64 paths (the reference's),
 * FP64 regression by normal equations.  Writes the price and its standard
 * error. */
int stocha_lsmc_american_option(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t,
                                uint64_t steps, uint64_t n_paths, int32_t is_put, uint64_t poly_degree,
                                uint64_t seed, double* price, double* std_err);
/* Same with the path precision chosen (STOCHA_FP32: FP32 paths, FP64
 * regression); no counterpart in the reference. */
int stocha_lsmc(stocha_ctx* ctx, double s0, double k, double r, double sigma, double t, uint64_t steps,
                uint64_t n_paths, int32_t is_put, uint64_t poly_degree, uint64_t seed, int32_t precision,
                double* price, double* std_err);

/* --------------------------------------------------------------- Greeks */
/* Model parameters of greeks_fd (the reference takes a dict, lib.rs:958-1040).
 * `present` has bit i set when field i (in declaration order: s0, r, sigma,
 * t, v0, kappa, theta, xi, rho, lambda_, mu_j, sigma_j) was given; the first
 * missing required key is reported as the reference does.  scheme: Heston
 * 0 euler, 1 qe, -1 for an unknown name. */
typedef struct stocha_greeks_params {
  double s0, r, sigma, t, v0, kappa, theta, xi, rho, lambda_, mu_j, sigma_j;
  uint32_t present;
  int32_t scheme;
} stocha_greeks_params;

/* Custom payoff: receives the n terminal prices of one scenario and returns
 * the sum of its payoff values (in order) and their count; non-zero return
 * aborts with STOCHA_ERR_CALLBACK. */
typedef int32_t (*stocha_payoff_fn)(void* user, const double* terminals, uint64_t n, double* payoff_sum,
                                    uint64_t* payoff_len);

/* replaces #[pyfunction] greeks_fd, src/lib.rs:1064-1156 -> finance/greeks.rs:322
 * greeks_fd_core.  model "gbm" | "heston" | "merton"; payoff "call" | "put",
 * or NULL with a callback.  greeks: names ("delta", "gamma", "vega",
 * "theta", "rho"); out[i] receives greeks[i].  precision STOCHA_FP64 runs the
 * reference's scenario-by-scenario revaluation; STOCHA_FP32 (built-in payoffs,
 * Heston euler) runs all scenarios of every path in one pass with common
 * random numbers. */
int stocha_greeks_fd(stocha_ctx* ctx, const char* model, const stocha_greeks_params* params, const char* payoff,
                     stocha_payoff_fn payoff_cb, void* user, double strike, uint64_t n_paths, uint64_t n_steps,
                     const char* const* greeks, uint64_t n_greeks, uint64_t seed, double bump_size,
                     int32_t precision, double* out);

/* replaces #[pyfunction] greeks_pathwise, src/lib.rs:1177-1242 ->
 * finance/greeks.rs:360 greeks_pathwise_core (GBM; "delta", "vega"). */
int stocha_greeks_pathwise(stocha_ctx* ctx, double s0, double r, double sigma, double t, double strike,
                           int32_t is_call, uint64_t n_paths, uint64_t n_steps, const char* const* greeks,
                           uint64_t n_greeks, uint64_t seed, double* out);

/* One instance of a batched Greeks run (no counterpart call in the
 * reference: each instance is one greeks_fd(model, params, payoff, strike,
 * n_paths, steps, all five greeks, seed, bump_size) call). */
typedef struct stocha_greeks_instance {
  int32_t model;  /* STOCHA_MODEL_GBM / _HESTON / _MERTON */
  int32_t payoff; /* STOCHA_PAYOFF_CALL / _PUT */
  int32_t scheme; /* Heston: 0 euler, 1 qe */
  int32_t pad;
  double s0, r, sigma, t, v0, kappa, theta, xi, rho, lambda_, mu_j, sigma_j, strike, bump_size;
  uint64_t n_paths, steps, seed;
} stocha_greeks_instance;

/* Prices and Greeks of n instances in one persistent launch (FP32 paths,
 * FP64 reductions) or, with STOCHA_FP64, instance by instance with the
 * reference's scenario revaluation.  out[7*i .. 7*i+6] = price, its standard
 * error, delta, gamma, vega, theta, rho. */
int stocha_greeks_batch(stocha_ctx* ctx, const stocha_greeks_instance* inst, uint64_t n, int32_t precision,
                        double* out);

/* ------------------------------------------------------------------ RNG
 * replaces #[pyclass] RNG, src/lib.rs:74-184 (-> prng/pcg64.rs, dist/normal.rs).
 * The state lives on the host (it is 48 bytes); draws are generated on the
 * device and the state advances exactly as the reference's sequential
 * generator would. */
typedef struct stocha_rng {
  uint64_t state_lo, state_hi; /* LCG state */
  uint64_t inc_lo, inc_hi;     /* LCG increment */
  uint64_t seed_lo, seed_hi;   /* seed (RNG.seed) */
} stocha_rng;

/* RNG(seed, algorithm): algorithm "pcg64dxsm" or "default" (lib.rs:87-101). */
int stocha_rng_new(uint64_t seed_lo, uint64_t seed_hi, const char* algorithm, stocha_rng* out);
/* RNG.uniform (lib.rs:110-113) */
int stocha_rng_uniform(stocha_ctx* ctx, stocha_rng* rng, uint64_t size, double* out);
/* RNG.standard_normal (lib.rs:116-120) */
int stocha_rng_standard_normal(stocha_ctx* ctx, stocha_rng* rng, uint64_t size, double* out);
/* RNG.normal (lib.rs:129-148) */
int stocha_rng_normal(stocha_ctx* ctx, stocha_rng* rng, uint64_t size, double loc, double scale, double* out);
/* RNG.save_state (lib.rs:158, pcg64.rs:58-65): JSON into buf (cap bytes);
 * *len receives the length without the terminating NUL. */
int stocha_rng_save_state(const stocha_rng* rng, char* buf, size_t cap, size_t* len);
/* RNG.from_state (lib.rs:173-179, pcg64.rs:68-77) */
int stocha_rng_from_state(const char* json, stocha_rng* out);
/* Raw generator output (no counterpart call in the reference API; used to
 * check the device generator against the reference bit for bit). */
int stocha_rng_raw_u64(stocha_ctx* ctx, stocha_rng* rng, uint64_t size, uint64_t* out);

/* -------------------------------------------------------- exotic options
 * replace barrier_price, asian_price, lookback_price (src/lib.rs:1549-1870;
 * src/finance/barrier.rs, asian.rs, lookback.rs).  Same argument checks and
 * messages; method "auto" / "analytical" / "mc".  The closed forms run on
 * the host (they are a few hundred flops); "mc" (and "auto" where the
 * reference falls back to it) runs the FP64 Monte Carlo kernel on the
 * device with the reference's streams.  Optional arguments: n_monitoring < 0
 * is None; running_avg, time_elapsed, running_max, running_min NaN is None.
 * precision: STOCHA_FP64 (the reference's arithmetic) or STOCHA_FP32 (a GB300
 * addition: the same draws, paths carried in log space in FP32; barrier
 * decisions can differ from FP64 only for paths within ~1e-7 of the barrier
 * in log price).  The closed forms ignore it. */
int stocha_barrier_price(stocha_ctx* ctx, double s, double k, double r, double sigma, double t, double barrier,
                         const char* barrier_type, const char* option_type, double q, uint64_t n_paths,
                         uint64_t n_steps, uint64_t seed, const char* method, int32_t n_monitoring, double rebate,
                         int32_t rebate_at_hit, int32_t precision, double* price);
int stocha_asian_price(stocha_ctx* ctx, double s, double k, double r, double sigma, double t, uint64_t n_steps,
                       const char* average_type, const char* strike_type, const char* option_type, double q,
                       uint64_t n_paths, uint64_t seed, const char* method, double running_avg, double time_elapsed,
                       int32_t precision, double* price);
int stocha_lookback_price(stocha_ctx* ctx, double s, double r, double sigma, double t, uint64_t n_steps,
                          const char* strike_type, const char* option_type, double k, double q, uint64_t n_paths,
                          uint64_t seed, const char* method, double running_max, double running_min,
                          int32_t precision, double* price);

/* --------------------------------------------------------------- VaR/CVaR
 * replaces var_cvar (src/lib.rs:505-520, src/risk/var_cvar.rs:7-43):
 * out2 = {VaR, CVaR} of the losses -returns at `confidence`.  The returns are
 * host memory (stocha_var_cvar) or device memory (stocha_var_cvar_device,
 * e.g. returns computed from device-resident paths).  No sort: a radix
 * select on total-order keys finds the VaR loss exactly; CVaR is the mean of
 * the sorted tail. */
int stocha_var_cvar(stocha_ctx* ctx, const double* returns, uint64_t n, double confidence, double* out2);
int stocha_var_cvar_device(stocha_ctx* ctx, const double* returns_dev, uint64_t n, double confidence, double* out2);

/* ------------------------------------------------------------- autotuner
 * No counterpart in the reference.  The fused FP32 pricing kernels have a
 * launch shape per model kind: the kernel form (variant 0: one path per
 * thread at a time; variant 1: ilp paths per thread in lockstep, 1 or 2;
 * variant 2: one path per thread, the ziggurat fed one draw per warp-wide
 * iteration so that wedge and tail attempts do not stall the warp), threads
 * per block (64/128/256) and grid waves (1 or 2 times the resident blocks):
 * 24 shapes.  stocha_autotune times every shape on the given model
 * and size (reps launches each, CUDA events on the context's stream) and
 * installs the fastest for that model kind; the table is process-wide.
 * Before any tuning every kind uses variant 2, 256 threads, 2 waves.
 * Draws and per-path values do not depend on the shape; the grouping of the
 * FP32 payoff partial sums does (their last bits). */
typedef struct stocha_tune_result {
  int32_t model, n_assets; /* STOCHA_MODEL_*; n_assets for multi-GBM (1..4) */
  int32_t block, ilp, waves, variant;
  int32_t candidates;      /* shapes timed */
  int32_t pad;
  double ms_best, ms_default; /* per launch: the chosen shape, and the default (variant 2 / 256 / 2 waves) */
} stocha_tune_result;

int stocha_autotune(stocha_ctx* ctx, const stocha_model* m, int32_t reps, stocha_tune_result* out);
int stocha_tune_get(int32_t model, int32_t n_assets, stocha_tune_result* out);
int stocha_tune_set(int32_t model, int32_t n_assets, int32_t block, int32_t ilp, int32_t waves, int32_t variant);

/* -------------------------------------------------------------- serving
 * No counterpart in the reference (its API is one blocking call per
 * pricing).  A server owns one device-memory budget, a set of CUDA streams
 * ("lanes": an eighth at the highest stream priority for small pricing and
 * Greeks batches, a quarter at a middle priority for LSMC jobs, the rest at
 * the lowest for large pricing and Greeks requests) and a dispatcher thread
 * that
 * admits requests as their bytes fit and batches small pricing/Greeks
 * requests into one launch as they arrive; each request is computed as the
 * reference's call would be:
 *   STOCHA_REQ_PRICE   European call/put price and standard error
 *                      (greeks.rs:322-329 mc_price), FP32 paths
 *   STOCHA_REQ_GREEKS  greeks_fd with all five Greeks (greeks.rs:330-358),
 *                      FP32 common-random-number batch
 *   STOCHA_REQ_LSMC    lsmc_american_option (lsmc.rs:25-115), FP32 paths
 *                      and FP64 regression; inst.payoff selects put/call,
 *                      inst.strike is k, inst.r the rate, poly_degree the
 *                      polynomial degree
 * Results depend only on the request, never on what else is in flight. */
#define STOCHA_REQ_PRICE 0
#define STOCHA_REQ_GREEKS 1
#define STOCHA_REQ_LSMC 2

typedef struct stocha_server stocha_server;

typedef struct stocha_request {
  int32_t kind;        /* STOCHA_REQ_* */
  int32_t poly_degree; /* LSMC: 1..4 */
  stocha_greeks_instance inst;
} stocha_request;

typedef struct stocha_result {
  int32_t status; /* 0 pending, 1 done, -STOCHA_ERR_* if the request failed */
  int32_t pad;
  double price, std_err;
  double greeks[5];                 /* delta gamma vega theta rho (STOCHA_REQ_GREEKS) */
  double t_submit, t_admit, t_done; /* seconds on the server's clock */
} stocha_result;

typedef struct stocha_server_counters {
  uint64_t submitted, completed, failed, jobs, batched_requests;
  uint64_t budget_bytes, peak_bytes, in_use_bytes;
  int32_t lanes, high_lanes; /* high_lanes: lanes above the lowest priority */
  uint64_t cancelled;
} stocha_server_counters;

int stocha_server_create(int32_t device, uint64_t budget_bytes, int32_t lanes, stocha_server** out);
/* Finishes every submitted request, then releases the server. */
int stocha_server_destroy(stocha_server* s);
/* Validates (the reference's messages) and queues a request. */
int stocha_server_submit(stocha_server* s, const stocha_request* req, uint64_t* ticket);
int stocha_server_poll(stocha_server* s, uint64_t ticket, stocha_result* out);
/* Cancels a request that has not been admitted yet (it still waits for a lane
 * or for device memory): *cancelled = 1, and its result's status becomes
 * -STOCHA_ERR_CANCELLED.  A request already admitted runs to completion:
 * *cancelled = 0.  Admission and cancellation are ordered under the server's
 * lock, so exactly one of them wins. */
int stocha_server_cancel(stocha_server* s, uint64_t ticket, int32_t* cancelled);
/* timeout_s < 0: wait without limit. */
int stocha_server_wait(stocha_server* s, uint64_t ticket, double timeout_s, stocha_result* out);
/* Open-loop load: submits reqs[i] at arrival_s[i] seconds after the call
 * starts, then waits for all; out[i] is request i's result. */
int stocha_server_replay(stocha_server* s, const stocha_request* reqs, const double* arrival_s, uint64_t n,
                         stocha_result* out);
int stocha_server_stats(stocha_server* s, stocha_server_counters* out);
/* Diagnostic (no counterpart in the reference): the serving arena's
 * allocator on a host-only script, see serve.cpp. */
int stocha_debug_arena(uint64_t capacity, const int64_t* ops, uint64_t n, int64_t* res);

#ifdef __cplusplus
}
#endif
#endif /* STOCHA_GPU_H */
