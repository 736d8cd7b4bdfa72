// C-ABI of the Monte Carlo engine: contexts, argument validation with the
// reference's messages (src/lib.rs), host preparation of every constant the
// kernels start from (in the reference's expression order; this file is
// built with -ffp-contract=off), and the path / pricing entry points.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "exp_table.inc"
#include "copula_t_kernels.h"
#include "host_common.h"
#include "ziggurat_table.inc"

namespace stocha {

namespace {
thread_local std::string g_err;
stocha_ctx* g_default = nullptr;
std::mutex g_default_mu;

const u128 kStreamOffset = ((u128)0xda3e39cb94b95bdbULL << 64) | (u128)0x7ef55da5c0374f5aULL;  // pcg64.rs:25

// Switches the calling thread to the context's device for one call.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Smallest m in [0, 2^53] with  (double)m * xs >= x_next ; 2^53 if none.
// Equivalently: the reference's fast-path test  u_frac*X[L] < X[L+1]
// (normal.rs:25-27) holds iff (u >> 11) < threshold.
uint64_t fast_threshold(double xs, double x_next) {
  uint64_t lo = 0, hi = 1ull << 53;
  while (lo < hi) {
    uint64_t mid = lo + (hi - lo) / 2;
    volatile double prod = (double)mid * xs;
    if (prod >= x_next)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

void build_tables(ZigTables* t) {
  static const double X[257] = STOCHA_ZIG_X_INIT;
  static const double Y[257] = STOCHA_ZIG_Y_INIT;
  std::memset(t, 0, sizeof *t);
  for (int i = 0; i < 257; ++i) {
    t->x[i] = X[i];
    t->y[i] = Y[i];
    t->x32[i] = (float)X[i];
    t->y32[i] = (float)Y[i];
  }
  for (int L = 0; L < 256; ++L) {
    t->xs[L] = std::ldexp(X[L], -53);
    t->thr[L] = fast_threshold(t->xs[L], X[L + 1]);
  }
  t->r = STOCHA_ZIG_R_HEX;
  t->r32 = (float)t->r;
  t->nrinv32 = (float)(-1.0 / t->r);
  t->nrinv = -1.0 / t->r;
  static const uint64_t E2[256] = STOCHA_EXP2_Q63_INIT;
  for (int j = 0; j < 256; ++j) t->exp2q[j] = E2[j];
}

// Brown's arbitrary-stride LCG jump (rand_pcg advance, pcg64.rs:41-43):
// state' = A*state + C after `delta` steps.
void lcg_affine(u128 inc, u128 delta, u128* A, u128* C) {
  u128 acc_mult = 1, acc_plus = 0, cur_mult = kPcgMul, cur_plus = inc;
  while (delta > 0) {
    if (delta & 1) {
      acc_mult *= cur_mult;
      acc_plus = acc_plus * cur_mult + cur_plus;
    }
    cur_plus = (cur_mult + 1) * cur_plus;
    cur_mult *= cur_mult;
    delta >>= 1;
  }
  *A = acc_mult;
  *C = acc_plus;
}

int create_ctx(int device, stocha_ctx** out) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return set_error(STOCHA_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return set_error(STOCHA_ERR_VALUE, "device index out of range");
  DeviceGuard g(device);
  stocha_ctx* c = new stocha_ctx();
  c->device = device;
  auto fail = [&](cudaError_t err, const char* what) {
    int rc = cuda_error(err, what);
    stocha_ctx_destroy(c);
    return rc;
  };
  if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
  c->stream = c->own;
  ZigTables host;
  build_tables(&host);
  if ((e = cudaMalloc(&c->d_tabs, sizeof(ZigTables))) != cudaSuccess) return fail(e, "tables");
  if ((e = cudaMemcpy(c->d_tabs, &host, sizeof host, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "tables");
  if ((e = cudaMalloc(&c->d_err, sizeof(unsigned))) != cudaSuccess) return fail(e, "err");
  if ((e = cudaMemset(c->d_err, 0, sizeof(unsigned))) != cudaSuccess) return fail(e, "err");
  if ((e = cudaMallocHost(&c->h_err, sizeof(unsigned))) != cudaSuccess) return fail(e, "err");
  if ((e = cudaMallocHost(&c->h_small, 4096 * sizeof(double))) != cudaSuccess) return fail(e, "small");
  *out = c;
  return STOCHA_OK;
}

// Decimal digits of a u128.
std::string u128_str(u128 v) {
  if (v == 0) return "0";
  char buf[48];
  int i = 47;
  buf[i] = 0;
  while (v > 0) {
    buf[--i] = (char)('0' + (int)(v % 10));
    v /= 10;
  }
  return std::string(buf + i);
}

}  // namespace

void fill_zig_tables(ZigTables* t) { build_tables(t); }

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  return set_error(STOCHA_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e) + " (" + what + ")");
}

int resolve_ctx(stocha_ctx** ctx) {
  if (*ctx) return STOCHA_OK;
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default) {
    int rc = create_ctx(0, &g_default);
    if (rc) return rc;
  }
  *ctx = g_default;
  return STOCHA_OK;
}

int ensure_buf(stocha_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes && b.ptr) return STOCHA_OK;
  if (b.ptr) {
    cudaStreamSynchronize(c->stream);
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.ptr, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(STOCHA_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
                                           cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return STOCHA_OK;
}

int begin_call(stocha_ctx* c) {
  STOCHA_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
  return STOCHA_OK;
}

int finish_call(stocha_ctx* c) {
  STOCHA_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  STOCHA_CUDA(cudaStreamSynchronize(c->stream));
  STOCHA_CUDA(cudaGetLastError());
  unsigned e = *c->h_err;
  if (e) {
    cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream);
    std::string what;
    if (e & kErrZigAttempts) what += " normal-draw attempt cap reached;";
    if (e & kErrTailIters) what += " ziggurat tail iteration cap reached;";
    if (e & kErrQueue) what += " work-queue inconsistency;";
    if (e & kErrGammaIters) what += " gamma rejection cap reached;";
    return set_error(STOCHA_ERR_DEVICE, "device check failed:" + what);
  }
  return STOCHA_OK;
}

void pcg_seed(u128 seed, u128* state, u128* inc) {  // pcg64.rs:23-30 -> Lcg128CmDxsm64::new
  u128 stream = seed + kStreamOffset;
  *inc = (stream << 1) | 1;
  u128 s = seed + *inc;
  *state = s * kPcgMul + *inc;
}

void pcg_advance(u128* state, u128 inc, u128 delta) {
  u128 A, C;
  lcg_affine(inc, delta, &A, &C);
  *state = A * *state + C;
}

static void fill_jumps(u128 inc, u128 block, StreamSpec* ss) {
  u128 A, C;
  lcg_affine(inc, block, &A, &C);
  for (int j = 0; j < kMaxJumpBits; ++j) {
    ss->jump[j].mul_lo = (uint64_t)A;
    ss->jump[j].mul_hi = (uint64_t)(A >> 64);
    ss->jump[j].add_lo = (uint64_t)C;
    ss->jump[j].add_hi = (uint64_t)(C >> 64);
    u128 A2 = A * A, C2 = A * C + C;
    A = A2;
    C = C2;
  }
}

void make_stream_spec(u128 seed, u128 block, StreamSpec* ss) {
  u128 st, inc;
  pcg_seed(seed, &st, &inc);
  ss->base_lo = (uint64_t)st;
  ss->base_hi = (uint64_t)(st >> 64);
  ss->inc_lo = (uint64_t)inc;
  ss->inc_hi = (uint64_t)(inc >> 64);
  fill_jumps(inc, block, ss);
}

void make_stream_spec_state(u128 state, u128 inc, u128 block, StreamSpec* ss) {
  ss->base_lo = (uint64_t)state;
  ss->base_hi = (uint64_t)(state >> 64);
  ss->inc_lo = (uint64_t)inc;
  ss->inc_hi = (uint64_t)(inc >> 64);
  fill_jumps(inc, block, ss);
}

std::string rust_f64(double v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
  char buf[512];
  auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::fixed);
  return std::string(buf, r.ptr);
}

// u < p with u = m*2^-53 (next_f64)  <=>  m < ceil(p*2^53)
uint64_t unit_threshold(double p) {
  if (!(p > 0.0)) return 0;  // also NaN
  double P = std::ldexp(p, 53);
  if (P >= 18446744073709551615.0) return ~0ull;
  return (uint64_t)std::ceil(P);
}

static double powi2(double a) { return a * a; }  // Rust powi(2)

int prepare_model(const stocha_model* m, PathLaunch* L, uint64_t* row_len, u128* block, bool check) {
  std::memset(L, 0, sizeof *L);
  L->model = m->kind;
  L->steps = m->steps;
  L->rows = m->n_paths;
  L->base_paths = m->n_paths;
  const double steps_f = (double)m->steps;
  switch (m->kind) {
    case STOCHA_MODEL_GBM: {  // lib.rs:219-238, gbm.rs:43-55
      if (check) {
        if (m->s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
        if (m->sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
        if (m->t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
        if (m->steps == 0 || m->n_paths == 0)
          return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
      }
      const double dt = m->t / steps_f;
      L->gbm.s0 = m->s0;
      L->gbm.drift = (m->mu - m->q - 0.5 * m->sigma * m->sigma) * dt;
      L->gbm.diffusion = m->sigma * std::sqrt(dt);
      if (m->antithetic) L->base_paths = (m->n_paths + 1) / 2;
      *row_len = m->steps + 1;
      *block = ((u128)m->steps + 1024) * 2;
      return STOCHA_OK;
    }
    case STOCHA_MODEL_HESTON: {  // lib.rs:342-391, heston.rs:44-150
      if (check) {
        if (m->s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
        if (m->v0 < 0.0) return set_error(STOCHA_ERR_VALUE, "v0 must be non-negative");
        if (m->kappa <= 0.0) return set_error(STOCHA_ERR_VALUE, "kappa must be positive");
        if (m->theta <= 0.0) return set_error(STOCHA_ERR_VALUE, "theta must be positive");
        if (m->xi <= 0.0) return set_error(STOCHA_ERR_VALUE, "xi must be positive");
        if (m->rho < -1.0 || m->rho > 1.0) return set_error(STOCHA_ERR_VALUE, "rho must be in [-1, 1]");
        if (m->t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
        if (m->steps == 0 || m->n_paths == 0)
          return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
      }
      if (m->scheme != 0 && m->scheme != 1) return set_error(STOCHA_ERR_VALUE, "scheme must be 'euler' or 'qe'");
      HestonK& h = L->heston;
      h.s0 = m->s0;
      h.v0 = m->v0;
      h.mu = m->mu;
      h.kappa = m->kappa;
      h.theta = m->theta;
      h.xi = m->xi;
      h.rho = m->rho;
      h.scheme = m->scheme;
      h.dt = m->t / steps_f;
      h.sqrt_dt = std::sqrt(h.dt);
      h.rho_comp = std::sqrt(1.0 - m->rho * m->rho);
      h.kdt = m->kappa * h.dt;
      h.xi_rho = m->xi * m->rho;
      h.xi_rho_comp = m->xi * h.rho_comp;
      // QE constants (heston.rs:93-94,112-116,143-150): loop-invariant
      // leading subexpressions, evaluated in the reference's order.
      h.e_kdt = std::exp(-m->kappa * h.dt);
      h.k1 = m->kappa * m->theta;
      h.qe_m0 = h.k1 * (1.0 - h.e_kdt) / m->kappa;
      h.one_m_ekdt = 1.0 - h.e_kdt;
      h.qe_s2b = h.k1 * m->xi * m->xi * powi2(1.0 - h.e_kdt) / (2.0 * m->kappa * m->kappa);
      const double krx = m->kappa * m->rho / m->xi;
      h.k0_s = (m->mu - krx * m->theta) * h.dt;
      h.k1_s = 0.5 * h.dt * (krx - 0.5) - m->rho / m->xi;
      h.k2_s = 0.5 * h.dt * (krx - 0.5) + m->rho / m->xi;
      h.k3_s = 0.5 * h.dt * (1.0 - m->rho * m->rho);
      h.k4_s = 0.5 * h.dt * (1.0 - m->rho * m->rho);
      *row_len = m->steps + 1;
      *block = ((u128)m->steps + 1024) * 6;
      return STOCHA_OK;
    }
    case STOCHA_MODEL_MERTON: {  // lib.rs:445-468, jump_diffusion.rs:49-64
      if (check) {
        if (m->s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
        if (m->sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
        if (m->lambda_ < 0.0) return set_error(STOCHA_ERR_VALUE, "lambda_ must be non-negative");
        if (m->sigma_j < 0.0) return set_error(STOCHA_ERR_VALUE, "sigma_j must be non-negative");
        if (m->t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
        if (m->steps == 0 || m->n_paths == 0)
          return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
      }
      const double dt = m->t / steps_f;
      const double sqrt_dt = std::sqrt(dt);
      const double m_bar = std::exp(m->mu_j + 0.5 * m->sigma_j * m->sigma_j) - 1.0;
      MertonK& M = L->merton;
      M.s0 = m->s0;
      M.drift = (m->mu - 0.5 * m->sigma * m->sigma - m->lambda_ * m_bar) * dt;
      M.diffusion = m->sigma * sqrt_dt;
      M.mu_j = m->mu_j;
      M.sigma_j = m->sigma_j;
      M.jump_thr = unit_threshold(m->lambda_ * dt);
      *row_len = m->steps + 1;
      *block = ((u128)m->steps + 1024) * 8;
      return STOCHA_OK;
    }
    case STOCHA_MODEL_MULTI_GBM: {  // lib.rs:771-812, multi_gbm.rs:22-40
      const int na = m->n_assets;
      if (na <= 0) return set_error(STOCHA_ERR_VALUE, "s0 must not be empty");
      for (int i = 0; i < na; ++i)
        if (m->s0_v[i] <= 0.0) return set_error(STOCHA_ERR_VALUE, "all s0 must be positive");
      for (int i = 0; i < na; ++i)
        if (m->sigma_v[i] <= 0.0) return set_error(STOCHA_ERR_VALUE, "all sigma must be positive");
      if (m->t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
      if (m->steps == 0 || m->n_paths == 0) return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
      if (na > kMaxAssets)
        return set_error(STOCHA_ERR_VALUE, "n_assets above " + std::to_string(kMaxAssets) + " is not supported");
      MultiK& K = L->multi;
      K.na = na;
      // Cholesky of corr (copula/gaussian.rs:76-99)
      double l[kMaxAssets * kMaxAssets] = {0};
      for (int i = 0; i < na; ++i)
        for (int j = 0; j <= i; ++j) {
          double sum = m->corr[i * na + j];
          for (int k = 0; k < j; ++k) sum -= l[i * na + k] * l[j * na + k];
          if (i == j) {
            if (sum <= 0.0)
              return set_error(STOCHA_ERR_VALUE, "matrix is not positive-definite (diagonal element " +
                                                     std::to_string(i) + " = " + rust_f64(sum) + ")");
            l[i * na + j] = std::sqrt(sum);
          } else {
            l[i * na + j] = sum / l[j * na + j];
          }
        }
      const double dt = m->t / steps_f;
      const double sqrt_dt = std::sqrt(dt);
      for (int i = 0; i < na; ++i) {
        K.s0[i] = m->s0_v[i];
        K.drift[i] = (m->mu_v[i] - 0.5 * m->sigma_v[i] * m->sigma_v[i]) * dt;
        K.diffusion[i] = m->sigma_v[i] * sqrt_dt;
        for (int j = 0; j < na; ++j) {
          K.L[i * kMaxAssets + j] = l[i * na + j];
          K.LD[i * kMaxAssets + j] = K.diffusion[i] * l[i * na + j];
        }
      }
      if (m->antithetic) L->base_paths = (m->n_paths + 1) / 2;
      *row_len = (m->steps + 1) * (uint64_t)na;
      *block = ((u128)m->steps * (u128)na + 1024) * 2;
      return STOCHA_OK;
    }
    case STOCHA_MODEL_HULL_WHITE: {  // lib.rs:617-636, hull_white.rs:26-45 (r0 in s0, a in kappa)
      if (check) {
        if (m->kappa <= 0.0) return set_error(STOCHA_ERR_VALUE, "a must be positive");
        if (m->sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
        if (m->t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
        if (m->steps == 0 || m->n_paths == 0)
          return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
      }
      const double dt = m->t / steps_f;
      const double e = std::exp(-m->kappa * dt);
      HullWhiteK& H = L->hw;
      H.r0 = m->s0;
      H.e = e;
      H.mean_reversion = (m->theta / m->kappa) * (1.0 - e);
      H.vol = m->sigma * std::sqrt((1.0 - e * e) / (2.0 * m->kappa));
      *row_len = m->steps + 1;
      *block = ((u128)m->steps + 1024) * 4;
      return STOCHA_OK;
    }
    default:
      return set_error(STOCHA_ERR_VALUE, "unknown model kind");
  }
}

void fill_f32_constants(PathLaunch* L) {
  F32K& f = L->f32;
  const double steps = (double)L->steps;
  f.strike = (float)L->strike;
  f.g_s0 = (float)L->gbm.s0;
  f.g_kdrift = (float)(steps * L->gbm.drift);
  f.g_diff = (float)L->gbm.diffusion;
  f.g_drift = (float)L->gbm.drift;
  f.m_s0 = (float)L->merton.s0;
  f.m_kdrift = (float)(steps * L->merton.drift);
  f.m_diff = (float)L->merton.diffusion;
  f.m_drift = (float)L->merton.drift;
  f.m_mu_j = (float)L->merton.mu_j;
  f.m_sigma_j = (float)L->merton.sigma_j;
  const HestonK& h = L->heston;
  f.h_s0 = (float)h.s0;
  f.h_v0 = (float)h.v0;
  f.h_rho = (float)h.rho;
  f.h_rho_comp = (float)h.rho_comp;
  f.h_kdt = (float)(h.kappa * h.dt);
  f.h_theta = (float)h.theta;
  f.h_xsdt = (float)(h.xi * h.sqrt_dt);
  f.h_nhdt = (float)(-0.5 * h.dt);
  f.h_mudt = (float)(h.mu * h.dt);
  f.h_sdt = (float)h.sqrt_dt;
  f.q_ekdt = (float)h.e_kdt;
  f.q_m0 = (float)h.qe_m0;
  f.q_cs2 = h.kappa > 0.0 ? (float)(h.xi * h.xi * h.e_kdt * h.one_m_ekdt / h.kappa) : 0.0f;
  f.q_s2b = (float)h.qe_s2b;
  f.q_k0 = (float)h.k0_s;
  f.q_k1 = (float)h.k1_s;
  f.q_k2 = (float)h.k2_s;
  f.q_k3 = (float)h.k3_s;
  f.q_k4 = (float)h.k4_s;
  f.q_ls0 = h.s0 > 0.0 ? (float)std::log(h.s0) : 0.0f;
  for (int i = 0; i < kMaxAssets; ++i) {
    f.a_s0[i] = (float)L->multi.s0[i];
    f.a_kdrift[i] = (float)(steps * L->multi.drift[i]);
    f.a_diff[i] = (float)L->multi.diffusion[i];
    f.a_drift[i] = (float)L->multi.drift[i];
    for (int j = 0; j < kMaxAssets; ++j) f.a_L[i * kMaxAssets + j] = (float)L->multi.L[i * kMaxAssets + j];
  }
}

// Materialises the paths of `m` into device memory (async, ctx stream).
// Rows [row_begin, row_begin + rows) of the model's paths into out_dev (which
// holds the whole array); rows == UINT64_MAX: all of them.
static int paths_to_device(stocha_ctx* c, const stocha_model* m, uint64_t seed, int precision, void* out_dev,
                           uint64_t row_begin = 0, uint64_t rows = UINT64_MAX) {
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(m, &L, &row_len, &block);
  if (rc) return rc;
  make_stream_spec((u128)seed, block, &L.ss);
  L.tabs = c->d_tabs;
  L.err = c->d_err;
  fill_f32_constants(&L);
  if (rows != UINT64_MAX) {
    L.row_begin = row_begin;
    L.rows = rows;
  }
  const size_t off = (size_t)L.row_begin * row_len;
  if (precision == STOCHA_FP32)
    L.out_f32 = (float*)out_dev + off;
  else
    L.out_f64 = (double*)out_dev + off;
  int g = precision == STOCHA_FP32 ? launch_paths_f32(L, c->stream) : launch_paths_f64(L, c->stream);
  if (g < 0) return cuda_error(cudaGetLastError(), "path kernel launch");
  return STOCHA_OK;
}

// Materialised results at least this large overlap their copy with compute
// when the destination is a cached host buffer.  The steady chunk is
// max(2^17, rows / 8) rows: 2^17 is about one wave of the FP64 kernels'
// resident threads (7 blocks of 128 per SM on 152 SMs), so a chunk fills the
// device.  The chunks before it ramp up from 2^14 rows, doubling: a thread
// computes its whole row, so a full-wave first chunk would hold back the
// first copy for a whole wave's time (about 1 ms for 3-asset multi-GBM at
// 252 steps), while 2^14 rows (one warp per scheduler) finish in a fraction
// of that; each next chunk computes while the one before it copies.
// Measured on GB300 at 1e6 x 252 FP64 into a cached buffer (median call):
// multi-GBM 32.73 -> 31.93 ms, Merton 11.02 -> 10.74 ms, Heston 11.57 ->
// 11.70 ms (a 1.5x ramp, more chunks: 11.78 ms); the link alone takes 31.4
// and 10.5 ms.  Chunk rows are multiples of 32, so every chunk starts on a
// whole warp of rows.
constexpr size_t kOverlapMin = 64u << 20;
constexpr uint64_t kOverlapMaxChunks = 8, kOverlapMinRows = 1u << 17, kOverlapFirstRows = 1u << 14;
constexpr int kOverlapMaxTotal = 32;
static_assert(sizeof(stocha_ctx::chunk_done) / sizeof(cudaEvent_t) >= kOverlapMaxTotal, "one event per chunk");

// Row boundaries of the overlapped chunks: bound[0] = 0 < ... < bound[n] =
// rows.  Returns n: at most 9 steady chunks after a ramp of at most 20
// chunks below 2^36 rows.
static int overlap_chunks(uint64_t rows, uint64_t bound[kOverlapMaxTotal + 1]) {
  const uint64_t per = (std::max<uint64_t>(kOverlapMinRows, (rows + kOverlapMaxChunks - 1) / kOverlapMaxChunks) + 31) /
                       32 * 32;
  int n = 0;
  bound[0] = 0;
  for (uint64_t r = 0, size = kOverlapFirstRows; r < rows && n < kOverlapMaxTotal; ++n) {
    r = std::min<uint64_t>(rows, r + std::min(size, per));
    bound[n + 1] = r;
    if (size < per) size *= 2;
  }
  return n;
}

static int paths_to_host(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, double* out) {
  // Arguments are validated before any CUDA call (as the reference validates
  // before simulating).
  PathLaunch probe;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(m, &probe, &row_len, &block);
  if (rc) return rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if (row_len != 0 && m->n_paths > (SIZE_MAX / 8) / row_len)
    return set_error(STOCHA_ERR_NOMEM, "output size overflows the address space");
  const size_t bytes = (size_t)m->n_paths * row_len * sizeof(double);
  if ((rc = ensure_buf(ctx, ctx->out, bytes))) return rc;
  if ((rc = begin_call(ctx))) return rc;
  if (bytes >= kOverlapMin && m->n_paths >= 2 * kOverlapMinRows && host_dst_cached(out, bytes)) {
    // The destination's pages exist, so each chunk's copy runs at the link's
    // rate: compute the rows in chunks and copy chunk i on a second stream
    // while chunk i + 1 computes.  Rows are contiguous in the output and each
    // row is a function of its own index, so the result is the same.
    if (!ctx->copy_stream) {
      STOCHA_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
      for (cudaEvent_t& e : ctx->chunk_done) STOCHA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    uint64_t bound[kOverlapMaxTotal + 1];
    const int nch = overlap_chunks(m->n_paths, bound);
    if (bound[nch] != m->n_paths) return set_error(STOCHA_ERR_VALUE, "too many rows for the overlapped copy");
    for (int i = 0; i < nch; ++i) {
      if ((rc = paths_to_device(ctx, m, seed, STOCHA_FP64, ctx->out.ptr, bound[i], bound[i + 1] - bound[i]))) return rc;
      STOCHA_CUDA(cudaEventRecord(ctx->chunk_done[i], ctx->stream));
    }
    for (int i = 0; i < nch; ++i) {
      const uint64_t r0 = bound[i], r1 = bound[i + 1];
      STOCHA_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_done[i], 0));
      const size_t o = (size_t)r0 * row_len, n = (size_t)(r1 - r0) * row_len;
      STOCHA_CUDA(cudaMemcpyAsync(out + o, (const double*)ctx->out.ptr + o, n * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->copy_stream));
    }
    STOCHA_CUDA(cudaStreamSynchronize(ctx->copy_stream));
    return finish_call(ctx);
  }
  if ((rc = paths_to_device(ctx, m, seed, STOCHA_FP64, ctx->out.ptr))) return rc;
  if ((rc = copy_to_host_populated(ctx->stream, out, ctx->out.ptr, bytes))) return rc;
  return finish_call(ctx);
}

int price_launch(stocha_ctx* c, const stocha_model* m, uint64_t seed, int precision, int payoff, double strike,
                 const double* aux4, bool check, double* sums_dev, int* nvals) {
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(m, &L, &row_len, &block, check);
  if (rc) return rc;
  if (payoff < kCall || payoff > kPwVegaPut || (precision == STOCHA_FP32 && payoff > kPut))
    return set_error(STOCHA_ERR_VALUE, "payoff must be call or put");
  make_stream_spec((u128)seed, block, &L.ss);
  L.tabs = c->d_tabs;
  L.err = c->d_err;
  L.strike = strike;
  L.payoff = payoff;
  if (aux4)
    for (int i = 0; i < 4; ++i) L.aux[i] = aux4[i];
  fill_f32_constants(&L);
  if (L.rows == 0) {  // nothing to simulate: zero sums
    const int na0 = m->kind == STOCHA_MODEL_MULTI_GBM ? m->n_assets : 1;
    STOCHA_CUDA(cudaMemsetAsync(sums_dev, 0, 2 * na0 * sizeof(double), c->stream));
    *nvals = 2 * na0;
    return STOCHA_OK;
  }
  const int na = m->kind == STOCHA_MODEL_MULTI_GBM ? m->n_assets : 1;
  // partial records: at most (SMs * 64) blocks of 2*na doubles, or one per
  // work-queue batch of the FP32 forms (32 rows per batch, more when the
  // rows would need over 65536 records); the queue counter follows them
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const uint64_t kMaxBatches = 1ull << 16;
  const uint64_t per_lane = (L.rows + 32 * kMaxBatches - 1) / (32 * kMaxBatches);
  L.batch_rows = (uint32_t)(32 * (per_lane ? per_lane : 1));
  const size_t nbatch = (size_t)((L.rows + L.batch_rows - 1) / L.batch_rows);
  size_t nrec = (size_t)sms * 64 + 1;
  if (nbatch > nrec) nrec = nbatch;
  const size_t rec_bytes = (nrec * 2 * na * sizeof(double) + 255) & ~(size_t)255;
  if ((rc = ensure_buf(c, c->partials, rec_bytes + 256))) return rc;
  L.partials = (double*)c->partials.ptr;
  if (precision == STOCHA_FP32) L.work = (unsigned long long*)((char*)c->partials.ptr + rec_bytes);
  int nb = precision == STOCHA_FP32 ? launch_paths_f32(L, c->stream) : launch_paths_f64(L, c->stream);
  if (nb < 0) return cuda_error(cudaGetLastError(), "pricing kernel launch");
  launch_reduce_partials(L.partials, nb, 2 * na, sums_dev, c->stream);
  *nvals = 2 * na;
  return STOCHA_OK;
}

int terminal_launch(stocha_ctx* c, const stocha_model* m, uint64_t seed, double* out_dev) {
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(m, &L, &row_len, &block, false);
  if (rc) return rc;
  if (L.rows == 0) return STOCHA_OK;
  make_stream_spec((u128)seed, block, &L.ss);
  L.tabs = c->d_tabs;
  L.err = c->d_err;
  L.out_f64 = out_dev;
  L.terminal_only = 1;
  fill_f32_constants(&L);
  if (launch_paths_f64(L, c->stream) < 0) return cuda_error(cudaGetLastError(), "terminal-price launch");
  return STOCHA_OK;
}

}  // namespace stocha

using namespace stocha;

extern "C" {

int stocha_ctx_create(int device, stocha_ctx** out) { return create_ctx(device, out); }

void stocha_ctx_destroy(stocha_ctx* c) {
  if (!c) return;
  if (c == g_default) return;  // the default context lives until exit
  DeviceGuard g(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->out, &c->partials, &c->small, &c->aux, &c->starts})
    if (b->ptr) cudaFree(b->ptr);
  if (c->lsmc_graphs) lsmc_graphs_release(c->lsmc_graphs);
  if (c->d_tabs) cudaFree(c->d_tabs);
  if (c->d_err) cudaFree(c->d_err);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_small) cudaFreeHost(c->h_small);
  for (cudaEvent_t e : c->chunk_done)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

void* stocha_ctx_stream(stocha_ctx* c) {
  if (resolve_ctx(&c)) return nullptr;
  return (void*)c->stream;
}

int stocha_ctx_set_stream(stocha_ctx* c, void* s) {
  int rc = resolve_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->stream = s ? (cudaStream_t)s : c->own;
  return STOCHA_OK;
}

// Synchronises the context's stream and reports device-side check failures
// of earlier asynchronous calls.
int stocha_ctx_sync(stocha_ctx* c) {
  int rc = resolve_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  DeviceGuard g(c->device);
  return finish_call(c);
}

int stocha_measure_peak(stocha_ctx* ctx, int32_t kind, double* ops_per_s) {
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (kind < 0 || kind > 3) return set_error(STOCHA_ERR_VALUE, "kind must be 0..3");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  double v = measure_peak(kind, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  if (v <= 0) return set_error(STOCHA_ERR_NOMEM, "peak benchmark allocation failed");
  *ops_per_s = v;
  return STOCHA_OK;
}

static int tune_slot_of(int32_t model, int32_t n_assets) {
  const int kind = model == STOCHA_MODEL_GBM ? kGbm : model == STOCHA_MODEL_HESTON ? kHeston
                   : model == STOCHA_MODEL_MERTON ? kMerton : model == STOCHA_MODEL_MULTI_GBM ? kMultiGbm : -1;
  return kind < 0 ? -1 : tune_slot(kind, n_assets);
}

int stocha_tune_get(int32_t model, int32_t n_assets, stocha_tune_result* out) {
  const int slot = tune_slot_of(model, n_assets);
  if (slot < 0 || !out) return set_error(STOCHA_ERR_VALUE, "no fused FP32 kernel for this model");
  const FusedTune t = get_fused_tune(slot);
  std::memset(out, 0, sizeof *out);
  out->model = model;
  out->n_assets = n_assets;
  out->block = t.block;
  out->ilp = t.ilp;
  out->waves = t.waves;
  out->variant = t.variant;
  return STOCHA_OK;
}

int stocha_tune_set(int32_t model, int32_t n_assets, int32_t block, int32_t ilp, int32_t waves, int32_t variant) {
  const int slot = tune_slot_of(model, n_assets);
  if (slot < 0) return set_error(STOCHA_ERR_VALUE, "no fused FP32 kernel for this model");
  if (set_fused_tune(slot, FusedTune{block, ilp, waves, variant}))
    return set_error(STOCHA_ERR_VALUE,
                     "block must be 64, 128 or 256; waves 1 or 2; variant 0 or 2 (ilp 1) or 1 (ilp 1 or 2)");
  return STOCHA_OK;
}

int stocha_autotune(stocha_ctx* ctx, const stocha_model* m, int32_t reps, stocha_tune_result* out) {
  STOCHA_RANGE("stocha_autotune");
  if (!m || !out) return set_error(STOCHA_ERR_VALUE, "model and out must not be NULL");
  const int slot = tune_slot_of(m->kind, m->n_assets);
  if (slot < 0 || (m->kind == STOCHA_MODEL_HESTON && m->scheme != 0))
    return set_error(STOCHA_ERR_VALUE, "no fused FP32 kernel for this model");
  {
    PathLaunch probe;
    uint64_t row_len = 0;
    u128 block = 0;
    int rc = prepare_model(m, &probe, &row_len, &block);
    if (rc) return rc;
  }
  if (reps < 1) reps = 1;
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->small, 64 * sizeof(double)))) return rc;
  double* sums = (double*)ctx->small.ptr;
  cudaEvent_t e0, e1;
  STOCHA_CUDA(cudaEventCreate(&e0));
  STOCHA_CUDA(cudaEventCreate(&e1));
  const FusedTune before = get_fused_tune(slot);
  auto time_cfg = [&](FusedTune t, double* ms) -> int {
    set_fused_tune(slot, t);
    int nv = 0, r;
    if ((r = begin_call(ctx))) return r;
    if ((r = price_launch(ctx, m, 1, STOCHA_FP32, kCall, m->s0, nullptr, true, sums, &nv))) return r;  // warm-up
    STOCHA_CUDA(cudaEventRecord(e0, ctx->stream));
    for (int i = 0; i < reps; ++i)
      if ((r = price_launch(ctx, m, 1 + i, STOCHA_FP32, kCall, m->s0, nullptr, true, sums, &nv))) return r;
    STOCHA_CUDA(cudaEventRecord(e1, ctx->stream));
    if ((r = finish_call(ctx))) return r;
    float f = 0.0f;
    STOCHA_CUDA(cudaEventElapsedTime(&f, e0, e1));
    *ms = (double)f / reps;
    return STOCHA_OK;
  };
  FusedTune best = before;
  double best_ms = 1e300, default_ms = 0.0;
  int n = 0;
  rc = STOCHA_OK;
  const int forms[4][2] = {{0, 1}, {1, 1}, {1, 2}, {2, 1}};  // (variant, ilp)
  for (int b : {64, 128, 256})
    for (const auto& fm : forms)
      for (int waves : {1, 2}) {
        if (rc) break;
        double ms = 0.0;
        const FusedTune t{b, fm[1], waves, fm[0]};
        if ((rc = time_cfg(t, &ms))) break;
        ++n;
        if (b == 256 && fm[0] == 2 && fm[1] == 1 && waves == 2) default_ms = ms;  // the built-in default
        if (ms < best_ms) {
          best_ms = ms;
          best = t;
        }
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  set_fused_tune(slot, rc ? before : best);
  if (rc) return rc;
  std::memset(out, 0, sizeof *out);
  out->model = m->kind;
  out->n_assets = m->n_assets;
  out->block = best.block;
  out->ilp = best.ilp;
  out->waves = best.waves;
  out->variant = best.variant;
  out->candidates = n;
  out->ms_best = best_ms;
  out->ms_default = default_ms;
  return STOCHA_OK;
}

static int debug_f64(int fn, stocha_ctx* ctx, const double* x, double* y, uint64_t n) {
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (n == 0) return STOCHA_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->aux, 2 * n * sizeof(double)))) return rc;
  double* d = (double*)ctx->aux.ptr;
  if ((rc = begin_call(ctx))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(d, x, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  launch_debug_f64(fn, d, d + n, n, ctx->d_tabs, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  STOCHA_CUDA(cudaMemcpyAsync(y, d + n, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  return finish_call(ctx);
}

int stocha_debug_exp(stocha_ctx* ctx, const double* x, double* y, uint64_t n) { return debug_f64(0, ctx, x, y, n); }

int stocha_debug_sqrt(stocha_ctx* ctx, const double* x, double* y, uint64_t n) { return debug_f64(1, ctx, x, y, n); }

int stocha_debug_f64(stocha_ctx* ctx, int32_t fn, const double* x, double* y, uint64_t n) {
  if (fn < 0 || fn > 6) return set_error(STOCHA_ERR_VALUE, "fn must be 0..6");
  return debug_f64(fn, ctx, x, y, n);
}

int stocha_debug_fast_log_error(stocha_ctx* ctx, double* abs_err_half_to_one, double* rel_err_below_half) {
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->aux, 2 * sizeof(unsigned)))) return rc;
  unsigned* d = (unsigned*)ctx->aux.ptr;
  STOCHA_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned), ctx->stream));
  launch_debug_logf_scan(d, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  unsigned h[2];
  STOCHA_CUDA(cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  STOCHA_CUDA(cudaStreamSynchronize(ctx->stream));
  float a, r;
  std::memcpy(&a, &h[0], 4);
  std::memcpy(&r, &h[1], 4);
  if (abs_err_half_to_one) *abs_err_half_to_one = a;
  if (rel_err_below_half) *rel_err_below_half = r;
  return STOCHA_OK;
}

int stocha_debug_capped_draws(stocha_ctx* ctx, int32_t sampler, int32_t cap, uint64_t seed, uint64_t n,
                              double* out) {
  if (sampler < 0 || sampler > 4) return set_error(STOCHA_ERR_VALUE, "sampler must be 0..4");
  if (cap < 1) return set_error(STOCHA_ERR_VALUE, "cap must be positive");
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (n == 0) return STOCHA_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->aux, n * sizeof(double)))) return rc;
  DebugCapped a;
  std::memset(&a, 0, sizeof a);
  make_stream_spec((u128)seed, (u128)(1 + 1024) * 2, &a.ss);  // one-step GBM streams (gbm.rs:55)
  a.tabs = ctx->d_tabs;
  a.err = ctx->d_err;
  a.out = (double*)ctx->aux.ptr;
  a.n = n;
  a.sampler = sampler;
  a.cap = cap;
  // gamma of shape nu / 2 = 2.5 (nu = 5), Marsaglia-Tsang: d = shape - 1/3, c = 1 / sqrt(9 d)
  a.d = 2.5 - 1.0 / 3.0;
  a.c = 1.0 / std::sqrt(9.0 * a.d);
  if ((rc = begin_call(ctx))) return rc;
  launch_debug_capped(a, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  STOCHA_CUDA(cudaMemcpyAsync(out, a.out, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  return finish_call(ctx);
}

int stocha_debug_zigfeed(stocha_ctx* ctx, int32_t form, uint64_t seed, uint64_t n_paths, uint32_t n, float* out,
                         uint64_t* state) {
  if (form < 0 || form > 1) return set_error(STOCHA_ERR_VALUE, "form must be 0 or 1");
  if (!out || !state) return set_error(STOCHA_ERR_VALUE, "out and state must not be NULL");
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (n_paths == 0 || n == 0) return STOCHA_OK;
  if (n_paths > (1ull << 36) / n) return set_error(STOCHA_ERR_VALUE, "n_paths * n must be at most 2^36");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  const size_t vbytes = (size_t)n_paths * n * sizeof(float), sbytes = (size_t)n_paths * 2 * sizeof(uint64_t);
  if ((rc = ensure_buf(ctx, ctx->aux, vbytes + sbytes))) return rc;
  DebugZig a;
  std::memset(&a, 0, sizeof a);
  make_stream_spec((u128)seed, ((u128)n + 1024) * 2, &a.ss);  // GBM-style streams (gbm.rs:55)
  a.tabs = ctx->d_tabs;
  a.err = ctx->d_err;
  a.out = (float*)ctx->aux.ptr;
  a.state = (uint64_t*)((char*)ctx->aux.ptr + vbytes);
  a.n_paths = n_paths;
  a.n = n;
  a.form = form;
  if ((rc = begin_call(ctx))) return rc;
  launch_debug_zigfeed(a, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  STOCHA_CUDA(cudaMemcpyAsync(out, a.out, vbytes, cudaMemcpyDeviceToHost, ctx->stream));
  STOCHA_CUDA(cudaMemcpyAsync(state, a.state, sbytes, cudaMemcpyDeviceToHost, ctx->stream));
  return finish_call(ctx);
}

int stocha_debug_zig_thresholds(uint64_t* thr256) {
  ZigTables t;
  build_tables(&t);
  std::memcpy(thr256, t.thr, sizeof t.thr);
  return STOCHA_OK;
}

const char* stocha_last_error(void) { return g_err.c_str(); }
const char* stocha_version(void) { return "1.7.1"; }

int stocha_gbm(stocha_ctx* ctx, double s0, double mu, double sigma, double t, uint64_t steps, uint64_t n_paths,
               uint64_t seed, int32_t antithetic, double q, double* out) {
  STOCHA_RANGE("stocha_gbm");
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_GBM;
  m.s0 = s0;
  m.mu = mu;
  m.sigma = sigma;
  m.t = t;
  m.q = q;
  m.steps = steps;
  m.n_paths = n_paths;
  m.antithetic = antithetic;
  return paths_to_host(ctx, &m, seed, out);
}

int stocha_heston(stocha_ctx* ctx, double s0, double v0, double mu, double kappa, double theta, double xi,
                  double rho, double t, uint64_t steps, uint64_t n_paths, uint64_t seed, const char* scheme,
                  double* out) {
  STOCHA_RANGE("stocha_heston");
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_HESTON;
  m.s0 = s0;
  m.v0 = v0;
  m.mu = mu;
  m.kappa = kappa;
  m.theta = theta;
  m.xi = xi;
  m.rho = rho;
  m.t = t;
  m.steps = steps;
  m.n_paths = n_paths;
  m.scheme = !scheme ? 0 : std::strcmp(scheme, "euler") == 0 ? 0 : std::strcmp(scheme, "qe") == 0 ? 1 : -1;
  return paths_to_host(ctx, &m, seed, out);
}

int stocha_merton_jump_diffusion(stocha_ctx* ctx, double s0, double mu, double sigma, double lambda_, double mu_j,
                                 double sigma_j, double t, uint64_t steps, uint64_t n_paths, uint64_t seed,
                                 double* out) {
  STOCHA_RANGE("stocha_merton_jump_diffusion");
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_MERTON;
  m.s0 = s0;
  m.mu = mu;
  m.sigma = sigma;
  m.lambda_ = lambda_;
  m.mu_j = mu_j;
  m.sigma_j = sigma_j;
  m.t = t;
  m.steps = steps;
  m.n_paths = n_paths;
  return paths_to_host(ctx, &m, seed, out);
}

int stocha_hull_white(stocha_ctx* ctx, double r0, double a, double theta, double sigma, double t, uint64_t steps,
                      uint64_t n_paths, uint64_t seed, double* out) {
  STOCHA_RANGE("stocha_hull_white");
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_HULL_WHITE;
  m.s0 = r0;
  m.kappa = a;
  m.theta = theta;
  m.sigma = sigma;
  m.t = t;
  m.steps = steps;
  m.n_paths = n_paths;
  return paths_to_host(ctx, &m, seed, out);
}

int stocha_multi_gbm(stocha_ctx* ctx, size_t n_assets, const double* s0, const double* mu, const double* sigma,
                     const double* corr, size_t corr_rows, size_t corr_cols, double t, uint64_t steps,
                     uint64_t n_paths, uint64_t seed, int32_t antithetic, double* out) {
  STOCHA_RANGE("stocha_multi_gbm");
  // lib.rs:771-809: the length checks come first, the corr shape last.
  if (n_assets == 0) return set_error(STOCHA_ERR_VALUE, "s0 must not be empty");
  for (size_t i = 0; i < n_assets; ++i)
    if (s0[i] <= 0.0) return set_error(STOCHA_ERR_VALUE, "all s0 must be positive");
  for (size_t i = 0; i < n_assets; ++i)
    if (sigma[i] <= 0.0) return set_error(STOCHA_ERR_VALUE, "all sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  if (steps == 0 || n_paths == 0) return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
  if (corr_rows != n_assets || corr_cols != n_assets)
    return set_error(STOCHA_ERR_VALUE, "corr must be (" + std::to_string(n_assets) + ", " +
                                           std::to_string(n_assets) + "), got (" + std::to_string(corr_rows) +
                                           ", " + std::to_string(corr_cols) + ")");
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_MULTI_GBM;
  m.n_assets = (int32_t)n_assets;
  m.s0_v = s0;
  m.mu_v = mu;
  m.sigma_v = sigma;
  m.corr = corr;
  m.t = t;
  m.steps = steps;
  m.n_paths = n_paths;
  m.antithetic = antithetic;
  return paths_to_host(ctx, &m, seed, out);
}

int stocha_paths_device(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, void* out_dev) {
  STOCHA_RANGE("stocha_paths_device");
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  return paths_to_device(ctx, m, seed, precision, out_dev);
}

int stocha_price_device(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff,
                        double strike, double rate, double* out_dev) {
  STOCHA_RANGE("stocha_price_device");
  (void)rate;  // the device form returns raw sums; see stocha_price
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  int nvals = 0;
  if (payoff != STOCHA_PAYOFF_CALL && payoff != STOCHA_PAYOFF_PUT)
    return set_error(STOCHA_ERR_VALUE, "payoff must be call or put");
  return price_launch(ctx, m, seed, precision, payoff, strike, nullptr, true, out_dev, &nvals);
}

int stocha_price(stocha_ctx* ctx, const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff,
                 double strike, double rate, double* out) {
  STOCHA_RANGE("stocha_price");
  {
    PathLaunch probe;
    uint64_t row_len = 0;
    u128 block = 0;
    int vrc = prepare_model(m, &probe, &row_len, &block);
    if (vrc) return vrc;
  }
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  DeviceGuard g(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->small, 64 * sizeof(double)))) return rc;
  if ((rc = begin_call(ctx))) return rc;
  int nvals = 0;
  double* sums = (double*)ctx->small.ptr;
  if (payoff != STOCHA_PAYOFF_CALL && payoff != STOCHA_PAYOFF_PUT)
    return set_error(STOCHA_ERR_VALUE, "payoff must be call or put");
  if ((rc = price_launch(ctx, m, seed, precision, payoff, strike, nullptr, true, sums, &nvals))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, sums, nvals * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if ((rc = finish_call(ctx))) return rc;
  const double n = (double)m->n_paths;
  const double disc = std::exp(-rate * m->t);
  for (int a = 0; a < nvals / 2; ++a) {
    double sum = ctx->h_small[2 * a], sum2 = ctx->h_small[2 * a + 1];
    double mean = sum / n;
    double var = n > 1 ? (sum2 - sum * mean) / (n - 1) : 0.0;
    if (var < 0) var = 0;
    out[2 * a] = disc * sum / n;  // greeks.rs:319 order: discount * sum / n
    out[2 * a + 1] = disc * std::sqrt(var / n);
  }
  return STOCHA_OK;
}

// ------------------------------------------------------------------ RNG --
int stocha_rng_new(uint64_t seed_lo, uint64_t seed_hi, const char* algorithm, stocha_rng* out) {
  // lib.rs:87-101
  if (algorithm && std::strcmp(algorithm, "pcg64dxsm") != 0 && std::strcmp(algorithm, "default") != 0)
    return set_error(STOCHA_ERR_VALUE,
                     std::string("Unknown algorithm: '") + algorithm + "'. Supported: 'pcg64dxsm'");
  u128 seed = ((u128)seed_hi << 64) | seed_lo, st, inc;
  pcg_seed(seed, &st, &inc);
  out->state_lo = (uint64_t)st;
  out->state_hi = (uint64_t)(st >> 64);
  out->inc_lo = (uint64_t)inc;
  out->inc_hi = (uint64_t)(inc >> 64);
  out->seed_lo = seed_lo;
  out->seed_hi = seed_hi;
  return STOCHA_OK;
}

// JSON of pcg64.rs:10-15,58-65 with serde's field names of rand_pcg's
// Lcg128CmDxsm64 ({"state","increment"}) and u128 numbers.
int stocha_rng_save_state(const stocha_rng* r, char* buf, size_t cap, size_t* len) {
  u128 st = ((u128)r->state_hi << 64) | r->state_lo;
  u128 inc = ((u128)r->inc_hi << 64) | r->inc_lo;
  u128 seed = ((u128)r->seed_hi << 64) | r->seed_lo;
  std::string j = "{\"version\":2,\"rng\":{\"state\":" + u128_str(st) + ",\"increment\":" + u128_str(inc) +
                  "},\"seed\":" + u128_str(seed) + "}";
  if (len) *len = j.size();
  if (!buf || cap < j.size() + 1) return set_error(STOCHA_ERR_VALUE, "buffer too small");
  std::memcpy(buf, j.c_str(), j.size() + 1);
  return STOCHA_OK;
}

}  // extern "C"
