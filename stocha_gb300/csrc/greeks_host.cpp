// Host side of the Monte Carlo Greeks (src/lib.rs:920-1242,
// src/finance/greeks.rs): argument parsing with the reference's messages,
// scenario planning (required_scenarios, compute_bump), the FP64
// scenario-by-scenario revaluation, the pathwise estimators, and the
// batched FP32 common-random-number launch (greeks.cu).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "greeks_kernels.h"
#include "host_common.h"

using namespace stocha;

namespace {

enum Greek { G_DELTA = 0, G_GAMMA, G_VEGA, G_THETA, G_RHO };
enum Bump { B_S0 = 0, B_SIGMA, B_T, B_MU };  // greeks.rs:26-31

const char* kGreekNames[5] = {"delta", "gamma", "vega", "theta", "rho"};

int parse_greeks(const char* const* names, uint64_t n, std::vector<int>* out) {  // lib.rs:920-938
  for (uint64_t i = 0; i < n; ++i) {
    int g = -1;
    for (int j = 0; j < 5; ++j)
      if (names[i] && std::strcmp(names[i], kGreekNames[j]) == 0) g = j;
    if (g < 0)
      return set_error(STOCHA_ERR_VALUE, std::string("Unknown greek: '") + (names[i] ? names[i] : "") +
                                             "'. Supported: delta, gamma, vega, theta, rho");
    out->push_back(g);
  }
  return STOCHA_OK;
}

// ModelSpec (greeks.rs:55-88) as a stocha_model; lib.rs:958-1040 order of
// required keys.
int build_spec(const char* model, const stocha_greeks_params* p, uint64_t n_paths, uint64_t n_steps,
               stocha_model* m) {
  std::memset(m, 0, sizeof *m);
  const char* keys[12] = {"s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j"};
  auto need = [&](std::initializer_list<int> idx) -> int {
    for (int i : idx)
      if (!(p->present & (1u << i)))
        return set_error(STOCHA_ERR_VALUE, std::string("Missing required param: '") + keys[i] + "'");
    return STOCHA_OK;
  };
  const std::string name = model ? model : "";
  m->steps = n_steps;
  m->n_paths = n_paths;
  m->s0 = p->s0;
  m->mu = p->r;
  m->t = p->t;
  if (name == "gbm") {
    if (int rc = need({0, 1, 2, 3})) return rc;
    m->kind = STOCHA_MODEL_GBM;
    m->sigma = p->sigma;
    return STOCHA_OK;
  }
  if (name == "heston") {
    if (int rc = need({0, 4, 1, 5, 6, 7, 8, 3})) return rc;
    if (p->scheme != 0 && p->scheme != 1) return set_error(STOCHA_ERR_VALUE, "scheme must be 'euler' or 'qe'");
    m->kind = STOCHA_MODEL_HESTON;
    m->v0 = p->v0;
    m->kappa = p->kappa;
    m->theta = p->theta;
    m->xi = p->xi;
    m->rho = p->rho;
    m->scheme = p->scheme;
    return STOCHA_OK;
  }
  if (name == "merton") {
    if (int rc = need({0, 1, 2, 9, 10, 11, 3})) return rc;
    m->kind = STOCHA_MODEL_MERTON;
    m->sigma = p->sigma;
    m->lambda_ = p->lambda_;
    m->mu_j = p->mu_j;
    m->sigma_j = p->sigma_j;
    return STOCHA_OK;
  }
  return set_error(STOCHA_ERR_VALUE, "Unknown model: '" + name + "'. Supported: gbm, heston, merton");
}

double* bump_field(stocha_model* m, int b) {  // greeks.rs:169-188, 206-225
  switch (b) {
    case B_S0: return &m->s0;
    case B_SIGMA: return m->kind == STOCHA_MODEL_HESTON ? &m->v0 : &m->sigma;
    case B_T: return &m->t;
    default: return &m->mu;
  }
}

double compute_bump(double v, double bump_size) { return std::fmax(std::fabs(v) * bump_size, 1e-8); }  // greeks.rs:227-229

// Scenario key: -1 base, else bump*2 + (down ? 1 : 0).  Order of first use as
// required_scenarios (greeks.rs:231-265) lists them.
void required_scenarios(const std::vector<int>& greeks, std::vector<int>* sc) {
  auto add = [&](int k) {
    for (int x : *sc)
      if (x == k) return;
    sc->push_back(k);
  };
  for (int g : greeks) {
    switch (g) {
      case G_DELTA: add(B_S0 * 2); add(B_S0 * 2 + 1); break;
      case G_GAMMA: add(B_S0 * 2); add(-1); add(B_S0 * 2 + 1); break;
      case G_VEGA: add(B_SIGMA * 2); add(B_SIGMA * 2 + 1); break;
      case G_THETA: add(B_T * 2 + 1); add(-1); break;
      default: add(B_MU * 2); add(B_MU * 2 + 1); break;
    }
  }
}

// greeks.rs:267-311
void greeks_from_prices(const std::vector<int>& greeks, const double* price /* [9] by key+1 */, const double* h,
                        double* out) {
  auto P = [&](int key) { return price[key + 1]; };
  for (size_t i = 0; i < greeks.size(); ++i) {
    switch (greeks[i]) {
      case G_DELTA: out[i] = (P(B_S0 * 2) - P(B_S0 * 2 + 1)) / (2.0 * h[B_S0]); break;
      case G_GAMMA: out[i] = (P(B_S0 * 2) - 2.0 * P(-1) + P(B_S0 * 2 + 1)) / (h[B_S0] * h[B_S0]); break;
      case G_VEGA: out[i] = (P(B_SIGMA * 2) - P(B_SIGMA * 2 + 1)) / (2.0 * h[B_SIGMA]); break;
      case G_THETA: out[i] = (P(B_T * 2 + 1) - P(-1)) / h[B_T]; break;
      default: out[i] = (P(B_MU * 2) - P(B_MU * 2 + 1)) / (2.0 * h[B_MU]); break;
    }
  }
}

// FP64 revaluation of every scenario (greeks.rs:322-358; lib.rs:1106-1150
// for a callable payoff).
int greeks_fp64(stocha_ctx* ctx, const stocha_model& base, int payoff, stocha_payoff_fn cb, void* user,
                double strike, const std::vector<int>& greeks, uint64_t seed, double bump_size, double* out) {
  std::vector<int> sc;
  required_scenarios(greeks, &sc);
  double h[4];
  for (int b = 0; b < 4; ++b) {
    stocha_model tmp = base;
    h[b] = compute_bump(*bump_field(&tmp, b), bump_size);
  }
  double price[9] = {0};
  int rc;
  if (!cb) {
    if ((rc = ensure_buf(ctx, ctx->small, 64 * sizeof(double)))) return rc;
    double* sums = (double*)ctx->small.ptr;
    if ((rc = begin_call(ctx))) return rc;
    for (size_t s = 0; s < sc.size(); ++s) {
      stocha_model m = base;
      if (sc[s] >= 0) *bump_field(&m, sc[s] / 2) += (sc[s] & 1) ? -h[sc[s] / 2] : h[sc[s] / 2];
      int nv = 0;
      if ((rc = price_launch(ctx, &m, seed, STOCHA_FP64, payoff, strike, nullptr, false, sums + 2 * s, &nv))) return rc;
    }
    STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, sums, 2 * sc.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
    if ((rc = finish_call(ctx))) return rc;
    for (size_t s = 0; s < sc.size(); ++s) {
      stocha_model m = base;
      if (sc[s] >= 0) *bump_field(&m, sc[s] / 2) += (sc[s] & 1) ? -h[sc[s] / 2] : h[sc[s] / 2];
      const double discount = std::exp(-m.mu * m.t);  // greeks.rs:316-319
      price[sc[s] + 1] = discount * ctx->h_small[2 * s] / (double)base.n_paths;
    }
  } else {
    const uint64_t n = base.n_paths;
    if ((rc = ensure_buf(ctx, ctx->aux, (n ? n : 1) * sizeof(double)))) return rc;
    std::vector<double> term(n);
    for (size_t s = 0; s < sc.size(); ++s) {
      stocha_model m = base;
      if (sc[s] >= 0) *bump_field(&m, sc[s] / 2) += (sc[s] & 1) ? -h[sc[s] / 2] : h[sc[s] / 2];
      if ((rc = begin_call(ctx))) return rc;
      if ((rc = terminal_launch(ctx, &m, seed, (double*)ctx->aux.ptr))) return rc;
      if (n) STOCHA_CUDA(cudaMemcpyAsync(term.data(), ctx->aux.ptr, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
      if ((rc = finish_call(ctx))) return rc;
      double sum = 0.0;
      uint64_t len = 0;
      if (cb(user, term.data(), n, &sum, &len) != 0) return set_error(STOCHA_ERR_CALLBACK, "payoff callback failed");
      const double discount = std::exp(-m.mu * m.t);
      price[sc[s] + 1] = discount * sum / (double)len;  // lib.rs:1143-1144
    }
  }
  greeks_from_prices(greeks, price, h, out);
  return STOCHA_OK;
}

}  // namespace

namespace stocha {

// Fills one device instance of the FP32 batch kernel (price_only: the price
// and its standard error only).
void greeks_make_inst(const stocha_model& m, int payoff, double strike, double bump_size, uint64_t seed,
                      bool price_only, GInst* I) {
  std::memset(I, 0, sizeof *I);
  I->price_only = price_only ? 1 : 0;
  I->model = m.kind == STOCHA_MODEL_GBM ? kGbm : m.kind == STOCHA_MODEL_HESTON ? kHeston : kMerton;
  I->payoff = payoff;
  I->steps = m.steps;
  I->n_paths = m.n_paths;
  const double steps = (double)m.steps;
  const double hs = compute_bump(m.s0, bump_size);
  const double hv = compute_bump(m.kind == STOCHA_MODEL_HESTON ? m.v0 : m.sigma, bump_size);
  const double ht = compute_bump(m.t, bump_size);
  const double hr = compute_bump(m.mu, bump_size);
  I->K = (float)strike;
  I->s0 = (float)m.s0;
  I->u = (float)(hs / m.s0);
  I->erp = (float)std::exp(hr * m.t);
  I->erm = (float)std::exp(-hr * m.t);
  I->sh2 = (float)(2.0 * std::sinh(hr * m.t));
  const u128 mult = m.kind == STOCHA_MODEL_GBM ? 2 : m.kind == STOCHA_MODEL_HESTON ? 6 : 8;
  make_stream_spec((u128)seed, ((u128)m.steps + 1024) * mult, &I->ss);  // gbm.rs:55, heston.rs:48, jump_diffusion.rs:64
  // trajectories: base, sigma+h, sigma-h, T-h
  const double sig[4] = {m.sigma, m.sigma + hv, m.sigma - hv, m.sigma};
  const double tt[4] = {m.t, m.t, m.t, m.t - ht};
  if (m.kind == STOCHA_MODEL_HESTON) {
    const double v0[4] = {m.v0, m.v0 + hv, m.v0 - hv, m.v0};
    for (int k = 0; k < 4; ++k) {
      const double dt = tt[k] / steps;
      I->hv0[k] = (float)v0[k];
      I->hkdt[k] = (float)(m.kappa * dt);
      I->hxsdt[k] = (float)(m.xi * std::sqrt(dt));
      I->hnhdt[k] = (float)(-0.5 * dt);
      I->hmudt[k] = (float)(m.mu * dt);
      I->hsdt[k] = (float)std::sqrt(dt);
    }
    I->hrho = (float)m.rho;
    I->hrho_comp = (float)std::sqrt(1.0 - m.rho * m.rho);
    I->htheta = (float)m.theta;
    return;
  }
  const double m_bar = m.kind == STOCHA_MODEL_MERTON ? std::exp(m.mu_j + 0.5 * m.sigma_j * m.sigma_j) - 1.0 : 0.0;
  const double lam = m.kind == STOCHA_MODEL_MERTON ? m.lambda_ : 0.0;
  for (int k = 0; k < 4; ++k) {
    const double dt = tt[k] / steps;
    const double drift = (m.mu - 0.5 * sig[k] * sig[k] - lam * m_bar) * dt;
    I->kdrift[k] = (float)(steps * drift);
    I->diff[k] = (float)(sig[k] * std::sqrt(dt));
  }
  if (m.kind == STOCHA_MODEL_MERTON) {
    I->mu_j = (float)m.mu_j;
    I->sigma_j = (float)m.sigma_j;
    I->jthr[0] = unit_threshold(lam * (tt[0] / steps));
    I->jthr[1] = unit_threshold(lam * (tt[3] / steps));
    I->theta_pass = 1;
  }
}

// Greeks of one instance from its FP64 totals of the FP32 per-path sums.
void greeks_from_sums(const stocha_model& m, double bump_size, const double* S, double* price, double* se,
                      double* g /* delta gamma vega theta rho */) {
  const double n = (double)m.n_paths;
  const double hs = compute_bump(m.s0, bump_size);
  const double hv = compute_bump(m.kind == STOCHA_MODEL_HESTON ? m.v0 : m.sigma, bump_size);
  const double ht = compute_bump(m.t, bump_size);
  const double hr = compute_bump(m.mu, bump_size);
  const double disc = std::exp(-m.mu * m.t);
  const double p0 = S[0] / n;
  *price = disc * p0;
  const double var = n > 1 ? std::fmax(S[1] - S[0] * p0, 0.0) / (n - 1.0) : 0.0;
  *se = disc * std::sqrt(var / n);
  g[0] = disc * (S[2] / n) / (2.0 * hs);
  g[1] = disc * (S[3] / n) / (hs * hs);
  g[2] = disc * (S[4] / n) / (2.0 * hv);
  // theta: (e^{-r(T-h)} E[P_T] - e^{-rT} E[P]) / h
  g[3] = disc * (S[5] / n + std::expm1(m.mu * ht) * (S[6] / n)) / ht;
  // rho: (e^{-(r+h)T} E[P+] - e^{-(r-h)T} E[P-]) / (2h), P+ = P- + D
  g[4] = disc * (std::exp(-hr * m.t) * (S[7] / n) - 2.0 * std::sinh(hr * m.t) * (S[8] / n)) / (2.0 * hr);
}

// The model of one batch instance (its r is the drift, greeks.rs:190-200).
stocha_model greeks_model_of(const stocha_greeks_instance& x) {
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = x.model;
  m.scheme = x.scheme;
  m.s0 = x.s0;
  m.mu = x.r;
  m.sigma = x.sigma;
  m.t = x.t;
  m.v0 = x.v0;
  m.kappa = x.kappa;
  m.theta = x.theta;
  m.xi = x.xi;
  m.rho = x.rho;
  m.lambda_ = x.lambda_;
  m.mu_j = x.mu_j;
  m.sigma_j = x.sigma_j;
  m.steps = x.steps;
  m.n_paths = x.n_paths;
  return m;
}

}  // namespace stocha

namespace {

int batch_fp32(stocha_ctx* ctx, const std::vector<stocha_model>& models, const std::vector<int>& payoffs,
               const std::vector<double>& strikes, const std::vector<double>& bumps,
               const std::vector<uint64_t>& seeds, std::vector<double>* sums) {
  const uint64_t n = models.size();
  const uint64_t chunk = 1024;
  std::vector<GInst> inst(n);
  std::vector<uint32_t> item_inst;
  uint64_t items = 0;
  for (uint64_t i = 0; i < n; ++i) {
    greeks_make_inst(models[i], payoffs[i], strikes[i], bumps[i], seeds[i], false, &inst[i]);
    inst[i].chunk = chunk;
    inst[i].item_begin = items;
    const uint64_t k = (models[i].n_paths + chunk - 1) / chunk;
    for (uint64_t j = 0; j < k; ++j) item_inst.push_back((uint32_t)i);
    items += k;
  }
  const size_t off_items = ((n * sizeof(GInst)) + 255) & ~(size_t)255;
  const size_t off_part = off_items + ((items * 4 + 255) & ~(size_t)255);
  const size_t off_sums = off_part + items * kGreekAcc * 8;
  const size_t off_ctr = off_sums + n * kGreekAcc * 8;
  int rc;
  if ((rc = ensure_buf(ctx, ctx->aux, off_ctr + 64))) return rc;
  char* base = (char*)ctx->aux.ptr;
  GreeksLaunch g;
  g.inst = (const GInst*)base;
  g.item_inst = (const uint32_t*)(base + off_items);
  g.total_items = items;
  g.counter = (unsigned long long*)(base + off_ctr);
  g.item_part = (double*)(base + off_part);
  g.inst_sums = (double*)(base + off_sums);
  g.n_inst = (int)n;
  g.tabs = ctx->d_tabs;
  g.direct = 0;
  g.err = ctx->d_err;
  if ((rc = begin_call(ctx))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(base, inst.data(), n * sizeof(GInst), cudaMemcpyHostToDevice, ctx->stream));
  if (items)
    STOCHA_CUDA(cudaMemcpyAsync(base + off_items, item_inst.data(), items * 4, cudaMemcpyHostToDevice, ctx->stream));
  launch_greeks_batch(g, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  sums->assign(n * kGreekAcc, 0.0);
  STOCHA_CUDA(cudaMemcpyAsync(sums->data(), g.inst_sums, n * kGreekAcc * 8, cudaMemcpyDeviceToHost, ctx->stream));
  // the host vectors above must outlive the asynchronous copies
  return finish_call(ctx);
}

}  // namespace

extern "C" {

int stocha_greeks_fd(stocha_ctx* ctx, const char* model, const stocha_greeks_params* params, const char* payoff,
                     stocha_payoff_fn payoff_cb, void* user, double strike, uint64_t n_paths, uint64_t n_steps,
                     const char* const* greeks, uint64_t n_greeks, uint64_t seed, double bump_size,
                     int32_t precision, double* out) {
  STOCHA_RANGE("stocha_greeks_fd");
  std::vector<int> gl;
  int rc = parse_greeks(greeks, n_greeks, &gl);  // lib.rs:1077
  if (rc) return rc;
  stocha_model m;
  if ((rc = build_spec(model, params, n_paths, n_steps, &m))) return rc;  // lib.rs:1078
  int pay = -1;
  if (payoff) {  // lib.rs:1080-1090
    if (std::strcmp(payoff, "call") == 0)
      pay = kCall;
    else if (std::strcmp(payoff, "put") == 0)
      pay = kPut;
    else
      return set_error(STOCHA_ERR_VALUE,
                       std::string("Unknown payoff: '") + payoff + "'. Supported: 'call', 'put', or a callable");
  } else if (!payoff_cb) {
    return set_error(STOCHA_ERR_VALUE, "payoff must be 'call', 'put', or a callable");
  }
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const bool fp32 = precision == STOCHA_FP32 && pay >= 0 && !(m.kind == STOCHA_MODEL_HESTON && m.scheme == 1);
  if (!fp32) return greeks_fp64(ctx, m, pay, payoff ? nullptr : payoff_cb, user, strike, gl, seed, bump_size, out);
  std::vector<double> sums;
  if ((rc = batch_fp32(ctx, {m}, {pay}, {strike}, {bump_size}, {seed}, &sums))) return rc;
  double price, se, g[5];
  greeks_from_sums(m, bump_size, sums.data(), &price, &se, g);
  for (size_t i = 0; i < gl.size(); ++i) out[i] = g[gl[i]];
  return STOCHA_OK;
}

int stocha_greeks_pathwise(stocha_ctx* ctx, double s0, double r, double sigma, double t, double strike,
                           int32_t is_call, uint64_t n_paths, uint64_t n_steps, const char* const* greeks,
                           uint64_t n_greeks, uint64_t seed, double* out) {
  STOCHA_RANGE("stocha_greeks_pathwise");
  // lib.rs:1191-1224
  if (s0 <= 0.0) return set_error(STOCHA_ERR_VALUE, "s0 must be positive");
  if (sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  if (n_paths == 0 || n_steps == 0) return set_error(STOCHA_ERR_VALUE, "n_paths and n_steps must be positive");
  std::vector<int> gl;
  int rc = parse_greeks(greeks, n_greeks, &gl);
  if (rc) return rc;
  for (int g : gl)
    if (g != G_DELTA && g != G_VEGA)
      return set_error(STOCHA_ERR_VALUE, std::string("Pathwise method only supports 'delta' and 'vega', got '") +
                                             kGreekNames[g] + "'");
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  stocha_model m;
  std::memset(&m, 0, sizeof m);
  m.kind = STOCHA_MODEL_GBM;
  m.s0 = s0;
  m.mu = r;
  m.sigma = sigma;
  m.t = t;
  m.steps = n_steps;
  m.n_paths = n_paths;
  const double aux[4] = {s0, r, sigma, t};
  if ((rc = ensure_buf(ctx, ctx->small, 64 * sizeof(double)))) return rc;
  double* sums = (double*)ctx->small.ptr;
  if ((rc = begin_call(ctx))) return rc;
  for (size_t i = 0; i < gl.size() && i < 16; ++i) {
    const int kind = gl[i] == G_DELTA ? (is_call ? kPwDeltaCall : kPwDeltaPut) : (is_call ? kPwVegaCall : kPwVegaPut);
    int nv = 0;
    if ((rc = price_launch(ctx, &m, seed, STOCHA_FP64, kind, strike, aux, true, sums + 2 * i, &nv))) return rc;
  }
  const size_t ng = gl.size() < 16 ? gl.size() : 16;
  STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, sums, 2 * ng * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if ((rc = finish_call(ctx))) return rc;
  const double discount = std::exp(-r * t);
  for (size_t i = 0; i < gl.size(); ++i) out[i] = discount * ctx->h_small[2 * (i < 16 ? i : 15)] / (double)n_paths;
  return STOCHA_OK;
}

int stocha_greeks_batch(stocha_ctx* ctx, const stocha_greeks_instance* inst, uint64_t n, int32_t precision,
                        double* out) {
  STOCHA_RANGE("stocha_greeks_batch");
  for (uint64_t i = 0; i < n; ++i) {
    const stocha_greeks_instance& x = inst[i];
    if (x.model != STOCHA_MODEL_GBM && x.model != STOCHA_MODEL_HESTON && x.model != STOCHA_MODEL_MERTON)
      return set_error(STOCHA_ERR_VALUE, "instance " + std::to_string(i) + ": unknown model");
    if (x.payoff != STOCHA_PAYOFF_CALL && x.payoff != STOCHA_PAYOFF_PUT)
      return set_error(STOCHA_ERR_VALUE, "instance " + std::to_string(i) + ": payoff must be call or put");
    if (x.n_paths == 0 || x.steps == 0)
      return set_error(STOCHA_ERR_VALUE, "instance " + std::to_string(i) + ": steps and n_paths must be positive");
    // the FP32 batch kernel counts a path's normals in 32 bits
    if (precision == STOCHA_FP32 && x.steps >= (1ull << 32))
      return set_error(STOCHA_ERR_VALUE, "instance " + std::to_string(i) + ": steps must be below 2^32 in fp32");
  }
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  std::vector<stocha_model> models;
  std::vector<int> pays;
  std::vector<double> strikes, bumps;
  std::vector<uint64_t> seeds, idx;
  const std::vector<int> all = {G_DELTA, G_GAMMA, G_VEGA, G_THETA, G_RHO};
  for (uint64_t i = 0; i < n; ++i) {
    const stocha_model m = greeks_model_of(inst[i]);
    const bool qe = m.kind == STOCHA_MODEL_HESTON && m.scheme == 1;
    if (precision == STOCHA_FP32 && !qe) {
      models.push_back(m);
      pays.push_back(inst[i].payoff);
      strikes.push_back(inst[i].strike);
      bumps.push_back(inst[i].bump_size);
      seeds.push_back(inst[i].seed);
      idx.push_back(i);
      continue;
    }
    // FP64 (or Heston QE): the reference's scenario revaluation
    double g[5];
    if ((rc = greeks_fp64(ctx, m, inst[i].payoff, nullptr, nullptr, inst[i].strike, all, inst[i].seed,
                          inst[i].bump_size, g)))
      return rc;
    int nv = 0;
    if ((rc = ensure_buf(ctx, ctx->small, 64 * sizeof(double)))) return rc;
    if ((rc = begin_call(ctx))) return rc;
    if ((rc = price_launch(ctx, &m, inst[i].seed, STOCHA_FP64, inst[i].payoff, inst[i].strike, nullptr, false,
                           (double*)ctx->small.ptr, &nv)))
      return rc;
    STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, ctx->small.ptr, 16, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = finish_call(ctx))) return rc;
    const double nn = (double)m.n_paths, disc = std::exp(-m.mu * m.t);
    const double s1 = ctx->h_small[0], s2 = ctx->h_small[1], mean = s1 / nn;
    const double var = nn > 1 ? std::fmax(s2 - s1 * mean, 0.0) / (nn - 1.0) : 0.0;
    out[7 * i] = disc * s1 / nn;
    out[7 * i + 1] = disc * std::sqrt(var / nn);
    for (int j = 0; j < 5; ++j) out[7 * i + 2 + j] = g[j];
  }
  if (!models.empty()) {
    std::vector<double> sums;
    if ((rc = batch_fp32(ctx, models, pays, strikes, bumps, seeds, &sums))) return rc;
    for (size_t k = 0; k < models.size(); ++k) {
      double price, se, g[5];
      greeks_from_sums(models[k], bumps[k], sums.data() + k * kGreekAcc, &price, &se, g);
      double* o = out + 7 * idx[k];
      o[0] = price;
      o[1] = se;
      for (int j = 0; j < 5; ++j) o[2 + j] = g[j];
    }
  }
  return STOCHA_OK;
}

}  // extern "C"
