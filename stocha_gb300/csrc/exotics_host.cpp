// Host side of the exotic options (src/lib.rs:1549-1870 barrier_price,
// asian_price, lookback_price): argument checks with the reference's
// messages, the method dispatch ("auto" / "analytical" / "mc"), the closed
// forms, and the Monte Carlo drivers of exotics.cu.
//
// The closed forms restate the published formulas the reference implements:
//   * normal CDF by the Abramowitz-Stegun 7.1.26 erf approximation
//     (|error| < 1.5e-7), as the reference's bs.rs:3-25 uses, so that the
//     analytical prices equal the reference's;
//   * Reiner-Rubinstein (1991) barrier prices with Haug's A-D terms, the
//     Broadie-Glasserman-Kou (1997) continuity correction and the rebate
//     values from first-passage probabilities (barrier.rs:48-268);
//   * Kemna-Vorst (1990) geometric-average Asian call/put with the seasoning
//     transformation (asian.rs:60-141);
//   * Goldman-Sosin-Gatto (1979) floating and Conze-Viswanathan (1991) fixed
//     strike lookbacks with running extremes (lookback.rs:38-156).
#include <cmath>
#include <cstring>
#include <string>

#include "exotics_kernels.h"
#include "host_common.h"

using namespace stocha;

namespace {

const double kSqrtHalf = 0.70710678118654752440;  // 1/sqrt(2)

double ncdf(double x) {  // bs.rs:3-25: A&S 7.1.26
  const double z = x * kSqrtHalf;
  const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741, a4 = -1.453152027, a5 = 1.061405429;
  const double p = 0.3275911;
  const double sign = z < 0.0 ? -1.0 : 1.0;
  const double az = std::fabs(z);
  const double t = 1.0 / (1.0 + p * az);
  const double y = 1.0 - (((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * std::exp(-az * az);
  return 0.5 * (1.0 + sign * y);
}

double npdf(double x) { return (1.0 / std::sqrt(2.0 * M_PI)) * std::exp(-0.5 * x * x); }

double bs_div(double s, double k, double r, double q, double t, double sigma, bool call) {  // bs.rs:31-41
  const double d1 = (std::log(s / k) + (r - q + 0.5 * sigma * sigma) * t) / (sigma * std::sqrt(t));
  const double d2 = d1 - sigma * std::sqrt(t);
  const double df = std::exp(-r * t), qf = std::exp(-q * t);
  return call ? s * qf * ncdf(d1) - k * df * ncdf(d2) : k * df * ncdf(-d2) - s * qf * ncdf(-d1);
}

// ---------------------------------------------------------------- barrier
struct Barrier {
  double s, k, r, q, sigma, t, h;
  int up;      // direction
  int in;      // knock-in
  int call;
  int n_mon;   // <= 0: continuous
  double rebate;
  int at_hit;
  int f32 = 0;  // Monte Carlo in the FP32 form
};

double hit_probability(double s, double h, double r, double q, double sigma, double t, bool up) {  // barrier.rs:48-66
  const double nu = r - q - 0.5 * sigma * sigma;
  const double mu = nu / (sigma * sigma);
  const double st = std::sqrt(t);
  double h1, h2;
  if (up) {
    const double a = std::log(s / h);
    h1 = (a + nu * t) / (sigma * st);
    h2 = (a - nu * t) / (sigma * st);
  } else {
    const double a = std::log(h / s);
    h1 = (a - nu * t) / (sigma * st);
    h2 = (a + nu * t) / (sigma * st);
  }
  const double p = ncdf(h1) + std::pow(h / s, 2.0 * mu) * ncdf(h2);
  return std::fmin(std::fmax(p, 0.0), 1.0);
}

double rebate_at_hit_value(double s, double h, double rebate, double r, double q, double sigma, double t,
                           bool up) {  // barrier.rs:68-89: first-passage value of R paid at the hit
  if (rebate == 0.0) return 0.0;
  const double nu = r - q - 0.5 * sigma * sigma, s2 = sigma * sigma;
  const double mu = nu / s2;
  const double lambda = std::sqrt(mu * mu + 2.0 * r / s2);
  const double st = std::sqrt(t);
  const double lr = up ? std::log(h / s) : std::log(s / h);
  const double d1 = (-lr + lambda * s2 * t) / (sigma * st);
  const double d2 = (-lr - lambda * s2 * t) / (sigma * st);
  const double ratio = h / s;
  return rebate * (std::pow(ratio, mu - lambda) * ncdf(d1) + std::pow(ratio, mu + lambda) * ncdf(d2));
}

double rebate_value(const Barrier& p) {  // barrier.rs:91-125
  if (p.rebate == 0.0) return 0.0;
  const bool hit0 = p.up ? p.s >= p.h : p.s <= p.h;
  if (!p.in && p.at_hit) return hit0 ? p.rebate : rebate_at_hit_value(p.s, p.h, p.rebate, p.r, p.q, p.sigma, p.t, p.up);
  if (!p.in) {
    const double prob = hit0 ? 1.0 : hit_probability(p.s, p.h, p.r, p.q, p.sigma, p.t, p.up);
    return p.rebate * std::exp(-p.r * p.t) * prob;
  }
  if (hit0) return 0.0;
  const double prob = hit_probability(p.s, p.h, p.r, p.q, p.sigma, p.t, p.up);
  return p.rebate * std::exp(-p.r * p.t) * (1.0 - prob);
}

const double kBgkBeta = 0.5825971579390106;  // -zeta(1/2) / sqrt(2 pi), Broadie-Glasserman-Kou

// barrier.rs:143-268; false when no closed form applies (t or sigma <= 0)
bool barrier_analytical(const Barrier& p, double* out) {
  double h = p.h;
  if (p.n_mon > 0) {  // barrier.rs:131-141: discrete monitoring, barrier shifted outward
    const double shift = kBgkBeta * p.sigma * std::sqrt(p.t / (double)p.n_mon);
    h = p.up ? h * std::exp(shift) : h * std::exp(-shift);
  }
  const double s = p.s, k = p.k, r = p.r, q = p.q, sigma = p.sigma, t = p.t;
  if (t <= 0.0 || sigma <= 0.0) return false;
  if (p.up ? s >= h : s <= h) {  // knocked already: out -> 0, in -> vanilla (barrier.rs:270-284)
    *out = (p.in ? bs_div(s, k, r, q, t, sigma, p.call) : 0.0) + rebate_value(p);
    return true;
  }
  const double st = std::sqrt(t);
  const double mu = (r - q - 0.5 * sigma * sigma) / (sigma * sigma);
  const double eq = std::exp(-q * t), er = std::exp(-r * t);
  auto d = [&](double x, double y) { return (std::log(x) + y * sigma * sigma * t) / (sigma * st); };
  auto A = [&](double phi) {
    const double d1 = d(s / k, 1.0 + mu), d2 = d1 - sigma * st;
    return phi * (s * eq * ncdf(phi * d1) - k * er * ncdf(phi * d2));
  };
  auto B = [&](double phi) {
    const double d1 = d(s / h, 1.0 + mu), d2 = d1 - sigma * st;
    return phi * (s * eq * ncdf(phi * d1) - k * er * ncdf(phi * d2));
  };
  auto C = [&](double phi, double eta) {
    const double pw = std::pow(h / s, 2.0 * (1.0 + mu));
    const double d1 = d(h * h / (s * k), 1.0 + mu), d2 = d1 - sigma * st;
    return phi * (s * eq * pw * ncdf(eta * d1) - k * er * std::pow(h / s, 2.0 * mu) * ncdf(eta * d2));
  };
  auto D = [&](double phi, double eta) {
    const double pw = std::pow(h / s, 2.0 * (1.0 + mu));
    const double d1 = d(h / s, 1.0 + mu), d2 = d1 - sigma * st;
    return phi * (s * eq * pw * ncdf(eta * d1) - k * er * std::pow(h / s, 2.0 * mu) * ncdf(eta * d2));
  };
  double price;
  if (!p.up && !p.in && p.call) price = h <= k ? A(1) - C(1, 1) : B(1) - D(1, 1);
  else if (!p.up && p.in && p.call) price = h <= k ? C(1, 1) : A(1) - B(1) + D(1, 1);
  else if (p.up && !p.in && p.call) price = h > k ? A(1) - B(1) + C(1, -1) - D(1, -1) : 0.0;
  else if (p.up && p.in && p.call) price = h > k ? B(1) - C(1, -1) + D(1, -1) : A(1);
  else if (!p.up && !p.in && !p.call) price = h < k ? A(-1) - B(-1) + C(-1, 1) - D(-1, 1) : 0.0;
  else if (!p.up && p.in && !p.call) price = h < k ? B(-1) - C(-1, 1) + D(-1, 1) : A(-1);
  else if (p.up && !p.in && !p.call) price = h >= k ? A(-1) - C(-1, -1) : B(-1) - D(-1, -1);
  else price = h >= k ? C(-1, -1) : A(-1) - B(-1) + D(-1, -1);
  *out = std::fmax(price, 0.0) + rebate_value(p);
  return true;
}

// ------------------------------------------------------------------ Asian
struct Asian {
  double s, k, r, q, sigma, t;
  uint64_t n_steps;
  int geometric, floating, call;
  double running_avg, time_elapsed;  // NaN: none
  int f32 = 0;  // Monte Carlo in the FP32 form
};

bool seasoning(const Asian& p, double* a, double* t1) {  // asian.rs:44-50
  if (std::isnan(p.running_avg) || std::isnan(p.time_elapsed)) return false;
  if (!(p.time_elapsed > 0.0 && p.running_avg >= 0.0)) return false;
  *a = p.running_avg;
  *t1 = p.time_elapsed;
  return true;
}

double expected_geo_avg(double s, double r, double q, double sigma, double t1, double T, double g_spent) {
  const double rem = T - t1;  // asian.rs:52-59
  const double lsp = (t1 / T) * std::log(g_spent);
  const double my = (rem * std::log(s) + (r - q - 0.5 * sigma * sigma) * rem * rem / 2.0) / T;
  const double vy = sigma * sigma * std::pow(rem, 3) / (3.0 * T * T);
  return std::exp(lsp + my + 0.5 * vy);
}

double expected_arith_avg(double s, double r, double q, double t1, double T, double a_spent) {  // asian.rs:62-73
  const double rem = T - t1, mu = r - q;
  const double e = std::fabs(mu) < 1e-12 ? s : s * (std::exp(mu * rem) - 1.0) / (mu * rem);
  return (t1 / T) * a_spent + (rem / T) * e;
}

bool asian_geo_fixed(Asian p, double* out) {  // asian.rs:78-141 (Kemna-Vorst)
  if (p.t <= 0.0 || p.sigma <= 0.0 || !p.geometric || p.floating) return false;
  double a_spent, t1;
  if (seasoning(p, &a_spent, &t1)) {
    if (t1 >= p.t) {
      *out = p.call ? std::fmax(a_spent - p.k, 0.0) : std::fmax(p.k - a_spent, 0.0);
      return true;
    }
    const double rem = p.t - t1;
    const double kstar = (p.t * p.k - t1 * a_spent) / rem;
    const double scale = rem / p.t;
    if (kstar > 0.0) {
      Asian pp = p;
      pp.k = kstar;
      pp.t = rem;
      pp.running_avg = pp.time_elapsed = NAN;
      double v;
      if (!asian_geo_fixed(pp, &v)) return false;
      *out = scale * v;
      return true;
    }
    if (!p.call) {
      *out = 0.0;
    } else {
      const double eg = expected_geo_avg(p.s, p.r, p.q, p.sigma, t1, p.t, a_spent);
      *out = std::fmax(std::exp(-p.r * rem) * (eg - p.k), 0.0);
    }
    return true;
  }
  const double sg = p.sigma / std::sqrt(3.0);
  const double mug = 0.5 * (p.r - p.q - 0.5 * p.sigma * p.sigma) + 0.5 * 0.5 * sg * sg;
  const double d1 = (std::log(p.s / p.k) + (mug + 0.5 * sg * sg) * p.t) / (sg * std::sqrt(p.t));
  const double d2 = d1 - sg * std::sqrt(p.t);
  const double df = std::exp(-p.r * p.t);
  const double price = p.call ? p.s * std::exp((mug - p.r) * p.t) * ncdf(d1) - p.k * df * ncdf(d2)
                              : p.k * df * ncdf(-d2) - p.s * std::exp((mug - p.r) * p.t) * ncdf(-d1);
  *out = std::fmax(price, 0.0);
  return true;
}

// --------------------------------------------------------------- lookback
struct Lookback {
  double s, k, r, q, sigma, t;
  uint64_t n_steps;
  int fixed, call;
  double running_max, running_min;  // NaN: none
  int f32 = 0;  // Monte Carlo in the FP32 form
};

double lb_d1(double s, double x, double r, double q, double sigma, double t) {  // lookback.rs:40-43
  return (std::log(s / x) + (r - q + 0.5 * sigma * sigma) * t) / (sigma * std::sqrt(t));
}

double lb_t3(double s, double x, double r, double q, double sigma, double t) {  // lookback.rs:45-66
  const double st = std::sqrt(t);
  const double d1 = lb_d1(s, x, r, q, sigma, t);
  const double b = r - q, ert = std::exp(-r * t);
  if (std::fabs(b) < 1e-12) return s * ert * sigma * st * (npdf(d1) - d1 * ncdf(-d1));
  const double y = 2.0 * b / (sigma * sigma);
  const double arg2 = -d1 + (2.0 * b / sigma) * st;
  const double br = std::pow(s / x, -y) * ncdf(arg2) - std::exp(b * t) * ncdf(-d1);
  return s * ert * (sigma * sigma / (2.0 * b)) * br;
}

bool lookback_analytical(const Lookback& p, double* out) {  // lookback.rs:70-156
  if (p.t <= 0.0 || p.sigma <= 0.0) return false;
  const double eq = std::exp(-p.q * p.t), er = std::exp(-p.r * p.t), st = std::sqrt(p.t);
  const double M = std::isnan(p.running_max) ? p.s : p.running_max;
  const double m = std::isnan(p.running_min) ? p.s : p.running_min;
  double price;
  if (!p.fixed) {
    if (p.call) {
      if (m > p.s) return false;
      const double d1 = lb_d1(p.s, m, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
      price = p.s * eq * ncdf(d1) - m * er * ncdf(d2) + lb_t3(p.s, m, p.r, p.q, p.sigma, p.t);
    } else {
      if (M < p.s) return false;
      const double d1 = lb_d1(p.s, M, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
      price = M * er * ncdf(-d2) - p.s * eq * ncdf(-d1) + lb_t3(p.s, M, p.r, p.q, p.sigma, p.t);
    }
  } else {
    if (p.k <= 0.0) return false;
    if (p.call) {
      if (M < p.s) return false;
      if (p.k > M) {
        const double d1 = lb_d1(p.s, p.k, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
        price = p.s * eq * ncdf(d1) - p.k * er * ncdf(d2) + lb_t3(p.s, p.k, p.r, p.q, p.sigma, p.t);
      } else {
        const double d1 = lb_d1(p.s, M, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
        price = er * (M - p.k) + p.s * eq * ncdf(d1) - M * er * ncdf(d2) + lb_t3(p.s, M, p.r, p.q, p.sigma, p.t);
      }
    } else {
      if (m > p.s) return false;
      if (p.k < m) {
        const double d1 = lb_d1(p.s, p.k, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
        price = p.k * er * ncdf(-d2) - p.s * eq * ncdf(-d1) + lb_t3(p.s, p.k, p.r, p.q, p.sigma, p.t);
      } else {
        const double d1 = lb_d1(p.s, m, p.r, p.q, p.sigma, p.t), d2 = d1 - p.sigma * st;
        price = er * (p.k - m) + m * er * ncdf(-d2) - p.s * eq * ncdf(-d1) + lb_t3(p.s, m, p.r, p.q, p.sigma, p.t);
      }
    }
  }
  *out = std::fmax(price, 0.0);
  return true;
}

// ----------------------------------------------------------- MC drivers
// Launch description common to the three payoffs: GBM step constants of
// (r - q, sigma) over `steps` steps of t, streams of `seed`.
ExoticLaunch base_launch(stocha_ctx* c, double s, double k, double r, double q, double sigma, double t,
                         uint64_t steps, uint64_t n, uint64_t seed, int kind) {
  ExoticLaunch a;
  std::memset(&a, 0, sizeof a);
  const double dt = t / (double)steps;
  a.kind = kind;
  a.n = n;
  a.steps = steps;
  a.s0 = s;
  a.k = k;
  a.r = r;
  a.dt = dt;
  a.drift = (r - q - 0.5 * sigma * sigma) * dt;  // barrier.rs:292-294, asian.rs:201-204, lookback.rs:165-168
  a.diffusion = sigma * std::sqrt(dt);
  a.discount = std::exp(-r * t);
  a.log_s0 = std::log(s);
  make_stream_spec((u128)seed, ((u128)steps + 1024) * 2, &a.ss);
  a.tabs = c->d_tabs;
  a.err = c->d_err;
  return a;
}

int sms_of(stocha_ctx* c) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  return sms;
}

// Runs a summing kind and returns the FP64 total of the per-path values.
int run_sum(stocha_ctx* c, ExoticLaunch& a, double* total) {
  const int grid = exotic_grid(a.n, sms_of(c));
  int rc;
  if ((rc = ensure_buf(c, c->partials, (size_t)grid * 2 * sizeof(double)))) return rc;
  if ((rc = ensure_buf(c, c->small, 64 * sizeof(double)))) return rc;
  a.partials = (double*)c->partials.ptr;
  if ((rc = begin_call(c))) return rc;
  launch_exotic(a, grid, c->stream);
  STOCHA_CUDA(cudaGetLastError());
  launch_reduce_partials(a.partials, grid, 2, (double*)c->small.ptr, c->stream);
  STOCHA_CUDA(cudaMemcpyAsync(c->h_small, c->small.ptr, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = finish_call(c))) return rc;
  *total = c->h_small[0];
  return STOCHA_OK;
}

int barrier_mc(stocha_ctx* c, const Barrier& p, uint64_t n, uint64_t steps, uint64_t seed, double* out) {
  ExoticLaunch a = base_launch(c, p.s, p.k, p.r, p.q, p.sigma, p.t, steps, n, seed, kExoBarrier);
  a.barrier = p.h;  // Monte Carlo monitors the given barrier at every step (barrier.rs:36-38)
  a.direction = p.up ? 0 : 1;
  a.kind_in = p.in;
  a.is_call = p.call;
  a.rebate = p.rebate;
  a.rebate_at_hit = p.at_hit;
  a.already_hit = p.up ? p.s >= p.h : p.s <= p.h;
  a.f32 = p.f32;
  a.lbarrier = std::log(p.h / p.s);
  double total = 0.0;
  int rc = n ? run_sum(c, a, &total) : STOCHA_OK;
  if (rc) return rc;
  *out = a.discount * total / (double)n;  // barrier.rs:370
  return STOCHA_OK;
}

int lookback_mc(stocha_ctx* c, const Lookback& p, uint64_t n, uint64_t seed, double* out) {
  ExoticLaunch a = base_launch(c, p.s, p.k, p.r, p.q, p.sigma, p.t, p.n_steps, n, seed, kExoLookback);
  a.strike_fixed = p.fixed;
  a.is_call = p.call;
  a.m0 = std::fmax(std::isnan(p.running_max) ? p.s : p.running_max, p.s);  // lookback.rs:185-186
  a.n0 = std::fmin(std::isnan(p.running_min) ? p.s : p.running_min, p.s);
  a.f32 = p.f32;
  a.lm0 = std::log(a.m0 / p.s);
  a.ln0 = std::log(a.n0 / p.s);
  double total = 0.0;
  int rc = n ? run_sum(c, a, &total) : STOCHA_OK;
  if (rc) return rc;
  *out = a.discount * total / (double)n;
  return STOCHA_OK;
}

int asian_mc(stocha_ctx* c, const Asian& p, uint64_t n, uint64_t seed, double* out);

int asian_floating_seasoned(stocha_ctx* c, const Asian& p, double a_spent, double t1, uint64_t n, uint64_t seed,
                            double* out) {  // asian.rs:292-352
  const double rem = p.t - t1;
  uint64_t nr = (uint64_t)std::llround((double)p.n_steps * rem / p.t);
  if (nr < 1) nr = 1;
  ExoticLaunch a = base_launch(c, p.s, 0.0, p.r, p.q, p.sigma, rem, nr, n, seed, kExoAsianSeasoned);
  a.is_call = p.call;
  a.geometric = p.geometric;
  a.a_spent = a_spent;
  a.w_spent = t1 / p.t;
  a.w_remain = rem / p.t;
  a.f32 = p.f32;
  double total = 0.0;
  int rc = n ? run_sum(c, a, &total) : STOCHA_OK;
  if (rc) return rc;
  *out = a.discount * total / (double)n;
  return STOCHA_OK;
}

int asian_mc(stocha_ctx* c, const Asian& p, uint64_t n, uint64_t seed, double* out) {  // asian.rs:143-290
  double a_spent, t1;
  if (seasoning(p, &a_spent, &t1)) {
    if (t1 >= p.t) {
      *out = !p.floating ? (p.call ? std::fmax(a_spent - p.k, 0.0) : std::fmax(p.k - a_spent, 0.0)) : 0.0;
      return STOCHA_OK;
    }
    if (!p.floating) {
      const double rem = p.t - t1;
      const double kstar = (p.t * p.k - t1 * a_spent) / rem;
      const double scale = rem / p.t;
      if (kstar > 0.0) {
        Asian pp = p;
        pp.k = kstar;
        pp.t = rem;
        pp.running_avg = pp.time_elapsed = NAN;
        double v = 0.0;
        int rc = asian_mc(c, pp, n, seed, &v);
        if (rc) return rc;
        *out = scale * v;
        return STOCHA_OK;
      }
      if (!p.call) {
        *out = 0.0;
      } else {
        const double e = p.geometric ? expected_geo_avg(p.s, p.r, p.q, p.sigma, t1, p.t, a_spent)
                                     : expected_arith_avg(p.s, p.r, p.q, t1, p.t, a_spent);
        *out = std::fmax(std::exp(-p.r * rem) * (e - p.k), 0.0);
      }
      return STOCHA_OK;
    }
    return asian_floating_seasoned(c, p, a_spent, t1, n, seed, out);
  }
  ExoticLaunch a = base_launch(c, p.s, p.k, p.r, p.q, p.sigma, p.t, p.n_steps, n, seed, kExoAsian);
  a.strike_floating = p.floating;
  a.is_call = p.call;
  a.f32 = p.f32;
  const bool use_cv = !p.geometric && !p.floating;
  double geo_analytical = 0.0;
  if (use_cv) {
    Asian g = p;
    g.geometric = 1;
    if (!asian_geo_fixed(g, &geo_analytical)) geo_analytical = 0.0;
  }
  if (n == 0) {
    *out = NAN;
    return STOCHA_OK;
  }
  const int sms = sms_of(c);
  const int grid = exotic_grid(n, sms);
  const int rgrid = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
  int rc;
  if ((rc = ensure_buf(c, c->aux, (size_t)n * 2 * sizeof(double)))) return rc;
  if ((rc = ensure_buf(c, c->partials, (size_t)(rgrid > grid ? rgrid : grid) * 2 * sizeof(double)))) return rc;
  if ((rc = ensure_buf(c, c->small, 64 * sizeof(double)))) return rc;
  a.arith = (double*)c->aux.ptr;
  a.geo = a.arith + n;
  a.partials = (double*)c->partials.ptr;
  double* sm = (double*)c->small.ptr;  // [0..1] totals, [2..3] means, [4..5] centred sums
  if ((rc = begin_call(c))) return rc;
  launch_exotic(a, grid, c->stream);
  STOCHA_CUDA(cudaGetLastError());
  launch_asian_sums(a.arith, a.geo, n, 0, nullptr, a.partials, rgrid, c->stream);
  launch_reduce_partials(a.partials, rgrid, 2, sm, c->stream);
  launch_asian_means(sm, n, sm + 2, c->stream);
  launch_asian_sums(a.arith, a.geo, n, 1, sm + 2, a.partials, rgrid, c->stream);
  launch_reduce_partials(a.partials, rgrid, 2, sm + 4, c->stream);
  STOCHA_CUDA(cudaGetLastError());
  STOCHA_CUDA(cudaMemcpyAsync(c->h_small, sm, 6 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = finish_call(c))) return rc;
  const double* h = c->h_small;
  const double ma = h[2], mg = h[3], cov = h[4], vg = h[5];
  if (use_cv && n > 1) {  // asian.rs:270-283
    const double beta = vg > 1e-30 ? cov / vg : 0.0;
    const double geo_mc = a.discount * mg;
    *out = std::fmax(a.discount * ma - beta * (geo_mc - geo_analytical), 0.0);
  } else {  // asian.rs:284-288: the mean of the arithmetic-average payoff
    *out = std::fmax(a.discount * ma, 0.0);
  }
  return STOCHA_OK;
}

int with_ctx(stocha_ctx** ctx) {
  int rc = resolve_ctx(ctx);
  if (rc) return rc;
  cudaSetDevice((*ctx)->device);
  return STOCHA_OK;
}

bool streq(const char* a, const char* b) { return a && std::strcmp(a, b) == 0; }

}  // namespace

extern "C" {

int stocha_barrier_price(stocha_ctx* ctx, double s, double k, double r, double sigma, double t, double barrier,
                         const char* barrier_type, const char* option_type, double q, uint64_t n_paths,
                         uint64_t n_steps, uint64_t seed, const char* method, int32_t n_monitoring, double rebate,
                         int32_t rebate_at_hit, int32_t precision, double* price) {
  STOCHA_RANGE("stocha_barrier_price");
  if (precision != STOCHA_FP64 && precision != STOCHA_FP32)
    return set_error(STOCHA_ERR_VALUE, "precision must be 'fp64' or 'fp32'");
  // lib.rs:1567-1582
  if (s <= 0.0) return set_error(STOCHA_ERR_VALUE, "s must be positive");
  if (k <= 0.0) return set_error(STOCHA_ERR_VALUE, "k must be positive");
  if (sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  if (barrier <= 0.0) return set_error(STOCHA_ERR_VALUE, "barrier must be positive");
  Barrier p;
  const std::string bt = barrier_type ? barrier_type : "";
  if (bt == "up-and-out" || bt == "uo") p.up = 1, p.in = 0;  // lib.rs:1584-1596
  else if (bt == "up-and-in" || bt == "ui") p.up = 1, p.in = 1;
  else if (bt == "down-and-out" || bt == "do") p.up = 0, p.in = 0;
  else if (bt == "down-and-in" || bt == "di") p.up = 0, p.in = 1;
  else
    return set_error(STOCHA_ERR_VALUE, "Unknown barrier_type: '" + bt +
                                           "'. Supported: 'up-and-out', 'up-and-in', 'down-and-out', 'down-and-in'");
  if (streq(option_type, "call")) p.call = 1;
  else if (streq(option_type, "put")) p.call = 0;
  else
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown option_type: '") + (option_type ? option_type : "") +
                                           "'. Supported: 'call', 'put'");
  p.s = s, p.k = k, p.r = r, p.q = q, p.sigma = sigma, p.t = t, p.h = barrier;
  p.n_mon = n_monitoring;
  p.rebate = rebate;
  p.at_hit = rebate_at_hit ? 1 : 0;
  p.f32 = precision == STOCHA_FP32;
  const std::string m = method ? method : "";
  int rc;
  if (m == "auto" || m == "analytical") {  // lib.rs:1618-1630
    double v = 0.0;
    const bool ok = barrier_analytical(p, &v);
    if (ok && (m == "analytical" || std::isfinite(v))) {
      *price = v;
      return STOCHA_OK;
    }
    if (m == "analytical")
      return set_error(STOCHA_ERR_VALUE, "Analytical solution not available for these parameters");
  } else if (m != "mc") {
    return set_error(STOCHA_ERR_VALUE, "Unknown method: '" + m + "'. Supported: 'auto', 'analytical', 'mc'");
  }
  if ((rc = with_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  return barrier_mc(ctx, p, n_paths, n_steps, seed, price);
}

int stocha_asian_price(stocha_ctx* ctx, double s, double k, double r, double sigma, double t, uint64_t n_steps,
                       const char* average_type, const char* strike_type, const char* option_type, double q,
                       uint64_t n_paths, uint64_t seed, const char* method, double running_avg, double time_elapsed,
                       int32_t precision, double* price) {
  STOCHA_RANGE("stocha_asian_price");
  if (precision != STOCHA_FP64 && precision != STOCHA_FP32)
    return set_error(STOCHA_ERR_VALUE, "precision must be 'fp64' or 'fp32'");
  // lib.rs:1664-1716
  if (s <= 0.0) return set_error(STOCHA_ERR_VALUE, "s must be positive");
  if (k <= 0.0) return set_error(STOCHA_ERR_VALUE, "k must be positive");
  if (sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  Asian p;
  if (streq(average_type, "arithmetic")) p.geometric = 0;
  else if (streq(average_type, "geometric")) p.geometric = 1;
  else
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown average_type: '") + (average_type ? average_type : "") +
                                           "'. Supported: 'arithmetic', 'geometric'");
  if (streq(strike_type, "fixed")) p.floating = 0;
  else if (streq(strike_type, "floating")) p.floating = 1;
  else
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown strike_type: '") + (strike_type ? strike_type : "") +
                                           "'. Supported: 'fixed', 'floating'");
  if (streq(option_type, "call")) p.call = 1;
  else if (streq(option_type, "put")) p.call = 0;
  else
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown option_type: '") + (option_type ? option_type : "") +
                                           "'. Supported: 'call', 'put'");
  p.s = s, p.k = k, p.r = r, p.q = q, p.sigma = sigma, p.t = t, p.n_steps = n_steps;
  p.running_avg = running_avg;
  p.time_elapsed = time_elapsed;
  p.f32 = precision == STOCHA_FP32;
  const bool has_analytical = p.geometric && !p.floating;
  const std::string m = method ? method : "";
  int rc;
  if (m == "auto") {  // lib.rs:1724-1734
    double v = 0.0;
    if (has_analytical && asian_geo_fixed(p, &v)) {
      *price = v;
      return STOCHA_OK;
    }
  } else if (m == "analytical") {
    double v = 0.0;
    if (!has_analytical)
      return set_error(STOCHA_ERR_VALUE, "Analytical solution only available for geometric average with fixed strike");
    if (!asian_geo_fixed(p, &v))
      return set_error(STOCHA_ERR_VALUE, "Analytical solution not available for these parameters");
    *price = v;
    return STOCHA_OK;
  } else if (m != "mc") {
    return set_error(STOCHA_ERR_VALUE, "Unknown method: '" + m + "'. Supported: 'auto', 'analytical', 'mc'");
  }
  if (p.n_steps == 0) return set_error(STOCHA_ERR_VALUE, "n_steps must be positive");
  // the device's Asian log sum weights each step exponent by an integer built
  // as an exact double, which holds below 2^53 steps
  if (p.n_steps >= (1ull << 53)) return set_error(STOCHA_ERR_VALUE, "n_steps must be below 2^53");
  if ((rc = with_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  return asian_mc(ctx, p, n_paths, seed, price);
}

int stocha_lookback_price(stocha_ctx* ctx, double s, double r, double sigma, double t, uint64_t n_steps,
                          const char* strike_type, const char* option_type, double k, double q, uint64_t n_paths,
                          uint64_t seed, const char* method, double running_max, double running_min,
                          int32_t precision, double* price) {
  STOCHA_RANGE("stocha_lookback_price");
  if (precision != STOCHA_FP64 && precision != STOCHA_FP32)
    return set_error(STOCHA_ERR_VALUE, "precision must be 'fp64' or 'fp32'");
  // lib.rs:1779-1814
  if (s <= 0.0) return set_error(STOCHA_ERR_VALUE, "s must be positive");
  if (sigma <= 0.0) return set_error(STOCHA_ERR_VALUE, "sigma must be positive");
  if (t <= 0.0) return set_error(STOCHA_ERR_VALUE, "t must be positive");
  Lookback p;
  if (streq(strike_type, "floating")) {
    p.fixed = 0;
  } else if (streq(strike_type, "fixed")) {
    if (k <= 0.0) return set_error(STOCHA_ERR_VALUE, "k must be positive for fixed strike lookback");
    p.fixed = 1;
  } else {
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown strike_type: '") + (strike_type ? strike_type : "") +
                                           "'. Supported: 'floating', 'fixed'");
  }
  if (streq(option_type, "call")) p.call = 1;
  else if (streq(option_type, "put")) p.call = 0;
  else
    return set_error(STOCHA_ERR_VALUE, std::string("Unknown option_type: '") + (option_type ? option_type : "") +
                                           "'. Supported: 'call', 'put'");
  p.s = s, p.k = k, p.r = r, p.q = q, p.sigma = sigma, p.t = t, p.n_steps = n_steps;
  p.running_max = running_max;
  p.running_min = running_min;
  p.f32 = precision == STOCHA_FP32;
  const std::string m = method ? method : "";
  int rc;
  if (m == "auto" || m == "analytical") {  // lib.rs:1836-1847
    double v = 0.0;
    if (lookback_analytical(p, &v) && std::isfinite(v)) {
      *price = v;
      return STOCHA_OK;
    }
    if (m == "analytical")
      return set_error(STOCHA_ERR_VALUE, "Analytical solution not available for these parameters");
  } else if (m != "mc") {
    return set_error(STOCHA_ERR_VALUE, "Unknown method: '" + m + "'. Supported: 'auto', 'analytical', 'mc'");
  }
  if (p.n_steps == 0) return set_error(STOCHA_ERR_VALUE, "n_steps must be positive");
  if ((rc = with_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  return lookback_mc(ctx, p, n_paths, seed, price);
}

}  // extern "C"
