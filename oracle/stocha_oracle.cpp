// CPU oracle for the stocha Monte Carlo path.  TEST INFRASTRUCTURE ONLY:
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
// library as the checker and as the timed CPU restatement.  The product
// (stocha_gb300/) never links, loads or calls it.
//
// Each function restates the reference's algorithm (heki1224/stocha v1.7.1,
// Rust) with the same floating-point operation order, so that results match
// the reference bit for bit except where a libm function (exp, ln) differs by
// an ulp from the platform libm the reference links.  Build with
// -ffp-contract=off: Rust never contracts a*b+c into an FMA.
//
// Parity pins:
//   * PCG64DXSM output and jump-ahead: pinned against NumPy's PCG64DXSM with
//     the state set directly (tests/golden/pcg64dxsm_numpy.json).
//   * Seeding (Pcg64Dxsm::new -> rand_pcg 0.10.2 Lcg128CmDxsm64::new):
//     restated from rand_pcg's published PCG seeding (increment =
//     (stream << 1) | 1; state += increment; one LCG step).  rand_pcg itself
//     is not in the reference tree and cannot be built here (no Rust
//     toolchain), so this mapping is parity-unpinned.
//   * Ziggurat tables: regenerated by stocha_gb300/gen_ziggurat.py and
//     compared value by value with src/dist/ziggurat_tables.rs.
//   * LSMC least squares: the reference calls faer 0.24 QR (lsmc.rs:83-84);
//     faer is not in the tree, so oracle_lsmc restates Householder QR least
//     squares (parity-unpinned at the rounding level) and also offers the
//     normal-equation solve the GPU uses.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "../stocha_gb300/csrc/ziggurat_table.inc"

typedef unsigned __int128 u128;

namespace {

const uint64_t kMul = 0xda942042e4dd58b5ULL;  // rand_pcg Lcg128CmDxsm64 "cheap multiplier"
const u128 kStreamOffset =
    ((u128)0xda3e39cb94b95bdbULL << 64) | (u128)0x7ef55da5c0374f5aULL;  // pcg64.rs:25
const double kTwoM53 = 1.0 / 9007199254740992.0;                     // pcg64.rs:38

const double kZigR = STOCHA_ZIG_R_HEX;
const double kZigX[257] = STOCHA_ZIG_X_INIT;
const double kZigY[257] = STOCHA_ZIG_Y_INIT;

// rand_pcg Lcg128CmDxsm64: 128-bit LCG, DXSM output of the state *before* the
// step (pcg64.rs:33-35 -> rand_pcg next_u64).
struct Pcg {
  u128 state;
  u128 inc;
  uint64_t used;  // u64 draws taken (consumption diagnostics)

  static Pcg seeded(u128 seed) {  // pcg64.rs:23-30
    Pcg p;
    u128 stream = seed + kStreamOffset;
    p.inc = (stream << 1) | 1;
    p.state = seed + p.inc;
    p.state = p.state * kMul + p.inc;
    p.used = 0;
    return p;
  }
  uint64_t next_u64() {
    uint64_t hi = (uint64_t)(state >> 64);
    uint64_t lo = (uint64_t)state | 1;
    hi ^= hi >> 32;
    hi *= kMul;
    hi ^= hi >> 48;
    hi *= lo;
    state = state * kMul + inc;
    ++used;
    return hi;
  }
  double next_f64() { return (double)(next_u64() >> 11) * kTwoM53; }
  // pcg64.rs:41-43 -> rand_pcg advance: Brown's arbitrary-stride LCG jump.
  void advance(u128 delta) {
    u128 acc_mult = 1, acc_plus = 0, cur_mult = kMul, cur_plus = inc;
    while (delta > 0) {
      if (delta & 1) {
        acc_mult *= cur_mult;
        acc_plus = acc_plus * cur_mult + cur_plus;
      }
      cur_plus = (cur_mult + 1) * cur_plus;
      cur_mult *= cur_mult;
      delta >>= 1;
    }
    state = acc_mult * state + acc_plus;
  }
};

// src/dist/normal.rs:54-67 (sample_tail)
double zig_tail(Pcg& g) {
  for (;;) {
    double u1 = g.next_f64();
    double u2 = g.next_f64();
    if (u1 <= 0.0 || u2 <= 0.0) continue;
    double x = -std::log(u1) / kZigR;
    if (-2.0 * std::log(u2) >= x * x) return x + kZigR;
  }
}

// src/dist/normal.rs:18-43 (NormalSampler::sample)
double zig_normal(Pcg& g) {
  for (;;) {
    uint64_t u = g.next_u64();
    unsigned layer = (unsigned)(u & 0xFF);
    double sign = (double)((u >> 8) & 1) * -2.0 + 1.0;
    double u_frac = (double)(u >> 11) * kTwoM53;
    double x = u_frac * kZigX[layer];
    if (x < kZigX[layer + 1]) return sign * x;
    if (layer == 0) return sign * zig_tail(g);
    double y = kZigY[layer] + g.next_f64() * (kZigY[layer + 1] - kZigY[layer]);
    if (y < std::exp(-0.5 * x * x)) return sign * x;
  }
}

Pcg path_stream(uint64_t seed, uint64_t path, u128 block) {  // gbm.rs:58-59
  Pcg g = Pcg::seeded((u128)seed);
  g.advance((u128)path * block);
  g.used = 0;
  return g;
}

int resolve_threads(int threads) {
  if (threads > 0) return threads;
  unsigned hc = std::thread::hardware_concurrency();
  return hc ? (int)hc : 1;
}

// Rayon-like parallel-for over [0, n) in contiguous ranges.
void parallel_for(uint64_t n, int threads, const std::function<void(uint64_t, uint64_t)>& body) {
  threads = resolve_threads(threads);
  if (threads <= 1 || n < 2) {
    body(0, n);
    return;
  }
  uint64_t nt = std::min<uint64_t>((uint64_t)threads, n);
  std::vector<std::thread> pool;
  pool.reserve(nt);
  for (uint64_t t = 0; t < nt; ++t) {
    uint64_t a = n * t / nt, b = n * (t + 1) / nt;
    pool.emplace_back([&body, a, b] { body(a, b); });
  }
  for (auto& th : pool) th.join();
}

// Runs `sim(i, row)` for n rows of `len` doubles.  gather=1 mimics the
// reference exactly: every path fills its own Vec, then one thread copies the
// Vec<Vec<f64>> into the output array (gbm.rs:78-105).
void run_rows(uint64_t n, uint64_t len, int threads, int gather, double* out,
              const std::function<void(uint64_t, double*)>& sim) {
  if (!gather) {
    parallel_for(n, threads, [&](uint64_t a, uint64_t b) {
      for (uint64_t i = a; i < b; ++i) sim(i, out + i * len);
    });
    return;
  }
  std::vector<std::vector<double>> rows(n);
  parallel_for(n, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) {
      rows[i].resize(len);
      sim(i, rows[i].data());
    }
  });
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t j = 0; j < len; ++j) out[i * len + j] = rows[i][j];
}

// compiler-rt __powidf2, which Rust's f64::powi lowers to (lsmc.rs:69,78,93).
double powi(double a, int b) {
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return r;
}

// Rust f64::max: NaN operands are ignored (same as C fmax).
inline double rmax(double a, double b) { return std::fmax(a, b); }

}  // namespace

#define ORACLE_API extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------- PCG ----
// State words are passed as (lo, hi) u64 pairs.
ORACLE_API void oracle_pcg_seed(uint64_t seed_lo, uint64_t seed_hi, uint64_t* state2, uint64_t* inc2) {
  Pcg g = Pcg::seeded(((u128)seed_hi << 64) | seed_lo);
  state2[0] = (uint64_t)g.state;
  state2[1] = (uint64_t)(g.state >> 64);
  inc2[0] = (uint64_t)g.inc;
  inc2[1] = (uint64_t)(g.inc >> 64);
}

ORACLE_API void oracle_pcg_advance(uint64_t* state2, const uint64_t* inc2, uint64_t delta_lo, uint64_t delta_hi) {
  Pcg g;
  g.state = ((u128)state2[1] << 64) | state2[0];
  g.inc = ((u128)inc2[1] << 64) | inc2[0];
  g.advance(((u128)delta_hi << 64) | delta_lo);
  state2[0] = (uint64_t)g.state;
  state2[1] = (uint64_t)(g.state >> 64);
}

// Raw u64 outputs from an explicit (state, inc); the state is updated.
ORACLE_API void oracle_pcg_fill_u64(uint64_t* state2, const uint64_t* inc2, uint64_t n, uint64_t* out) {
  Pcg g;
  g.state = ((u128)state2[1] << 64) | state2[0];
  g.inc = ((u128)inc2[1] << 64) | inc2[0];
  for (uint64_t i = 0; i < n; ++i) out[i] = g.next_u64();
  state2[0] = (uint64_t)g.state;
  state2[1] = (uint64_t)(g.state >> 64);
}

// One sequential stream of draws, as RNG.uniform / standard_normal / normal
// do (lib.rs:110-148).  kind: 0 uniform, 1 standard normal, 2 loc+scale*z.
// Returns the number of u64 consumed.
ORACLE_API uint64_t oracle_stream_fill(uint64_t* state2, const uint64_t* inc2, int kind, double loc, double scale,
                            uint64_t n, double* out) {
  Pcg g;
  g.state = ((u128)state2[1] << 64) | state2[0];
  g.inc = ((u128)inc2[1] << 64) | inc2[0];
  g.used = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (kind == 0)
      out[i] = g.next_f64();
    else if (kind == 1)
      out[i] = zig_normal(g);
    else
      out[i] = loc + scale * zig_normal(g);  // normal.rs:77-79
  }
  state2[0] = (uint64_t)g.state;
  state2[1] = (uint64_t)(g.state >> 64);
  return g.used;
}

// -------------------------------------------------------------- models ---
namespace {

// Per-path simulators.  Each writes one output row and returns the u64 count.
struct GbmSim {  // src/finance/gbm.rs:42-107
  double s0, drift, diffusion;
  uint64_t steps, base, seed;
  u128 block;
  GbmSim(double s0_, double mu, double sigma, double q, double t, uint64_t steps_, uint64_t n_paths,
         int antithetic, uint64_t seed_)
      : s0(s0_), steps(steps_), seed(seed_) {
    const double dt = t / (double)steps;
    drift = (mu - q - 0.5 * sigma * sigma) * dt;
    diffusion = sigma * std::sqrt(dt);
    base = antithetic ? (n_paths + 1) / 2 : n_paths;
    block = ((u128)steps + 1024) * 2;
  }
  uint64_t operator()(uint64_t row, double* path) const {
    bool neg = row >= base;
    Pcg g = path_stream(seed, neg ? row - base : row, block);
    double s = s0;
    path[0] = s0;
    for (uint64_t k = 0; k < steps; ++k) {
      double z = neg ? -zig_normal(g) : zig_normal(g);
      s *= std::exp(drift + diffusion * z);
      path[k + 1] = s;
    }
    return g.used;
  }
};

struct HestonSim {  // src/finance/heston.rs:44-174
  double s0, v0, mu, kappa, theta, xi, rho, dt, sqrt_dt, rho_comp, e_kdt, k1;
  uint64_t steps, seed;
  int scheme;
  u128 block;
  HestonSim(double s0_, double v0_, double mu_, double kappa_, double theta_, double xi_, double rho_, double t,
            uint64_t steps_, int scheme_, uint64_t seed_)
      : s0(s0_), v0(v0_), mu(mu_), kappa(kappa_), theta(theta_), xi(xi_), rho(rho_), steps(steps_),
        seed(seed_), scheme(scheme_) {
    dt = t / (double)steps;
    sqrt_dt = std::sqrt(dt);
    rho_comp = std::sqrt(1.0 - rho * rho);
    e_kdt = std::exp(-kappa * dt);
    k1 = kappa * theta;
    block = ((u128)steps + 1024) * 6;
  }
  uint64_t operator()(uint64_t i, double* path) const {
    Pcg g = path_stream(seed, i, block);
    double s = s0, v = v0;
    path[0] = s0;
    if (scheme == 0) {
      for (uint64_t k = 0; k < steps; ++k) {
        double dw1 = zig_normal(g);
        double dz = zig_normal(g);
        double dw2 = rho * dw1 + rho_comp * dz;
        double v_plus = rmax(v, 0.0);
        double sqrt_v = std::sqrt(v_plus);
        v += kappa * (theta - v_plus) * dt + xi * sqrt_v * sqrt_dt * dw2;
        s *= std::exp((mu - 0.5 * v_plus) * dt + sqrt_v * sqrt_dt * dw1);
        path[k + 1] = s;
      }
      return g.used;
    }
    for (uint64_t k = 0; k < steps; ++k) {
      double v_plus = rmax(v, 0.0);
      double m = k1 * (1.0 - e_kdt) / kappa + v_plus * e_kdt;
      m = rmax(m, 1e-15);
      double s2 = v_plus * xi * xi * e_kdt * (1.0 - e_kdt) / kappa +
                  k1 * xi * xi * powi(1.0 - e_kdt, 2) / (2.0 * kappa * kappa);
      double psi = s2 / (m * m);
      double v_next;
      if (psi <= 1.5) {
        double b2 = 2.0 / psi - 1.0 + std::sqrt(2.0 / psi * (2.0 / psi - 1.0));
        b2 = rmax(b2, 0.0);
        double a = m / (1.0 + b2);
        double b = std::sqrt(b2);
        double z = zig_normal(g);
        v_next = a * (b + z) * (b + z);
      } else {
        double p = (psi - 1.0) / (psi + 1.0);
        double beta = (1.0 - p) / m;
        double u = g.next_f64();
        v_next = (u <= p) ? 0.0 : std::log((1.0 - p) / (1.0 - u)) / beta;
      }
      v_next = rmax(v_next, 0.0);
      double z1 = zig_normal(g);
      double kappa_rho_xi = kappa * rho / xi;
      double k0_s = (mu - kappa_rho_xi * theta) * dt;
      double k1_s = 0.5 * dt * (kappa_rho_xi - 0.5) - rho / xi;
      double k2_s = 0.5 * dt * (kappa_rho_xi - 0.5) + rho / xi;
      double k3_s = 0.5 * dt * (1.0 - rho * rho);
      double k4_s = 0.5 * dt * (1.0 - rho * rho);
      double var_term = rmax(k3_s * v_plus + k4_s * v_next, 0.0);
      double log_s = std::log(s) + k0_s + k1_s * v_plus + k2_s * v_next + std::sqrt(var_term) * z1;
      s = std::exp(std::min(std::max(log_s, -500.0), 500.0));  // f64::clamp(-500, 500)
      v = v_next;
      path[k + 1] = s;
    }
    return g.used;
  }
};

struct MertonSim {  // src/finance/jump_diffusion.rs:48-105
  double s0, mu_j, sigma_j, drift, diffusion, jump_prob;
  uint64_t steps, seed;
  u128 block;
  MertonSim(double s0_, double mu, double sigma, double lambda, double mu_j_, double sigma_j_, double t,
            uint64_t steps_, uint64_t seed_)
      : s0(s0_), mu_j(mu_j_), sigma_j(sigma_j_), steps(steps_), seed(seed_) {
    const double dt = t / (double)steps;
    const double sqrt_dt = std::sqrt(dt);
    const double m_bar = std::exp(mu_j + 0.5 * sigma_j * sigma_j) - 1.0;
    drift = (mu - 0.5 * sigma * sigma - lambda * m_bar) * dt;
    diffusion = sigma * sqrt_dt;
    jump_prob = lambda * dt;
    block = ((u128)steps + 1024) * 8;
  }
  uint64_t operator()(uint64_t i, double* path) const {
    Pcg g = path_stream(seed, i, block);
    double s = s0;
    path[0] = s0;
    for (uint64_t k = 0; k < steps; ++k) {
      double z = zig_normal(g);
      double diffusion_return = drift + diffusion * z;
      double u = g.next_f64();
      double jump_return = 0.0;
      if (u < jump_prob) {
        double z_j = zig_normal(g);
        jump_return = mu_j + sigma_j * z_j;
      }
      s *= std::exp(diffusion_return + jump_return);
      path[k + 1] = s;
    }
    return g.used;
  }
};

struct MultiGbmSim {  // src/finance/multi_gbm.rs:22-113
  int na;
  std::vector<double> s0, l, drift, diffusion;
  uint64_t steps, base, seed;
  u128 block;
  uint64_t operator()(uint64_t row, double* path) const {
    bool neg = row >= base;
    Pcg g = path_stream(seed, neg ? row - base : row, block);
    std::vector<double> z(na), s(s0);
    for (int i = 0; i < na; ++i) path[i] = s0[i];
    uint64_t w = na;
    for (uint64_t k = 0; k < steps; ++k) {
      for (int i = 0; i < na; ++i) z[i] = zig_normal(g);
      if (neg)
        for (int i = 0; i < na; ++i) z[i] = -z[i];
      for (int i = 0; i < na; ++i) {
        double eps = 0.0;
        for (int m = 0; m <= i; ++m) eps += l[i * na + m] * z[m];
        s[i] *= std::exp(drift[i] + diffusion[i] * eps);
        path[w++] = s[i];
      }
    }
    return g.used;
  }
};

template <class Sim>
void run_sim(const Sim& sim, uint64_t n, uint64_t len, int threads, int gather, double* out, uint64_t* used) {
  run_rows(n, len, threads, gather, out, [&](uint64_t i, double* row) {
    uint64_t u = sim(i, row);
    if (used) used[i] = u;
  });
}

// Terminal column only, one path at a time per worker (greeks.rs:165-166 keeps
// the last column of the full array; the values are the same).
template <class Sim>
void run_terminal(const Sim& sim, uint64_t n, uint64_t len, int threads, double* terminal) {
  parallel_for(n, threads, [&](uint64_t a, uint64_t b) {
    std::vector<double> row(len);
    for (uint64_t i = a; i < b; ++i) {
      sim(i, row.data());
      terminal[i] = row[len - 1];
    }
  });
}

}  // namespace

ORACLE_API void oracle_gbm(double s0, double mu, double sigma, double q, double t, uint64_t steps, uint64_t n_paths,
                int antithetic, uint64_t seed, int threads, int gather, double* out, uint64_t* used) {
  GbmSim sim(s0, mu, sigma, q, t, steps, n_paths, antithetic, seed);
  run_sim(sim, n_paths, steps + 1, threads, gather, out, used);
}

// src/copula/gaussian.rs:76-99.  Returns 0, or 1 + failing diagonal index.
ORACLE_API int oracle_cholesky(int n, const double* a, double* l, double* bad_value) {
  for (int i = 0; i < n * n; ++i) l[i] = 0.0;
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      double sum = a[i * n + j];
      for (int k = 0; k < j; ++k) sum -= l[i * n + k] * l[j * n + k];
      if (i == j) {
        if (sum <= 0.0) {
          if (bad_value) *bad_value = sum;
          return 1 + i;
        }
        l[i * n + j] = std::sqrt(sum);
      } else {
        l[i * n + j] = sum / l[j * n + j];
      }
    }
  }
  return 0;
}

// out: n_paths x (steps+1) x n_assets.  Returns 1 if corr is not PD.
ORACLE_API int oracle_multi_gbm(int n_assets, const double* s0, const double* mu, const double* sigma, const double* corr,
                     double t, uint64_t steps, uint64_t n_paths, int antithetic, uint64_t seed, int threads,
                     int gather, double* out, uint64_t* used) {
  MultiGbmSim sim;
  sim.na = n_assets;
  sim.l.resize((size_t)n_assets * n_assets);
  if (oracle_cholesky(n_assets, corr, sim.l.data(), nullptr) != 0) return 1;
  const double dt = t / (double)steps;
  const double sqrt_dt = std::sqrt(dt);
  sim.s0.assign(s0, s0 + n_assets);
  sim.drift.resize(n_assets);
  sim.diffusion.resize(n_assets);
  for (int i = 0; i < n_assets; ++i) {
    sim.drift[i] = (mu[i] - 0.5 * sigma[i] * sigma[i]) * dt;
    sim.diffusion[i] = sigma[i] * sqrt_dt;
  }
  sim.steps = steps;
  sim.seed = seed;
  sim.base = antithetic ? (n_paths + 1) / 2 : n_paths;
  sim.block = ((u128)steps * (u128)n_assets + 1024) * 2;
  run_sim(sim, n_paths, (steps + 1) * (uint64_t)n_assets, threads, gather, out, used);
  return 0;
}

// scheme 0: full-truncation Euler (default); 1: Andersen QE.
ORACLE_API void oracle_heston(double s0, double v0, double mu, double kappa, double theta, double xi, double rho, double t,
                   uint64_t steps, uint64_t n_paths, int scheme, uint64_t seed, int threads, int gather,
                   double* out, uint64_t* used) {
  HestonSim sim(s0, v0, mu, kappa, theta, xi, rho, t, steps, scheme, seed);
  run_sim(sim, n_paths, steps + 1, threads, gather, out, used);
}

ORACLE_API void oracle_merton(double s0, double mu, double sigma, double lambda, double mu_j, double sigma_j, double t,
                   uint64_t steps, uint64_t n_paths, uint64_t seed, int threads, int gather, double* out,
                   uint64_t* used) {
  MertonSim sim(s0, mu, sigma, lambda, mu_j, sigma_j, t, steps, seed);
  run_sim(sim, n_paths, steps + 1, threads, gather, out, used);
}

// ---------------------------------------------------------------- LSMC ---
namespace {

inline double intrinsic(double s, double k, bool is_put) {  // lsmc.rs:117-123
  return is_put ? rmax(k - s, 0.0) : rmax(s - k, 0.0);
}

// Least squares min ||X c - y|| by Householder QR (column-major X, m x nc).
void lstsq_qr(std::vector<double>& X, std::vector<double>& y, int m, int nc, double* c) {
  for (int j = 0; j < nc; ++j) {
    double* col = &X[(size_t)j * m];
    double norm = 0.0;
    for (int i = j; i < m; ++i) norm += col[i] * col[i];
    norm = std::sqrt(norm);
    if (norm == 0.0) continue;
    double alpha = col[j] > 0 ? -norm : norm;
    double v0 = col[j] - alpha;
    // v = [v0, col[j+1..]]; H = I - 2 v v^T / (v^T v)
    double vtv = v0 * v0;
    for (int i = j + 1; i < m; ++i) vtv += col[i] * col[i];
    auto apply = [&](double* w) {
      double d = v0 * w[j];
      for (int i = j + 1; i < m; ++i) d += col[i] * w[i];
      double f = 2.0 * d / vtv;
      w[j] -= f * v0;
      for (int i = j + 1; i < m; ++i) w[i] -= f * col[i];
    };
    for (int jj = j + 1; jj < nc; ++jj) apply(&X[(size_t)jj * m]);
    apply(y.data());
    col[j] = alpha;
  }
  for (int j = nc - 1; j >= 0; --j) {
    double acc = y[j];
    for (int jj = j + 1; jj < nc; ++jj) acc -= X[(size_t)jj * m + j] * c[jj];
    c[j] = acc / X[(size_t)j * m + j];
  }
}

// Normal equations (X^T X) c = X^T y by Cholesky, as the device sweep does.
void lstsq_normal(const std::vector<double>& X, const std::vector<double>& y, int m, int nc, double* c) {
  double G[25] = {0}, b[5] = {0}, L[25] = {0};
  for (int r = 0; r < m; ++r)
    for (int i = 0; i < nc; ++i) {
      double xi = X[(size_t)i * m + r];
      b[i] += xi * y[r];
      for (int j = 0; j <= i; ++j) G[i * 5 + j] += xi * X[(size_t)j * m + r];
    }
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = G[i * 5 + j];
      for (int k = 0; k < j; ++k) s -= L[i * 5 + k] * L[j * 5 + k];
      L[i * 5 + j] = (i == j) ? std::sqrt(s) : s / L[j * 5 + j];
    }
  double w[5];
  for (int i = 0; i < nc; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * 5 + k] * w[k];
    w[i] = s / L[i * 5 + i];
  }
  for (int i = nc - 1; i >= 0; --i) {
    double s = w[i];
    for (int k = i + 1; k < nc; ++k) s -= L[k * 5 + i] * c[k];
    c[i] = s / L[i * 5 + i];
  }
}

}  // namespace

// src/finance/lsmc.rs:25-115.  solver: 0 = Householder QR (reference), 1 =
// normal equations.  paths (optional, n x (steps+1)) replaces the internal
// GBM draw so that a caller can feed the device's own paths.
ORACLE_API void oracle_lsmc(double s0, double k, double r, double sigma, double t, uint64_t steps, uint64_t n_paths,
                 int is_put, int poly_degree, uint64_t seed, int solver, int threads, const double* paths_in,
                 double* price, double* std_err) {
  const double dt = t / (double)steps;
  const double discount = std::exp(-r * dt);
  const uint64_t n = n_paths, len = steps + 1;
  std::vector<double> own;
  const double* paths = paths_in;
  if (!paths) {
    own.resize(n * len);
    oracle_gbm(s0, r, sigma, 0.0, t, steps, n, 0, seed, threads, 0, own.data(), nullptr);
    paths = own.data();
  }
  std::vector<double> cashflow(n);
  for (uint64_t i = 0; i < n; ++i) cashflow[i] = intrinsic(paths[i * len + steps], k, is_put);
  const int ncols = poly_degree + 1;
  std::vector<uint64_t> itm;
  std::vector<double> X, y;
  for (uint64_t step = steps - 1; step >= 1; --step) {
    for (auto& cf : cashflow) cf *= discount;
    itm.clear();
    for (uint64_t i = 0; i < n; ++i)
      if (intrinsic(paths[i * len + step], k, is_put) > 0.0) itm.push_back(i);
    if (itm.size() < (size_t)ncols + 1) continue;
    double s_mean = 0.0;
    for (uint64_t i : itm) s_mean += paths[i * len + step];
    s_mean /= (double)itm.size();
    double v = 0.0;
    for (uint64_t i : itm) v += powi(paths[i * len + step] - s_mean, 2);
    v /= (double)itm.size();
    double s_std = rmax(std::sqrt(v), 1e-12);
    const int m = (int)itm.size();
    X.assign((size_t)m * ncols, 0.0);
    y.assign(m, 0.0);
    for (int row = 0; row < m; ++row) {
      double x = (paths[itm[row] * len + step] - s_mean) / s_std;
      for (int col = 0; col < ncols; ++col) X[(size_t)col * m + row] = powi(x, col);
      y[row] = cashflow[itm[row]];
    }
    double coeffs[5] = {0};
    if (solver == 0)
      lstsq_qr(X, y, m, ncols, coeffs);
    else
      lstsq_normal(X, y, m, ncols, coeffs);
    for (uint64_t i : itm) {
      double sp = paths[i * len + step];
      double x = (sp - s_mean) / s_std;
      double cont = 0.0;
      for (int col = 0; col < ncols; ++col) cont += coeffs[col] * powi(x, col);
      double ex = intrinsic(sp, k, is_put);
      if (ex > rmax(cont, 0.0)) cashflow[i] = ex;
    }
  }
  for (auto& cf : cashflow) cf *= discount;
  double mean = 0.0;
  for (double c : cashflow) mean += c;
  mean /= (double)n;
  double se = 0.0;
  if (n > 1) {
    double var = 0.0;
    for (double c : cashflow) var += powi(c - mean, 2);
    var /= (double)(n - 1);
    se = std::sqrt(var / (double)n);
  }
  *price = mean;
  *std_err = se;
}

// -------------------------------------------------------------- Greeks ---
// src/finance/greeks.rs.  model: 0 gbm, 1 heston, 2 merton.
// p[11] = {s0, mu(=r), sigma, t, v0, kappa, theta, xi, rho, lambda, mu_j,
// sigma_j} minus one: index map below.  Heston's "Sigma" bump moves v0
// (greeks.rs:178, :214).
enum { P_S0 = 0, P_MU, P_SIGMA, P_T, P_V0, P_KAPPA, P_THETA, P_XI, P_RHO, P_LAMBDA, P_MUJ, P_SIGJ, P_COUNT };

// greeks.rs:91-167: terminal prices of one scenario.
ORACLE_API void oracle_terminal(int model, const double* p, int scheme, uint64_t steps, uint64_t n_paths, uint64_t seed,
                     int threads, double* terminal) {
  const uint64_t len = steps + 1;
  if (model == 0) {
    GbmSim sim(p[P_S0], p[P_MU], p[P_SIGMA], 0.0, p[P_T], steps, n_paths, 0, seed);
    run_terminal(sim, n_paths, len, threads, terminal);
  } else if (model == 1) {
    HestonSim sim(p[P_S0], p[P_V0], p[P_MU], p[P_KAPPA], p[P_THETA], p[P_XI], p[P_RHO], p[P_T], steps, scheme,
                  seed);
    run_terminal(sim, n_paths, len, threads, terminal);
  } else {
    MertonSim sim(p[P_S0], p[P_MU], p[P_SIGMA], p[P_LAMBDA], p[P_MUJ], p[P_SIGJ], p[P_T], steps, seed);
    run_terminal(sim, n_paths, len, threads, terminal);
  }
}

// greeks.rs:313-320 (mc_price).  payoff: 0 call, 1 put (greeks.rs:12-18).
ORACLE_API double oracle_mc_price(int model, const double* p, int scheme, int payoff, double strike, uint64_t steps,
                       uint64_t n_paths, uint64_t seed, int threads) {
  std::vector<double> term(n_paths);
  oracle_terminal(model, p, scheme, steps, n_paths, seed, threads, term.data());
  double sum = 0.0;
  for (double s : term) sum += payoff == 0 ? rmax(s - strike, 0.0) : rmax(strike - s, 0.0);
  double discount = std::exp(-p[P_MU] * p[P_T]);
  return discount * sum / (double)n_paths;
}

// greeks.rs:322-358 (greeks_fd_core) with required_scenarios (:231-265),
// compute_bump (:227-229) and compute_greeks_from_prices (:267-311).
// greeks: codes 0 delta, 1 gamma, 2 vega, 3 theta, 4 rho; out[i] per request.
ORACLE_API void oracle_greeks_fd(int model, const double* p_in, int scheme, int payoff, double strike, uint64_t n_paths,
                      uint64_t steps, const int* greeks, int n_greeks, uint64_t seed, double bump_size,
                      int threads, double* out) {
  // bump parameters: 0 S0, 1 Sigma (v0 for Heston), 2 T, 3 Mu
  auto pidx = [&](int bp) {
    if (bp == 0) return (int)P_S0;
    if (bp == 1) return model == 1 ? (int)P_V0 : (int)P_SIGMA;
    if (bp == 2) return (int)P_T;
    return (int)P_MU;
  };
  double h[4];
  for (int bp = 0; bp < 4; ++bp) h[bp] = rmax(std::fabs(p_in[pidx(bp)]) * bump_size, 1e-8);
  // scenario price cache: key = -1 base, else bp*2 + (down ? 1 : 0)
  double cache[9] = {0};
  bool have[9] = {false};
  auto price = [&](int bp, int down) {
    int key = bp < 0 ? 8 : bp * 2 + down;
    if (!have[key]) {
      double p[P_COUNT];
      std::memcpy(p, p_in, sizeof p);
      if (bp >= 0) p[pidx(bp)] += down ? -h[bp] : h[bp];
      cache[key] = oracle_mc_price(model, p, scheme, payoff, strike, steps, n_paths, seed, threads);
      have[key] = true;
    }
    return cache[key];
  };
  for (int gi = 0; gi < n_greeks; ++gi) {
    switch (greeks[gi]) {
      case 0:
        out[gi] = (price(0, 0) - price(0, 1)) / (2.0 * h[0]);
        break;
      case 1:
        out[gi] = (price(0, 0) - 2.0 * price(-1, 0) + price(0, 1)) / (h[0] * h[0]);
        break;
      case 2:
        out[gi] = (price(1, 0) - price(1, 1)) / (2.0 * h[1]);
        break;
      case 3:
        out[gi] = (price(2, 1) - price(-1, 0)) / h[2];
        break;
      default:
        out[gi] = (price(3, 0) - price(3, 1)) / (2.0 * h[3]);
        break;
    }
  }
}

// greeks.rs:360-424 (greeks_pathwise_core), GBM only; greeks: 0 delta, 2 vega.
ORACLE_API void oracle_greeks_pathwise(double s0, double r, double sigma, double t, double strike, int is_call,
                            uint64_t n_paths, uint64_t steps, const int* greeks, int n_greeks, uint64_t seed,
                            int threads, double* out) {
  double p[P_COUNT] = {0};
  p[P_S0] = s0;
  p[P_MU] = r;
  p[P_SIGMA] = sigma;
  p[P_T] = t;
  std::vector<double> term(n_paths);
  oracle_terminal(0, p, 0, steps, n_paths, seed, threads, term.data());
  const double discount = std::exp(-r * t);
  const double n = (double)n_paths;
  for (int gi = 0; gi < n_greeks; ++gi) {
    double sum = 0.0;
    for (double s_t : term) {
      bool in_money = is_call ? s_t > strike : s_t < strike;
      double sign = is_call ? 1.0 : -1.0;
      if (greeks[gi] == 0) {
        sum += in_money ? sign * s_t / s0 : 0.0;
      } else {
        double log_return = std::log(s_t / s0);
        sum += in_money ? sign * s_t * (log_return - (r + 0.5 * sigma * sigma) * t) / sigma : 0.0;
      }
    }
    out[gi] = (greeks[gi] == 0 || greeks[gi] == 2) ? discount * sum / n : NAN;
  }
}


// ------------------------------------------------------ exotic MC -------
// src/finance/barrier.rs:286-372 (barrier_mc, rebate_path_pv), asian.rs:143-290
// and 292-352 (asian_mc, asian_mc_floating_seasoned), lookback.rs:158-210
// (lookback_mc).  Per path: Pcg64Dxsm::new(seed) advanced by path * block,
// block = (steps + 1024) * 2; GBM step s *= exp(drift + diffusion * z).
// The reference adds the per-chunk sums with a Rayon reduction; here the paths
// are added in order (the sums differ only in summation order).
namespace {

double rebate_path_pv(int kind_in, int at_hit, double rebate, double r, int hit_step, uint64_t steps, double dt) {
  const bool knocked = hit_step >= 0;  // barrier.rs:379-403
  if (!kind_in && at_hit) return knocked ? rebate * std::exp(-r * ((double)hit_step * dt)) : 0.0;
  if (!kind_in) return knocked ? rebate * std::exp(-r * ((double)steps * dt)) : 0.0;
  return knocked ? 0.0 : rebate * std::exp(-r * ((double)steps * dt));
}

inline double vanilla_intrinsic(double s, double k, int is_call) {
  return is_call ? std::max(s - k, 0.0) : std::max(k - s, 0.0);
}

}  // namespace

// direction: 0 up, 1 down; kind_in: 1 knock-in, 0 knock-out.
ORACLE_API double oracle_barrier_mc(double s0, double k, double r, double q, double sigma, double t, double barrier,
                                    int direction, int kind_in, int is_call, double rebate, int rebate_at_hit,
                                    uint64_t n_paths, uint64_t steps, uint64_t seed, int threads) {
  const double dt = t / (double)steps;
  const double drift = (r - q - 0.5 * sigma * sigma) * dt;
  const double diffusion = sigma * std::sqrt(dt);
  const double discount = std::exp(-r * t);
  const u128 block = ((u128)steps + 1024) * 2;
  const bool already_hit = direction == 0 ? s0 >= barrier : s0 <= barrier;
  std::vector<double> pay(n_paths);
  parallel_for(n_paths, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) {
      Pcg g = path_stream(seed, i, block);
      double s = s0;
      int hit = -1;
      if (already_hit) {
        hit = 0;
      } else {
        for (uint64_t st = 1; st <= steps; ++st) {
          const double z = zig_normal(g);
          s *= std::exp(drift + diffusion * z);
          if (direction == 0 ? s >= barrier : s <= barrier) {
            hit = (int)st;
            break;
          }
        }
      }
      const bool knocked = hit >= 0;
      if (knocked && kind_in && (uint64_t)hit < steps)
        for (uint64_t st = (uint64_t)hit; st < steps; ++st) {
          const double z = zig_normal(g);
          s *= std::exp(drift + diffusion * z);
        }
      const double opt = kind_in ? (knocked ? vanilla_intrinsic(s, k, is_call) : 0.0)
                                 : (knocked ? 0.0 : vanilla_intrinsic(s, k, is_call));
      const double rpv = rebate == 0.0 ? 0.0 : rebate_path_pv(kind_in, rebate_at_hit, rebate, r, hit, steps, dt);
      pay[i] = opt + rpv / discount;
    }
  });
  double total = 0.0;
  for (double v : pay) total += v;
  return discount * total / (double)n_paths;
}

// Per-path (arithmetic, geometric) payoffs of asian_mc (asian.rs:225-268):
// fixed (strike_floating = 0) or floating strike, call or put.
ORACLE_API void oracle_asian_paths(double s0, double k, double r, double q, double sigma, double t, uint64_t steps,
                                   int strike_floating, int is_call, uint64_t n_paths, uint64_t seed, int threads,
                                   double* arith, double* geo) {
  const double dt = t / (double)steps;
  const double drift = (r - q - 0.5 * sigma * sigma) * dt;
  const double diffusion = sigma * std::sqrt(dt);
  const u128 block = ((u128)steps + 1024) * 2;
  parallel_for(n_paths, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) {
      Pcg g = path_stream(seed, i, block);
      double s = s0, sum_arith = 0.0, sum_log = 0.0;
      for (uint64_t st = 0; st < steps; ++st) {
        const double z = zig_normal(g);
        s *= std::exp(drift + diffusion * z);
        sum_arith += s;
        sum_log += std::log(s);
      }
      const double avg_a = sum_arith / (double)steps;
      const double avg_g = std::exp(sum_log / (double)steps);
      if (!strike_floating) {
        arith[i] = is_call ? std::max(avg_a - k, 0.0) : std::max(k - avg_a, 0.0);
        geo[i] = is_call ? std::max(avg_g - k, 0.0) : std::max(k - avg_g, 0.0);
      } else {
        arith[i] = is_call ? std::max(s - avg_a, 0.0) : std::max(avg_a - s, 0.0);
        geo[i] = is_call ? std::max(s - avg_g, 0.0) : std::max(avg_g - s, 0.0);
      }
    }
  });
}

// asian_mc's estimator (asian.rs:270-289): geometric control variate for the
// arithmetic fixed-strike case (use_cv), else the plain mean.
ORACLE_API double oracle_asian_estimate(const double* arith, const double* geo, uint64_t n, int use_cv,
                                        double geo_analytical, double discount) {
  if (use_cv && n > 1) {
    double ma = 0.0, mg = 0.0;
    for (uint64_t i = 0; i < n; ++i) ma += arith[i];
    ma /= (double)n;
    for (uint64_t i = 0; i < n; ++i) mg += geo[i];
    mg /= (double)n;
    double cov = 0.0, vg = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
      cov += (arith[i] - ma) * (geo[i] - mg);
      vg += (geo[i] - mg) * (geo[i] - mg);
    }
    const double beta = vg > 1e-30 ? cov / vg : 0.0;
    const double geo_mc = discount * mg;
    return std::max(discount * ma - beta * (geo_mc - geo_analytical), 0.0);
  }
  double m = 0.0;
  for (uint64_t i = 0; i < n; ++i) m += arith[i];
  return std::max(discount * (m / (double)n), 0.0);
}

// asian_mc_floating_seasoned (asian.rs:292-352): remaining-period paths with
// the spent average blended in; geometric = 1 for the geometric average.
ORACLE_API double oracle_asian_floating_seasoned(double s0, double r, double q, double sigma, double t, uint64_t n_steps,
                                                 int geometric, int is_call, double a_spent, double t1,
                                                 uint64_t n_paths, uint64_t seed, int threads) {
  const double remaining = t - t1;
  uint64_t nr = (uint64_t)std::llround((double)n_steps * remaining / t);
  if (nr < 1) nr = 1;
  const double dt = remaining / (double)nr;
  const double drift = (r - q - 0.5 * sigma * sigma) * dt;
  const double diffusion = sigma * std::sqrt(dt);
  const double discount = std::exp(-r * remaining);
  const double w_spent = t1 / t, w_remain = remaining / t;
  const u128 block = ((u128)nr + 1024) * 2;
  std::vector<double> pay(n_paths);
  parallel_for(n_paths, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) {
      Pcg g = path_stream(seed, i, block);
      double s = s0, sum_arith = 0.0, sum_log = 0.0;
      for (uint64_t st = 0; st < nr; ++st) {
        const double z = zig_normal(g);
        s *= std::exp(drift + diffusion * z);
        sum_arith += s;
        sum_log += std::log(s);
      }
      const double avg_rem = geometric ? std::exp(sum_log / (double)nr) : sum_arith / (double)nr;
      const double avg_t = geometric ? std::exp(std::log(a_spent) * w_spent + std::log(avg_rem) * w_remain)
                                     : w_spent * a_spent + w_remain * avg_rem;
      pay[i] = is_call ? std::max(s - avg_t, 0.0) : std::max(avg_t - s, 0.0);
    }
  });
  double total = 0.0;
  for (double v : pay) total += v;
  return discount * total / (double)n_paths;
}

// lookback_mc (lookback.rs:158-210); running_max / running_min: NaN = none.
ORACLE_API double oracle_lookback_mc(double s0, double k, double r, double q, double sigma, double t, uint64_t steps,
                                     int strike_fixed, int is_call, double running_max, double running_min,
                                     uint64_t n_paths, uint64_t seed, int threads) {
  const double dt = t / (double)steps;
  const double drift = (r - q - 0.5 * sigma * sigma) * dt;
  const double diffusion = sigma * std::sqrt(dt);
  const double discount = std::exp(-r * t);
  const u128 block = ((u128)steps + 1024) * 2;
  const double m0 = std::max(std::isnan(running_max) ? s0 : running_max, s0);
  const double n0 = std::min(std::isnan(running_min) ? s0 : running_min, s0);
  std::vector<double> pay(n_paths);
  parallel_for(n_paths, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) {
      Pcg g = path_stream(seed, i, block);
      double s = s0, mx = m0, mn = n0;
      for (uint64_t st = 0; st < steps; ++st) {
        const double z = zig_normal(g);
        s *= std::exp(drift + diffusion * z);
        if (s > mx) mx = s;
        if (s < mn) mn = s;
      }
      if (!strike_fixed)
        pay[i] = is_call ? s - mn : mx - s;
      else
        pay[i] = is_call ? std::max(mx - k, 0.0) : std::max(k - mn, 0.0);
    }
  });
  double total = 0.0;
  for (double v : pay) total += v;
  return discount * total / (double)n_paths;
}

// hull_white.rs:26-57: exact-transition short-rate paths, one stream per path
// with block (steps + 1024) * 4.
ORACLE_API void oracle_hull_white(double r0, double a, double theta, double sigma, double t, uint64_t steps,
                                  uint64_t n_paths, uint64_t seed, int threads, double* out) {
  const double dt = t / (double)steps;
  const double e = std::exp(-a * dt);
  const double mean_reversion = (theta / a) * (1.0 - e);
  const double vol = sigma * std::sqrt((1.0 - e * e) / (2.0 * a));
  const u128 block = ((u128)steps + 1024) * 4;
  const uint64_t len = steps + 1;
  parallel_for(n_paths, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      Pcg g = path_stream(seed, i, block);
      double* row = out + i * len;
      row[0] = r0;
      for (uint64_t s = 0; s < steps; ++s) {
        const double z = zig_normal(g);
        row[s + 1] = row[s] * e + mean_reversion + vol * z;
      }
    }
  });
}

// var_cvar.rs:7-43: losses = -returns sorted by total_cmp; VaR = losses[idx],
// idx = min(ceil(confidence * n), n - 1); CVaR = mean of losses[idx..].
ORACLE_API void oracle_var_cvar(const double* returns, uint64_t n, double confidence, double* out2) {
  std::vector<double> losses(n);
  for (uint64_t i = 0; i < n; ++i) losses[i] = -returns[i];
  auto key = [](double v) {
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
  };
  std::sort(losses.begin(), losses.end(), [&](double a, double b) { return key(a) < key(b); });
  uint64_t idx = (uint64_t)std::ceil(confidence * (double)n);
  if (idx > n - 1) idx = n - 1;
  double s = 0.0;
  for (uint64_t i = idx; i < n; ++i) s += losses[i];
  out2[0] = losses[idx];
  out2[1] = s / (double)(n - idx);
}

// copula/gaussian.rs:15-73 with dist/normal_cdf.rs:3-22: one sequential
// stream; sample i takes the next dim normals; x = L z; u = Phi(x).
ORACLE_API int oracle_gaussian_copula(const double* corr, int dim, uint64_t n, uint64_t seed, double* out) {
  std::vector<double> l((size_t)dim * dim, 0.0);
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j <= i; ++j) {
      double sum = corr[i * dim + j];
      for (int k = 0; k < j; ++k) sum -= l[i * dim + k] * l[j * dim + k];
      if (i == j) {
        if (sum <= 0.0) return -1;
        l[i * dim + j] = std::sqrt(sum);
      } else {
        l[i * dim + j] = sum / l[j * dim + j];
      }
    }
  Pcg g = Pcg::seeded((u128)seed);
  std::vector<double> z(dim);
  const double sqrt_2pi = std::sqrt(2.0 * M_PI);
  for (uint64_t i = 0; i < n; ++i) {
    for (int j = 0; j < dim; ++j) z[j] = zig_normal(g);
    for (int j = 0; j < dim; ++j) {
      double x = 0.0;
      for (int k = 0; k <= j; ++k) x += l[j * dim + k] * z[k];
      const double t = 1.0 / (1.0 + 0.2316419 * std::fabs(x));
      const double poly =
          t * (0.319381530 + t * (-0.356563782 + t * (1.781477937 + t * (-1.821255978 + t * 1.330274429))));
      const double pdf = std::exp(-0.5 * x * x) / sqrt_2pi;
      const double cdf_pos = 1.0 - pdf * poly;
      out[i * dim + j] = x >= 0.0 ? cdf_pos : 1.0 - cdf_pos;
    }
  }
  return 0;
}

// copula/student_t.rs:6-170: one sequential stream; per sample chi-square(nu)
// by Marsaglia-Tsang gamma, then dim normals; u = T_nu((L z)_j sqrt(nu/chi2)).
namespace {

double st_lgamma(double x) {  // student_t.rs:74-91 (Lanczos g = 7)
  static const double C[9] = {0.99999999999980993,  676.5203681218851,     -1259.1392167224028,
                              771.32342877765313,   -176.61502916214059,   12.507343278686905,
                              -0.13857109526572012, 9.9843695780195716e-6, 1.5056327351493116e-7};
  if (x < 0.5) return std::log(M_PI) - std::log(std::sin(M_PI * x)) - st_lgamma(1.0 - x);
  x -= 1.0;
  double acc = C[0];
  for (int i = 1; i < 9; ++i) acc += C[i] / (x + (double)i);
  const double t = x + 7.0 + 0.5;
  return 0.5 * std::log(2.0 * M_PI) + (x + 0.5) * std::log(t) - t + std::log(acc);
}

double st_beta_cf(double x, double a, double b) {  // student_t.rs:33-72
  const double EPS = 3e-7, FPMIN = 1e-30;
  const double qab = a + b, qap = a + 1.0, qam = a - 1.0;
  double c = 1.0, d = std::max(1.0 - qab * x / qap, FPMIN);
  d = 1.0 / d;
  double h = d;
  for (int m = 1; m <= 200; ++m) {
    const double mf = m, m2 = 2.0 * mf;
    double aa = mf * (b - mf) * x / ((qam + m2) * (a + m2));
    d = std::max(std::fabs(1.0 + aa * d), FPMIN);
    c = std::max(std::fabs(1.0 + aa / c), FPMIN);
    d = 1.0 / d;
    h *= d * c;
    aa = -(a + mf) * (qab + mf) * x / ((a + m2) * (qap + m2));
    d = std::max(std::fabs(1.0 + aa * d), FPMIN);
    c = std::max(std::fabs(1.0 + aa / c), FPMIN);
    d = 1.0 / d;
    const double del = d * c;
    h *= del;
    if (std::fabs(del - 1.0) < EPS) break;
  }
  return h;
}

double st_ibeta(double x, double a, double b) {  // student_t.rs:19-31
  if (x <= 0.0) return 0.0;
  if (x >= 1.0) return 1.0;
  if (x > (a + 1.0) / (a + b + 2.0)) return 1.0 - st_ibeta(1.0 - x, b, a);
  const double lb = st_lgamma(a) + st_lgamma(b) - st_lgamma(a + b);
  const double front = std::exp(a * std::log(x) + b * std::log(1.0 - x) - lb) / a;
  return front * st_beta_cf(x, a, b);
}

double st_gamma(Pcg& g, double shape) {  // student_t.rs:93-119
  const double d = shape - 1.0 / 3.0;
  const double c = 1.0 / std::sqrt(9.0 * d);
  for (;;) {
    const double x = zig_normal(g);
    const double v_inner = 1.0 + c * x;
    if (v_inner <= 0.0) continue;
    const double v = v_inner * v_inner * v_inner;
    const double u = g.next_f64();
    if (u < 1.0 - 0.0331 * (x * x) * (x * x)) return d * v;
    if (std::log(u) < 0.5 * x * x + d * (1.0 - v + std::log(v))) return d * v;
  }
}

}  // namespace

ORACLE_API int oracle_student_t_copula(const double* corr, int dim, double nu, uint64_t n, uint64_t seed,
                                       double* out) {
  std::vector<double> l((size_t)dim * dim, 0.0);
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j <= i; ++j) {
      double sum = corr[i * dim + j];
      for (int k = 0; k < j; ++k) sum -= l[i * dim + k] * l[j * dim + k];
      if (i == j) {
        if (sum <= 0.0) return -1;
        l[i * dim + j] = std::sqrt(sum);
      } else {
        l[i * dim + j] = sum / l[j * dim + j];
      }
    }
  Pcg g = Pcg::seeded((u128)seed);
  std::vector<double> z(dim);
  for (uint64_t i = 0; i < n; ++i) {
    const double chi = 2.0 * st_gamma(g, nu / 2.0);
    const double scale = std::sqrt(nu / chi);
    for (int j = 0; j < dim; ++j) z[j] = zig_normal(g);
    for (int j = 0; j < dim; ++j) {
      double x = 0.0;
      for (int k = 0; k <= j; ++k) x += l[j * dim + k] * z[k];
      const double xs = x * scale;
      const double ib = st_ibeta(nu / (nu + xs * xs), nu / 2.0, 0.5);
      out[i * dim + j] = xs >= 0.0 ? 1.0 - 0.5 * ib : 0.5 * ib;
    }
  }
  return 0;
}

ORACLE_API double oracle_student_t_cdf(double x, double nu) {  // student_t.rs:8-16
  const double ib = st_ibeta(nu / (nu + x * x), nu / 2.0, 0.5);
  return x >= 0.0 ? 1.0 - 0.5 * ib : 0.5 * ib;
}
