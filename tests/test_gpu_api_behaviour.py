"""The reference's behavioural assertions, run against the device through the
drop-in API.

The parity tests pin the device output to the oracle value by value; this file
checks, on the same functions, the properties the reference's own test suite
asserts of its results, with the same sizes, seeds and tolerances:

  * tests/test_models.py  TestGBM, TestHeston, TestHestonQE, TestMertonJumpDiffusion,
                          TestHullWhite, TestHullWhiteZcb, TestMultiGBM,
                          TestLsmcAmericanOption
  * tests/test_rng.py     TestRNG, TestStandardNormal

so that a user moving from the reference finds the same guarantees.  The
argument-validation cases of those classes need no GPU and sit in
test_abi.py (exact messages).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_S = 100.0 * math.exp(0.05)  # E[S(T)] = s0 e^(mu T) for s0 = 100, mu = 0.05, T = 1


def _norm_cdf(x):
    return 0.5 * (1.0 + math.erf(x / math.sqrt(2.0)))


def _bs_put(s, k, r, sigma, t):
    d1 = (math.log(s / k) + (r + 0.5 * sigma * sigma) * t) / (sigma * math.sqrt(t))
    d2 = d1 - sigma * math.sqrt(t)
    return k * math.exp(-r * t) * _norm_cdf(-d2) - s * _norm_cdf(-d1)


def _sample_corr(paths):
    """Correlation of the two assets' one-step log-returns over all steps."""
    lr = np.log(paths[:, 1:, :] / paths[:, :-1, :]).reshape(-1, 2)
    return float(np.corrcoef(lr.T)[0, 1])


# ------------------------------------------------------------ single-asset --
HESTON = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0, steps=252, seed=42)
MERTON = dict(s0=100.0, mu=0.05, sigma=0.2, lambda_=1.0, mu_j=-0.05, sigma_j=0.1, t=1.0, steps=252, seed=42)

# (name, call(n_paths), n_paths of the expectation run, relative tolerance of E[S(T)])
MODELS = [
    ("gbm", lambda s, n: s.gbm(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=n, seed=0), 100_000, 5e-3),
    ("heston", lambda s, n: s.heston(**HESTON, n_paths=n), 100_000, 2e-2),
    ("heston_qe", lambda s, n: s.heston(**HESTON, n_paths=n, scheme="qe"), 100_000, 2e-2),
    ("merton", lambda s, n: s.merton_jump_diffusion(**MERTON, n_paths=n), 200_000, 2e-2),
]


@pytest.mark.parametrize("name,fn,n_big,rtol", MODELS, ids=[m[0] for m in MODELS])
def test_shape_start_positivity_reproducibility(stocha, name, fn, n_big, rtol):
    """test_output_shape, test_initial_price, test_positive_prices, test_reproducibility
    (test_models.py:32-47, 95-111, 145-156, 194-212)."""
    a = fn(stocha, 1000)
    assert a.shape == (1000, 253) and a.dtype == np.float64 and a.flags.c_contiguous
    np.testing.assert_array_equal(a[:, 0], 100.0)
    assert (a > 0).all()
    np.testing.assert_array_equal(a, fn(stocha, 1000))


@pytest.mark.parametrize("name,fn,n_big,rtol", MODELS, ids=[m[0] for m in MODELS])
def test_expected_terminal_price(stocha, name, fn, n_big, rtol):
    """E[S(T)] = s0 e^(mu T) for GBM, Heston (both schemes) and Merton with its
    compensator (test_models.py:48-54, 112-117, 157-161, 214-219)."""
    p = fn(stocha, n_big)
    assert p[:, -1].mean() == pytest.approx(E_S, rel=rtol)


def test_gbm_positive_at_higher_vol_and_antithetic_variance(stocha):
    """test_positive_prices at sigma 0.3 and test_antithetic_reduces_variance (test_models.py:56-66)."""
    assert (stocha.gbm(s0=100.0, mu=0.05, sigma=0.3, t=1.0, steps=252, n_paths=10_000, seed=0) > 0).all()
    kw = dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=50_000, seed=42)
    plain = stocha.gbm(**kw, antithetic=False)
    anti = stocha.gbm(**kw, antithetic=True)
    assert anti[:, -1].std() < plain[:, -1].std()


def test_heston_qe_feller_violated_and_euler_default(stocha):
    """test_feller_violated_stability (2 kappa theta < xi^2 is fine for QE) and
    test_euler_default_backward_compat (test_models.py:163-181)."""
    p = stocha.heston(s0=100.0, v0=0.04, mu=0.05, kappa=1.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0, steps=252,
                      n_paths=5000, seed=77, scheme="qe")
    assert p.shape == (5000, 253) and (p > 0).all()
    kw = dict(HESTON, steps=50, n_paths=10)
    np.testing.assert_array_equal(stocha.heston(**kw), stocha.heston(**kw, scheme="euler"))


# -------------------------------------------------------------- multi-GBM --
CORR2 = np.array([[1.0, 0.6], [0.6, 1.0]])
CORR3 = np.array([[1.0, 0.6, 0.3], [0.6, 1.0, 0.5], [0.3, 0.5, 1.0]])
TWO = dict(s0=[100.0, 50.0], mu=[0.05, 0.08], sigma=[0.2, 0.3], corr=CORR2, t=1.0, steps=252)
THREE = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15], corr=CORR3, t=1.0)


def test_multi_gbm_shapes_start_positivity_reproducibility(stocha):
    """TestMultiGBM test_output_shape, test_three_assets, test_initial_prices,
    test_positive_prices, test_reproducibility, test_antithetic_shape (test_models.py:628-663, 690-696)."""
    a = stocha.multi_gbm(**TWO, n_paths=1000, seed=42)
    assert a.shape == (1000, 253, 2) and a.dtype == np.float64
    np.testing.assert_array_equal(a, stocha.multi_gbm(**TWO, n_paths=1000, seed=42))
    assert stocha.multi_gbm(**THREE, steps=252, n_paths=500, seed=0).shape == (500, 253, 3)
    b = stocha.multi_gbm(**THREE, steps=10, n_paths=100, seed=0)
    for i, s0 in enumerate(THREE["s0"]):
        np.testing.assert_array_equal(b[:, 0, i], s0)
    assert (stocha.multi_gbm(**TWO, n_paths=10_000, seed=0) > 0).all()
    assert stocha.multi_gbm(**TWO, n_paths=1000, seed=42, antithetic=True).shape == (1000, 253, 2)


def test_multi_gbm_moments_and_correlation(stocha):
    """test_expected_terminal_prices (each asset within 2 %) and
    test_correlation_structure (sample correlation of log-returns within 0.05 of 0.6)
    (test_models.py:665-688)."""
    p = stocha.multi_gbm(**TWO, n_paths=100_000, seed=0)
    for i in range(2):
        want = TWO["s0"][i] * math.exp(TWO["mu"][i])
        assert abs(p[:, -1, i].mean() - want) / want < 0.02
    c = _sample_corr(stocha.multi_gbm(**TWO, n_paths=50_000, seed=0))
    assert abs(c - 0.6) < 0.05, c


def test_multi_gbm_antithetic_portfolio_and_uncorrelated(stocha):
    """test_antithetic_reduces_variance (equal-weight portfolio) and
    test_uncorrelated_assets (|corr| < 0.02 with corr = I) (test_models.py:698-717)."""
    plain = stocha.multi_gbm(**TWO, n_paths=50_000, seed=42, antithetic=False)
    anti = stocha.multi_gbm(**TWO, n_paths=50_000, seed=42, antithetic=True)
    assert anti[:, -1, :].sum(axis=1).std() < plain[:, -1, :].sum(axis=1).std()
    u = stocha.multi_gbm(s0=[100.0, 100.0], mu=[0.05, 0.05], sigma=[0.2, 0.2], corr=np.eye(2), t=1.0, steps=252,
                         n_paths=50_000, seed=0)
    assert abs(_sample_corr(u)) < 0.02


# ------------------------------------------------------------- Hull-White --
def _vasicek_zcb(r0, a, theta, sigma, T):
    """P(0, T) of dr = (theta - a r) dt + sigma dW in closed form (Vasicek)."""
    B = (1.0 - math.exp(-a * T)) / a
    b = theta / a
    return math.exp((b - sigma * sigma / (2.0 * a * a)) * (B - T) - sigma * sigma * B * B / (4.0 * a) - B * r0)


def test_hull_white_shape_start_mean_reversion(stocha):
    """TestHullWhite test_shape, test_initial_rate, test_mean_reversion (test_models.py:368-393)."""
    r = stocha.hull_white(r0=0.05, a=0.1, theta=0.005, sigma=0.01, t=1.0, steps=12, n_paths=100)
    assert r.shape == (100, 13)
    r = stocha.hull_white(r0=0.05, a=0.1, theta=0.005, sigma=0.01, t=1.0, steps=12, n_paths=500)
    np.testing.assert_allclose(r[:, 0], 0.05)
    r = stocha.hull_white(r0=0.10, a=1.0, theta=0.05, sigma=0.001, t=10.0, steps=100, n_paths=2000, seed=0)
    assert abs(r[:, -1].mean() - 0.05) < 0.01


@pytest.mark.parametrize("r0,a,theta,sigma,T", [
    (0.03, 0.10, 0.005, 0.010, 1.0), (0.03, 0.10, 0.005, 0.010, 5.0), (0.03, 0.10, 0.005, 0.010, 10.0),
    (0.03, 0.05, 0.0025, 0.010, 5.0), (0.03, 0.50, 0.025, 0.010, 5.0), (0.03, 0.10, 0.005, 0.003, 5.0),
    (0.03, 0.10, 0.005, 0.020, 5.0), (-0.01, 0.10, 0.005, 0.010, 5.0), (0.08, 0.10, 0.002, 0.010, 5.0),
    (0.01, 0.10, 0.008, 0.010, 5.0),
])
def test_hull_white_zcb_matches_vasicek(stocha, r0, a, theta, sigma, T):
    """TestHullWhiteZcb: the trapezoid-discounted mean over 5e4 paths at dt ~ 0.02
    prices P(0, T) within atol 1.5e-3 / rtol 2e-3 of Vasicek (test_models.py:437-491)."""
    steps = max(50, int(252 * T / 5.0))
    paths = stocha.hull_white(r0=r0, a=a, theta=theta, sigma=sigma, t=T, steps=steps, n_paths=50_000, seed=42)
    dt = T / steps
    integral = dt * (paths[:, 1:-1].sum(axis=1) + 0.5 * (paths[:, 0] + paths[:, -1]))
    p_mc = float(np.exp(-integral).mean())
    assert p_mc == pytest.approx(_vasicek_zcb(r0, a, theta, sigma, T), abs=1.5e-3, rel=2e-3)


# ------------------------------------------------------------------- LSMC --
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_lsmc_reference_assertions(stocha, precision):
    """TestLsmcAmericanOption: types and signs, American >= European - 3 SE, the
    ATM benchmark (~6.07 within 0.30), deep ITM > 15, deep OTM < 2, a call > 0, and
    reproducibility (test_models.py:746-811).  Both precisions."""
    f = lambda **kw: stocha.lsmc_american_option(**kw, precision=precision)
    price, se = f(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=10, n_paths=1000)
    assert isinstance(price, float) and isinstance(se, float) and price > 0 and se > 0
    price, se = f(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=30_000, seed=0)
    assert price >= _bs_put(100.0, 100.0, 0.05, 0.20, 1.0) - 3 * se
    price, _ = f(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=50_000, seed=42)
    assert abs(price - 6.07) < 0.30
    assert f(s0=80.0, k=100.0, r=0.01, sigma=0.10, t=1.0, steps=50, n_paths=10_000)[0] > 15.0
    assert f(s0=150.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=10_000)[0] < 2.0
    assert f(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=20_000, is_put=False)[0] > 0
    kw = dict(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=5_000, seed=7)
    assert f(**kw)[0] == f(**kw)[0]


# -------------------------------------------------------------------- RNG --
def test_rng_reference_assertions(stocha):
    """TestRNG: uniform range and dtype, normal moments, loc/scale, same seed ->
    same draws, different seeds differ, save_state is JSON text, from_state at the
    start and mid-stream, the seed-only legacy format (test_rng.py:18-88)."""
    u = stocha.RNG(seed=0).uniform(size=10_000)
    assert u.dtype == np.float64 and u.min() >= 0.0 and u.max() < 1.0
    z = stocha.RNG(seed=42).normal(size=1_000_000)
    assert z.dtype == np.float64 and abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    y = stocha.RNG(seed=1).normal(size=100_000, loc=5.0, scale=2.0)
    assert y.mean() == pytest.approx(5.0, rel=1e-2) and y.std() == pytest.approx(2.0, rel=1e-2)
    np.testing.assert_array_equal(stocha.RNG(seed=99).normal(size=1_000), stocha.RNG(seed=99).normal(size=1_000))
    assert not np.array_equal(stocha.RNG(seed=1).normal(size=100), stocha.RNG(seed=2).normal(size=100))
    r = stocha.RNG(seed=7)
    r.uniform(size=100)
    js = r.save_state()
    assert isinstance(js, str) and len(js) > 0
    fresh = stocha.RNG.from_state(stocha.RNG(seed=123).save_state())
    np.testing.assert_array_equal(fresh.normal(size=50), stocha.RNG(seed=123).normal(size=50))
    r = stocha.RNG(seed=42)
    r.normal(size=500)
    js = r.save_state()
    want = r.normal(size=100)
    np.testing.assert_array_equal(stocha.RNG.from_state(js).normal(size=100), want)
    np.testing.assert_array_equal(stocha.RNG.from_state('{"seed":42}').normal(size=50),
                                  stocha.RNG(seed=42).normal(size=50))


def test_standard_normal_reference_assertions(stocha):
    """TestStandardNormal: shape and dtype, moments at 5e5, a KS test at 1e5 with
    p > 0.01, reproducibility (test_rng.py:92-119)."""
    stats = pytest.importorskip("scipy.stats")
    out = stocha.RNG(seed=0).standard_normal(size=10_000)
    assert out.shape == (10_000,) and out.dtype == np.float64
    out = stocha.RNG(seed=0).standard_normal(size=500_000)
    assert abs(out.mean()) < 0.005 and abs(out.std() - 1.0) < 0.01
    assert stats.kstest(stocha.RNG(seed=123).standard_normal(size=100_000), "norm").pvalue > 0.01
    np.testing.assert_array_equal(stocha.RNG(seed=42).standard_normal(size=1_000),
                                  stocha.RNG(seed=42).standard_normal(size=1_000))
