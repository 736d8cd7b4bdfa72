"""LSMC American option (src/finance/lsmc.rs) on the device.

* Paths are the FP64 GBM paths (identical to the oracle's to 1e-12); the
  device regression solves the normal equations, so against the oracle run
  with the same solver the price agrees to LSMC_SAME_SOLVER_RTOL, and against
  the oracle's Householder-QR solve (the reference's method) to
  LSMC_QR_RTOL (exercise decisions differ only at near-ties).
* The reference's own expectations (tests/test_models.py LSMC block),
  restated: the 6.07 benchmark, American >= European - 3 SE, deep ITM/OTM,
  call, reproducibility.
* FP32 paths with the FP64 regression: within FP32_RTOL of the FP64 form.
"""
import math

import pytest

pytestmark = pytest.mark.gpu

LSMC_SAME_SOLVER_RTOL = 1e-9
LSMC_QR_RTOL = 1e-6
FP32_RTOL = 1e-4


def _bs_put(s, k, r, sigma, t):
    N = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))
    d1 = (math.log(s / k) + (r + 0.5 * sigma**2) * t) / (sigma * math.sqrt(t))
    d2 = d1 - sigma * math.sqrt(t)
    return k * math.exp(-r * t) * N(-d2) - s * N(-d1)


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
@pytest.mark.parametrize("is_put", [True, False])
def test_lsmc_matches_oracle(stocha, oracle, deg, is_put):
    kw = dict(s0=100.0, k=100.0, r=0.05, sigma=0.2, t=1.0, steps=50, n_paths=20_000, is_put=is_put,
              poly_degree=deg, seed=42)
    p, se = stocha.lsmc_american_option(**kw)
    p_ne, se_ne = oracle.lsmc(*[kw[k] for k in ("s0", "k", "r", "sigma", "t", "steps", "n_paths")], is_put=is_put,
                              poly_degree=deg, seed=42, solver="normal")
    p_qr, _ = oracle.lsmc(*[kw[k] for k in ("s0", "k", "r", "sigma", "t", "steps", "n_paths")], is_put=is_put,
                          poly_degree=deg, seed=42, solver="qr")
    assert abs(p - p_ne) <= LSMC_SAME_SOLVER_RTOL * p_ne, (p, p_ne)
    assert abs(se - se_ne) <= 1e-8 * se_ne
    assert abs(p - p_qr) <= LSMC_QR_RTOL * p_qr, (p, p_qr)


def test_lsmc_reference_expectations(stocha):
    price, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.20, 1.0, 50, 50_000, seed=42)
    assert abs(price - 6.07) < 0.30
    price, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.20, 1.0, 50, 30_000, seed=0)
    assert price >= _bs_put(100, 100, 0.05, 0.2, 1.0) - 3 * se
    assert stocha.lsmc_american_option(80.0, 100.0, 0.01, 0.10, 1.0, 50, 10_000)[0] > 15.0
    assert stocha.lsmc_american_option(150.0, 100.0, 0.05, 0.20, 1.0, 50, 10_000)[0] < 2.0
    assert stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.20, 1.0, 50, 20_000, is_put=False)[0] > 0
    kw = dict(s0=100.0, k=100.0, r=0.05, sigma=0.20, t=1.0, steps=50, n_paths=5_000, seed=7)
    assert stocha.lsmc_american_option(**kw) == stocha.lsmc_american_option(**kw)
    p, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.20, 1.0, 10, 1000)
    assert isinstance(p, float) and isinstance(se, float) and p > 0 and se > 0


def test_lsmc_edges(stocha, oracle):
    # one step: no regression at all, only the terminal payoff discounted
    p, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.2, 1.0, 1, 1000, seed=3)
    pq, seq = oracle.lsmc(100.0, 100.0, 0.05, 0.2, 1.0, 1, 1000, seed=3)
    assert abs(p - pq) <= 1e-12 * pq and abs(se - seq) <= 1e-10 * seq
    # two paths: steps are skipped (fewer ITM paths than ncols + 1)
    p, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.2, 1.0, 5, 2, seed=3)
    pq, seq = oracle.lsmc(100.0, 100.0, 0.05, 0.2, 1.0, 5, 2, seed=3)
    assert abs(p - pq) <= 1e-12 * max(pq, 1e-12)


@pytest.mark.parametrize("n", [50_000, 4_000_000])
def test_lsmc_fp32_paths(stocha, n):
    """FP32 paths move a few exercise decisions at near-ties: the difference
    is a small fraction of one standard error, and within FP32_RTOL at the
    4e6-path size of the benchmark configuration."""
    kw = dict(s0=100.0, k=100.0, r=0.05, sigma=0.2, t=1.0, steps=50, n_paths=n, seed=42)
    p64, se64 = stocha.lsmc_american_option(**kw)
    p32, se32 = stocha.lsmc_american_option(**kw, precision="fp32")
    assert abs(p32 - p64) <= 0.1 * se64, (p32, p64, se64)
    if n >= 1_000_000:
        assert abs(p32 - p64) <= FP32_RTOL * p64, (p32, p64)
    assert abs(se32 - se64) <= 1e-3 * se64


@pytest.mark.parametrize("n,prec", [(600_000, "fp64"), (600_000, "fp32"), (30_000, "fp32")])
def test_lsmc_sweep_forms(stocha, oracle, n, prec):
    """Above 2^19 paths the sweep runs as one launch per step, below as one
    cluster launch: both against the oracle (FP64: same solver, LSMC_SAME_SOLVER_RTOL;
    FP32: a tenth of a standard error)."""
    kw = dict(s0=100.0, k=100.0, r=0.05, sigma=0.2, t=1.0, steps=50, n_paths=n, seed=11)
    p, se = stocha.lsmc_american_option(**kw, precision=prec)
    pq, seq = oracle.lsmc(100.0, 100.0, 0.05, 0.2, 1.0, 50, n, seed=11, solver="normal")
    if prec == "fp64":
        assert abs(p - pq) <= LSMC_SAME_SOLVER_RTOL * pq, (p, pq)
        assert abs(se - seq) <= 1e-8 * seq
    else:
        assert abs(p - pq) <= 0.1 * seq, (p, pq, seq)
