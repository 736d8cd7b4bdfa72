"""Monte Carlo Greeks (src/finance/greeks.rs) on the device.

* FP64 greeks_fd revalues every scenario with the reference's arithmetic:
  scenario prices equal the oracle's to summation order, so the Greeks agree
  to GREEK_FP64_RTOL (finite differences amplify the last-bit differences of
  the prices by value/(difference)).
* The reference's own expectations (tests/test_greeks.py), restated.
* FP32 common-random-number form against the FP64 form: the error of every
  Greek is reported and bounded by FP32_GREEK_RTOL (per Greek).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GREEK_FP64_RTOL = 1e-8
ALL = ["delta", "gamma", "vega", "theta", "rho"]
FP32_GREEK_RTOL = {"delta": 2e-4, "gamma": 5e-3, "vega": 2e-3, "theta": 2e-3, "rho": 2e-4}

GBM = {"s0": 100.0, "r": 0.05, "sigma": 0.2, "t": 1.0}
HESTON = {"s0": 100.0, "v0": 0.04, "r": 0.05, "kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "t": 1.0}
MERTON = {"s0": 100.0, "r": 0.05, "sigma": 0.2, "lambda_": 1.0, "mu_j": -0.05, "sigma_j": 0.1, "t": 1.0}


def _close(a, b, rtol, atol=1e-9):
    return abs(a - b) <= rtol * abs(b) + atol


@pytest.mark.parametrize("model,params", [("gbm", GBM), ("heston", HESTON), ("heston", dict(HESTON, scheme="qe")),
                                          ("merton", MERTON)])
@pytest.mark.parametrize("payoff", ["call", "put"])
def test_greeks_fd_matches_oracle(stocha, oracle, model, params, payoff):
    kw = dict(strike=100.0, n_paths=20_000, n_steps=52, greeks=ALL, seed=42)
    got = stocha.greeks_fd(model, params, payoff, **kw)
    want = oracle.greeks_fd(model, params, payoff, kw["strike"], kw["n_paths"], kw["n_steps"], ALL, seed=42)
    for g in ALL:
        assert _close(got[g], want[g], GREEK_FP64_RTOL), (g, got[g], want[g])


def test_tiny_bump_floor(stocha, oracle):
    # r = 0 -> the rho bump is the 1e-8 floor (greeks.rs:227-229)
    p = dict(GBM, r=0.0)
    got = stocha.greeks_fd("gbm", p, "call", 100.0, 5000, 12, ["rho", "delta"], seed=1)
    want = oracle.greeks_fd("gbm", p, "call", 100.0, 5000, 12, ["rho", "delta"], seed=1)
    assert _close(got["delta"], want["delta"], GREEK_FP64_RTOL)
    assert _close(got["rho"], want["rho"], 1e-5, atol=1e-3)  # a 1e-8 bump amplifies summation order 1e8x


def _bs(s, k, r, sig, t):
    N = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))
    n = lambda x: math.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)
    d1 = (math.log(s / k) + (r + 0.5 * sig * sig) * t) / (sig * math.sqrt(t))
    d2 = d1 - sig * math.sqrt(t)
    return {"delta": N(d1), "put_delta": N(d1) - 1, "gamma": n(d1) / (s * sig * math.sqrt(t)),
            "vega": s * n(d1) * math.sqrt(t),
            "theta": -s * n(d1) * sig / (2 * math.sqrt(t)) - r * k * math.exp(-r * t) * N(d2),
            "rho": k * t * math.exp(-r * t) * N(d2)}


def test_reference_expectations(stocha):
    bs = _bs(100, 100, 0.05, 0.2, 1.0)
    r = stocha.greeks_fd("gbm", GBM, "call", 100.0, 200_000, 252, ALL, seed=42)
    tol = {"delta": 0.02, "gamma": 0.005, "vega": 2.0, "theta": 1.0, "rho": 2.0}
    for g in ALL:
        assert abs(r[g] - bs[g]) < tol[g], (g, r[g], bs[g])
    assert set(r) == set(ALL) and 0 < r["delta"] < 1 and r["gamma"] > 0 and r["theta"] < 0
    put = stocha.greeks_fd("gbm", GBM, "put", 100.0, 200_000, 252, ["delta"], seed=42)
    assert abs(put["delta"] - bs["put_delta"]) < 0.02
    assert abs(r["delta"] - put["delta"] - 1.0) < 0.03
    pw = stocha.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, True, 200_000, 252, ["delta", "vega"], seed=42)
    assert abs(pw["delta"] - bs["delta"]) < 0.015 and abs(pw["vega"] - bs["vega"]) < 1.5
    assert abs(r["delta"] - pw["delta"]) < 0.03
    a = stocha.greeks_fd("gbm", GBM, "call", 100.0, 10_000, 50, ["delta", "vega"], seed=123)
    b = stocha.greeks_fd("gbm", GBM, "call", 100.0, 10_000, 50, ["delta", "vega"], seed=123)
    assert a == b
    h = stocha.greeks_fd("heston", HESTON, "call", 100.0, 50_000, 100, ["delta"], seed=42)
    m = stocha.greeks_fd("merton", MERTON, "call", 100.0, 50_000, 100, ["delta"], seed=42)
    assert 0 < h["delta"] < 1 and 0 < m["delta"] < 1


def test_callable_payoff_matches_builtin(stocha):
    calls = []

    def custom(terminals):
        calls.append(len(terminals))
        return np.maximum(terminals - 100.0, 0.0)

    a = stocha.greeks_fd("gbm", GBM, "call", 100.0, 50_000, 50, ["delta"], seed=42)
    b = stocha.greeks_fd("gbm", GBM, custom, 100.0, 50_000, 50, ["delta"], seed=42)
    assert abs(a["delta"] - b["delta"]) < 1e-10
    assert calls == [50_000, 50_000]  # one call per scenario (lib.rs:1134-1138)

    def boom(terminals):
        raise RuntimeError("payoff failed")

    with pytest.raises(RuntimeError, match="payoff failed"):
        stocha.greeks_fd("gbm", GBM, boom, 100.0, 100, 5, ["delta"])


@pytest.mark.parametrize("is_call", [True, False])
def test_pathwise_matches_oracle(stocha, oracle, is_call):
    got = stocha.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, is_call, 30_000, 52, ["delta", "vega"], seed=7)
    want = oracle.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, is_call, 30_000, 52, ["delta", "vega"], seed=7)
    for g in ("delta", "vega"):
        assert _close(got[g], want[g], 1e-10), (g, got[g], want[g])


@pytest.mark.parametrize("model,params", [("gbm", GBM), ("heston", HESTON), ("merton", MERTON)])
@pytest.mark.parametrize("payoff", ["call", "put"])
def test_fp32_greeks_against_fp64(stocha, model, params, payoff):
    kw = dict(strike=100.0, n_paths=200_000, n_steps=52, greeks=ALL, seed=42)
    g64 = stocha.greeks_fd(model, params, payoff, **kw)
    g32 = stocha.greeks_fd(model, params, payoff, **kw, precision="fp32")
    for g in ALL:
        assert _close(g32[g], g64[g], FP32_GREEK_RTOL[g], atol=1e-4), (model, payoff, g, g32[g], g64[g])


def test_fp32_rho_with_bump_floor(stocha):
    # r tiny: the 1e-8 rho bump would cancel catastrophically without the
    # per-path difference; the FP32 form must stay close to the FP64 one.
    p = dict(GBM, r=1e-9)
    g64 = stocha.greeks_fd("gbm", p, "call", 100.0, 100_000, 52, ["rho"], seed=5)
    g32 = stocha.greeks_fd("gbm", p, "call", 100.0, 100_000, 52, ["rho"], seed=5, precision="fp32")
    assert _close(g32["rho"], g64["rho"], 1e-3), (g32, g64)


def test_greeks_batch_mixed(stocha):
    rng = np.random.default_rng(1)
    insts = []
    for i in range(24):
        model = ["gbm", "heston", "merton"][i % 3]
        s0 = float(rng.uniform(80, 120))
        d = dict(model=model, s0=s0, r=float(rng.uniform(0, 0.06)), sigma=float(rng.uniform(0.1, 0.5)),
                 t=float(rng.uniform(0.1, 2.0)), strike=s0 * float(rng.uniform(0.8, 1.2)),
                 n_paths=int(10 ** rng.uniform(3.5, 4.5)), steps=int(rng.choice([12, 52])), seed=42 + i,
                 payoff="call" if i % 2 == 0 else "put")
        if model == "heston":
            d.update(v0=d["sigma"] ** 2, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7)
        if model == "merton":
            d.update(lambda_=1.0, mu_j=-0.05, sigma_j=0.1)
        insts.append(d)
    b32 = stocha.greeks_batch(insts, precision="fp32")
    b64 = stocha.greeks_batch(insts, precision="fp64")
    assert b32.shape == (24, 7)
    for i, d in enumerate(insts):
        keys = ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j")
        params = {k: d[k] for k in keys if k in d}
        one = stocha.greeks_fd(d["model"], params, d["payoff"], d["strike"], d["n_paths"], d["steps"], ALL,
                               seed=d["seed"])
        for j, g in enumerate(ALL):
            assert _close(b64[i, 2 + j], one[g], GREEK_FP64_RTOL), (i, g)
        assert _close(b32[i, 0], b64[i, 0], 1e-4, atol=1e-5), (i, b32[i, 0], b64[i, 0])


# configuration 4's FP32 batch against FP64, per Greek, as
# |fp32 - fp64| / max(|fp64|, 1e-3); measured maxima over the 128 instances:
# price 1.3e-6, delta 1.0e-6, gamma 4.8e-6, vega 2.8e-5, theta 2.8e-5, rho 1.6e-6
CONFIG4_BARS = {"price": 1e-5, "delta": 1e-5, "gamma": 1e-4, "vega": 2e-4, "theta": 2e-4, "rho": 1e-5}


@pytest.mark.slow
def test_config4_batch_fp32_against_fp64(stocha):
    """The 512 seeded Greeks instances of configuration 4 in one FP32 launch;
    every 4th instance (128) revalued scenario by scenario in FP64."""
    from bench import greeks_instances

    insts = greeks_instances()
    assert len(insts) == 512
    g32 = stocha.greeks_batch(insts, precision="fp32")
    sample = list(range(0, 512, 4))
    g64 = stocha.greeks_batch([insts[i] for i in sample], precision="fp64")
    cols = {"price": 0, "delta": 2, "gamma": 3, "vega": 4, "theta": 5, "rho": 6}
    for name, j in cols.items():
        err = np.abs(g32[sample, j] - g64[:, j]) / np.maximum(np.abs(g64[:, j]), 1e-3)
        assert err.max() <= CONFIG4_BARS[name], (name, float(err.max()), int(np.argmax(err)))
