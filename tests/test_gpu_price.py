"""Fused in-kernel pricing.

* FP64 fused price equals exp(-rT) * mean(payoff(S_T)) of the oracle's own
  paths (the reference workflow, greeks.rs:313-320) to FP64_PRICE_RTOL: only
  the summation order differs.
* FP32 fused price is within FP32_PRICE_RTOL of the FP64 price (the target
  accuracy of the FP32 forms is 1e-4 relative; the samplers consume the same
  draws, so the gap is rounding).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_PRICE_RTOL = 1e-12
FP32_PRICE_RTOL = 1e-4

MODELS = {
    "gbm": dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0),
    "heston": dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0),
    "merton": dict(s0=100.0, mu=0.05, sigma=0.2, lambda_=1.0, mu_j=-0.05, sigma_j=0.1, t=1.0),
}


def _oracle_terminal(oracle, model, p, steps, n, seed):
    if model == "gbm":
        return oracle.gbm(p["s0"], p["mu"], p["sigma"], p["t"], steps, n, seed=seed)[:, -1]
    if model == "heston":
        return oracle.heston(p["s0"], p["v0"], p["mu"], p["kappa"], p["theta"], p["xi"], p["rho"], p["t"], steps, n,
                             seed=seed)[:, -1]
    return oracle.merton(p["s0"], p["mu"], p["sigma"], p["lambda_"], p["mu_j"], p["sigma_j"], p["t"], steps, n,
                         seed=seed)[:, -1]


@pytest.mark.parametrize("model", ["gbm", "heston", "merton"])
@pytest.mark.parametrize("payoff", ["call", "put"])
def test_fp64_fused_matches_oracle(stocha, oracle, model, payoff):
    p = MODELS[model]
    n, steps = 20_000, 252
    price, se = stocha.price_european(model, p, strike=100.0, payoff=payoff, steps=steps, n_paths=n, seed=42,
                                      precision="fp64")
    sT = _oracle_terminal(oracle, model, p, steps, n, 42)
    pay = np.maximum(sT - 100.0, 0) if payoff == "call" else np.maximum(100.0 - sT, 0)
    want = math.exp(-p["mu"] * p["t"]) * pay.sum() / n
    assert abs(price - want) <= FP64_PRICE_RTOL * abs(want)
    want_se = math.exp(-p["mu"] * p["t"]) * pay.std(ddof=1) / math.sqrt(n)
    assert abs(se - want_se) <= 1e-8 * want_se


@pytest.mark.parametrize("model", ["gbm", "heston", "merton"])
def test_fp32_fused_within_1e4_of_fp64(stocha, model):
    p = MODELS[model]
    kw = dict(strike=100.0, payoff="call", steps=252, n_paths=200_000, seed=42)
    p64, _ = stocha.price_european(model, p, precision="fp64", **kw)
    p32, _ = stocha.price_european(model, p, precision="fp32", **kw)
    assert abs(p32 - p64) <= FP32_PRICE_RTOL * abs(p64), (p32, p64)


@pytest.mark.parametrize("n", [1, 2, 1001, 300_001])
def test_antithetic_fused(stocha, oracle, n):
    p = MODELS["gbm"]
    kw = dict(strike=100.0, payoff="call", steps=52, n_paths=n, seed=11, antithetic=True)
    p64, _ = stocha.price_european("gbm", p, precision="fp64", **kw)
    p32, _ = stocha.price_european("gbm", p, precision="fp32", **kw)
    paths = oracle.gbm(p["s0"], p["mu"], p["sigma"], p["t"], 52, n, seed=11, antithetic=True)
    want = math.exp(-0.05) * np.maximum(paths[:, -1] - 100.0, 0).sum() / n
    assert abs(p64 - want) <= FP64_PRICE_RTOL * max(abs(want), 1e-12)
    assert abs(p32 - p64) <= FP32_PRICE_RTOL * max(abs(p64), 1e-3)


def test_fused_small_and_uneven_counts(stocha):
    # fewer paths than lanes, and counts that do not divide the grid
    for n in (1, 7, 255, 257, 4099):
        for model in ("gbm", "heston", "merton"):
            p64, _ = stocha.price_european(model, MODELS[model], 100.0, steps=12, n_paths=n, seed=3,
                                           precision="fp64")
            p32, _ = stocha.price_european(model, MODELS[model], 100.0, steps=12, n_paths=n, seed=3,
                                           precision="fp32")
            assert abs(p32 - p64) <= FP32_PRICE_RTOL * max(abs(p64), 1e-2), (model, n, p32, p64)


def test_multi_asset_fused(stocha, oracle):
    corr = np.array([[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], float)
    m = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15], corr=corr, t=1.0)
    res64 = stocha.price_european("multi_gbm", m, strike=100.0, steps=252, n_paths=20_000, seed=42, rate=0.05,
                                  precision="fp64")
    paths = oracle.multi_gbm(m["s0"], m["mu"], m["sigma"], corr, 1.0, 252, 20_000, seed=42)
    for a in range(3):
        want = math.exp(-0.05) * np.maximum(paths[:, -1, a] - 100.0, 0).sum() / 20_000
        assert abs(res64[a][0] - want) <= FP64_PRICE_RTOL * max(abs(want), 1e-300)
    res32 = stocha.price_european("multi_gbm", m, strike=100.0, steps=252, n_paths=200_000, seed=42, rate=0.05,
                                  precision="fp32")
    res64b = stocha.price_european("multi_gbm", m, strike=100.0, steps=252, n_paths=200_000, seed=42, rate=0.05,
                                   precision="fp64")
    for a in range(3):
        assert abs(res32[a][0] - res64b[a][0]) <= FP32_PRICE_RTOL * abs(res64b[a][0])


def test_fp32_materialised_close_to_fp64(stocha):
    import ctypes

    from stocha_gb300 import _lib

    torch = pytest.importorskip("torch")
    d64 = torch.empty((5000, 253), dtype=torch.float64, device="cuda")
    d32 = torch.empty((5000, 253), dtype=torch.float32, device="cuda")
    m = stocha.model_struct("heston", MODELS["heston"], steps=252, n_paths=5000)
    lib = _lib.load()
    torch.cuda.synchronize()
    _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, _lib.FP64, ctypes.c_void_p(d64.data_ptr())))
    _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, _lib.FP32, ctypes.c_void_p(d32.data_ptr())))
    _lib.check(lib.stocha_ctx_sync(None))
    a, b = d64.cpu().numpy(), d32.cpu().double().numpy()
    assert np.max(np.abs(a - b) / a) < 1e-4


@pytest.mark.parametrize("model", ["gbm", "heston", "merton", "multi_gbm"])
def test_every_tuned_launch_shape(stocha, model):
    """Each launch shape the autotuner can install (threads per block, paths
    per thread in lockstep, grid waves) draws the same values: the FP32 fused
    price stays within 1e-5 of the FP64 plain price for all eighteen, on odd
    path counts (the lockstep tail) and antithetic multi-GBM; then a real
    autotune installs one of them."""
    if model == "multi_gbm":
        p = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15],
                 corr=[[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], t=1.0)
        na = 3
    else:
        p, na = MODELS[model], 0
    before = stocha.tune_get(model, na)
    try:
        for n in (1, 777, 100_003):
            kw = dict(strike=100.0, payoff="put", steps=50, n_paths=n, seed=9)
            want = stocha.price_european(model, p, precision="fp64", **kw)
            for block in (64, 128, 256):
                for variant, ilp in ((0, 1), (1, 1), (1, 2), (2, 1)):
                    for waves in (1, 2):
                        stocha.tune_set(model, block, ilp, waves, variant=variant, n_assets=na)
                        got = stocha.price_european(model, p, precision="fp32", **kw)
                        pairs = zip(got, want) if model == "multi_gbm" else [(got, want)]
                        for (g, _), (w, _) in pairs:
                            assert abs(g - w) <= 1e-5 * max(abs(w), 1e-3), (n, block, ilp, waves, g, w)
        t = stocha.autotune(model, p, steps=50, n_paths=200_000, reps=2)
        assert t["candidates"] == 24 and t["ms_best"] <= t["ms_default"] * 1.0001
        assert stocha.tune_get(model, na)["block"] == t["block"]
    finally:
        stocha.tune_set(model, before["block"], before["ilp"], before["waves"], variant=before["variant"],
                        n_assets=na)


@pytest.mark.parametrize("model", ["gbm", "heston", "merton", "multi_gbm"])
def test_work_queue_price_is_shape_independent(stocha, model):
    """The single-path forms take batches of 32 rows from a work queue and
    write one record per batch in a fixed lane order, so a form's FP32 price
    is bit-identical run to run and across its block sizes and grid waves,
    including row counts that leave a partial batch."""
    if model == "multi_gbm":
        p = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15],
                 corr=[[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], t=1.0)
        na = 3
    else:
        p, na = MODELS[model], 0
    before = stocha.tune_get(model, na)
    try:
        for n in (1, 33, 200_017):
            kw = dict(strike=100.0, payoff="call", steps=30, n_paths=n, seed=11, precision="fp32")
            for variant in (0, 1, 2):
                got = set()
                for block in (64, 256):
                    for waves in (1, 2):
                        stocha.tune_set(model, block, 1, waves, variant=variant, n_assets=na)
                        for _ in range(2):
                            got.add(repr(stocha.price_european(model, p, **kw)))
                assert len(got) == 1, (n, variant, got)
    finally:
        stocha.tune_set(model, before["block"], before["ilp"], before["waves"], variant=before["variant"],
                        n_assets=na)


@pytest.mark.parametrize("model", ["gbm", "multi_gbm"])
def test_work_queue_multi_row_batches(stocha, model):
    """Above 32 * 65536 rows a queue batch holds several 32-row groups per
    warp (here 64 rows, the last batch partial): every row is priced once."""
    if model == "multi_gbm":
        p = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15],
                 corr=[[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], t=1.0)
    else:
        p = MODELS[model]
    kw = dict(strike=100.0, payoff="call", steps=4, n_paths=2_100_001, seed=5)
    got = stocha.price_european(model, p, precision="fp32", **kw)
    again = stocha.price_european(model, p, precision="fp32", **kw)
    want = stocha.price_european(model, p, precision="fp64", **kw)
    pairs = zip(got, want) if model == "multi_gbm" else [(got, want)]
    for (g, _), (w, _) in pairs:
        assert abs(g - w) <= 1e-5 * abs(w), (g, w)
    assert repr(got) == repr(again)
