"""Heston QE (heston.rs:89-174) in FP32: fused pricing and materialised paths
against the FP64 form on the same draws.

The FP32 form takes the FP64 form's branches and draws; a quadratic /
exponential decision psi <= 1.5 made in FP32 can differ for psi within ~1e-6
of 1.5, and that path draws differently from there on (a valid path of the
same scheme).  Bars: the European price within PRICE_RTOL of FP64 at the
configuration's size (1e6 paths x 252 steps), and, for materialised paths,
at least ROW_SHARE of the rows within ROW_RTOL of their FP64 rows.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRICE_RTOL = 1e-4
ROW_RTOL = 1e-4
ROW_SHARE = 0.999
HESTON = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0, scheme="qe")


@pytest.mark.parametrize("payoff,strike", [("call", 100.0), ("put", 90.0)])
def test_fp32_qe_price_at_config_size(stocha, payoff, strike):
    p64, se64 = stocha.price_european("heston", HESTON, strike, payoff=payoff, steps=252, n_paths=1_000_000,
                                      precision="fp64")
    p32, se32 = stocha.price_european("heston", HESTON, strike, payoff=payoff, steps=252, n_paths=1_000_000,
                                      precision="fp32")
    assert abs(p32 - p64) <= PRICE_RTOL * abs(p64), (p32, p64)
    assert abs(se32 - se64) <= 1e-3 * se64


def test_fp32_qe_feller_violating(stocha):
    """kappa = 1 (2 kappa theta < xi^2 is not needed for QE's exponential
    branch to fire: small v does it), many exponential-branch steps."""
    prm = dict(HESTON, kappa=1.0, xi=0.9)
    p64, _ = stocha.price_european("heston", prm, 100.0, steps=52, n_paths=400_000, precision="fp64")
    p32, _ = stocha.price_european("heston", prm, 100.0, steps=52, n_paths=400_000, precision="fp32")
    assert abs(p32 - p64) <= PRICE_RTOL * abs(p64), (p32, p64)


@pytest.mark.parametrize("steps,n", [(12, 1001), (252, 20_000)])
def test_fp32_qe_materialised_rows(stocha, steps, n):
    torch = pytest.importorskip("torch")
    from stocha_gb300 import _lib

    lib = _lib.load()
    m = stocha.model_struct("heston", HESTON, steps=steps, n_paths=n)
    out = {}
    for prec, dt, P in (("fp64", torch.float64, _lib.FP64), ("fp32", torch.float32, _lib.FP32)):
        buf = torch.full((n, steps + 1), float("nan"), dtype=dt, device="cuda")
        _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, P, ctypes.c_void_p(buf.data_ptr())))
        _lib.check(lib.stocha_ctx_sync(None))
        out[prec] = buf.cpu().numpy().astype(np.float64)
    assert not np.isnan(out["fp32"]).any()
    np.testing.assert_array_equal(out["fp32"][:, 0], np.float32(100.0))
    rel = np.max(np.abs(out["fp32"] - out["fp64"]) / out["fp64"], axis=1)
    assert np.mean(rel <= ROW_RTOL) >= ROW_SHARE, np.sort(rel)[-5:]
