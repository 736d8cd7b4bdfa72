"""stocha_price_noalloc: fused pricing for callers that cannot allocate
device memory (a host application that owns all device memory, or a request
path that must never reach cudaMalloc).

It runs the same kernels as stocha_price_device with its scratch in a static
device array, so through the C ABI its raw payoff sums must equal the existing
entry point's, call after call.  This file is collected last on purpose: it
needs nothing from the other tests and must pass alone in a fresh process as
well as after them.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-12  # same kernels and reduction order: the tolerance of the FP64 price tests
# Above 524,288 FP32 rows the allocation-free form takes 64-row work-queue
# batches (its 16384 records would not hold 32-row ones), so the FP32 payoff
# sums are grouped differently from stocha_price_device's: they agree to FP32
# rounding of the per-batch sums, far inside the 1e-4 FP32 price bar.
GROUPED_RTOL = 1e-6

HESTON = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0)
MULTI = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15],
             corr=np.array([[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], float), t=1.0)


@pytest.mark.parametrize("model,params,precision,n", [("heston", HESTON, "fp64", 20_000),
                                                       ("heston", HESTON, "fp32", 300_000),
                                                       ("heston", HESTON, "fp32", 600_000),
                                                       ("multi_gbm", MULTI, "fp64", 10_000),
                                                       ("gbm", dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0), "fp32", 1)])
def test_noalloc_matches_price_device(stocha, model, params, precision, n):
    torch = pytest.importorskip("torch")
    from stocha_gb300 import _lib

    lib = _lib.load()
    m = stocha.model_struct(model, params, steps=52, n_paths=n)
    na = m.n_assets if model == "multi_gbm" else 1
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    ref = torch.zeros(2 * na, dtype=torch.float64, device="cuda")
    _lib.check(lib.stocha_price_device(None, ctypes.byref(m), 42, prec, _lib.PAYOFF_CALL, 100.0, 0.05,
                                       ctypes.c_void_p(ref.data_ptr())))
    _lib.check(lib.stocha_ctx_sync(None))
    want = ref.cpu().numpy()
    stream = torch.cuda.Stream()
    for _ in range(2):  # two calls in a row share (and reuse) the static scratch
        out = torch.full((2 * na,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.check(lib.stocha_price_noalloc(ctypes.byref(m), 42, prec, _lib.PAYOFF_CALL, 100.0,
                                            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))
        got = out.cpu().numpy()
        rtol = GROUPED_RTOL if precision == "fp32" and n > 524_288 else SUM_RTOL
        assert np.all(np.abs(got - want) <= rtol * np.abs(want)), (got, want)


def test_noalloc_rejects_beyond_its_scratch(stocha):
    from stocha_gb300 import _lib

    lib = _lib.load()
    corr = np.eye(5)
    m = stocha.model_struct("multi_gbm", dict(s0=[100.0] * 5, mu=[0.05] * 5, sigma=[0.2] * 5, corr=corr, t=1.0),
                            steps=12, n_paths=100)
    rc = lib.stocha_price_noalloc(ctypes.byref(m), 42, _lib.FP64, _lib.PAYOFF_CALL, 100.0, ctypes.c_void_p(1), None)
    assert rc == _lib.STOCHA_ERR_VALUE
    assert "at most 4 assets" in lib.stocha_last_error().decode()
