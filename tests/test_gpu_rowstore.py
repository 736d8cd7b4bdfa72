"""Row-major path output through the staged sector writer (row_store.cuh).

The materialised kernels write each row in whole 32-byte sectors: a lane
stages its values in shared memory and stores a sector when it is complete;
the sector two rows share is merged across neighbouring lanes at the end of
the row; sectors whose neighbour row is not in the warp (a launch's first or
last rows, or a launch that does not start on a sector boundary) are written
element by element.  These tests cover the layouts where that logic has
cases: row lengths around the two-sector minimum, partial warps, every
phase of a row within its first sector, multi-asset rows, chunked host
copies, and output buffers that do not start on a sector.

Bars: FP64 paths equal the oracle within PATH_RTOL (the FP64 parity bar);
FP32 rows are all written (no NaN sentinel left) and within F32_RTOL of the
FP64 paths of the same draws.
"""
import ctypes
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PATH_RTOL = 1e-12
# FP32 materialised paths: log-space compensated sums and one expf per value;
# measured ~1e-6 relative at 252 steps
F32_RTOL = 2e-5


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


@pytest.mark.parametrize("steps", [6, 7, 8, 9, 10, 11, 15, 16, 17])
@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 65, 257])
def test_gbm_row_lengths_and_partial_warps(stocha, oracle, steps, n):
    got = stocha.gbm(100.0, 0.05, 0.2, 1.0, steps, n, seed=3)
    want = oracle.gbm(100.0, 0.05, 0.2, 1.0, steps, n, seed=3)
    assert got.shape == (n, steps + 1)
    assert _rel(got, want) <= PATH_RTOL


@pytest.mark.parametrize("na,steps", [(2, 3), (2, 4), (3, 2), (3, 3), (3, 7), (4, 1), (5, 1), (5, 2), (7, 5)])
def test_multi_gbm_row_layouts(stocha, oracle, na, steps):
    rng = np.random.default_rng(10 * na + steps)
    a = rng.normal(size=(na, na))
    cov = a @ a.T + na * np.eye(na)
    d = np.sqrt(np.diag(cov))
    corr = cov / np.outer(d, d)
    args = (list(rng.uniform(50, 200, na)), list(rng.uniform(0.0, 0.1, na)), list(rng.uniform(0.1, 0.4, na)), corr,
            1.0, steps, 97)
    got = stocha.multi_gbm(*args, seed=4)
    want = oracle.multi_gbm(*args, seed=4)
    assert got.shape == (97, steps + 1, na)
    assert _rel(got, want) <= PATH_RTOL


def _overlap_bounds(rows):
    """Row boundaries of the overlapped copy's chunks: a ramp from 2^14 rows,
    doubling, up to the steady max(2^17, rows / 8) rows (rounded up to 32)."""
    per = (max(1 << 17, (rows + 7) // 8) + 31) // 32 * 32
    b, size = [0], 1 << 14
    while b[-1] < rows:
        b.append(min(rows, b[-1] + min(size, per)))
        size = size * 2 if size < per else size
    return b


def test_chunked_host_copy(stocha, oracle):
    """2^21 + 8 rows of 9 doubles into a cached host buffer: the overlap path
    computes row chunks (a ramp of 2^14, 2^15, ... 2^18 rows, then
    262 176-row chunks; all multiples of 32 rows) whose copies overlap the
    next chunk.
    The result must equal the one-launch result (first call, fresh memory)
    and the oracle around every chunk boundary."""
    n, steps = (1 << 21) + 8, 8
    kw = dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=steps, n_paths=n, seed=21)
    a = stocha.gbm(**kw)
    assert a.nbytes >= 64 << 20
    first = a.copy()
    del a
    gc.collect()
    b = stocha.gbm(**kw)  # the cached buffer: chunked launches
    np.testing.assert_array_equal(b, first)
    bounds = _overlap_bounds(n)[1:-1]
    assert bounds[:5] == [1 << 14, 3 << 14, 7 << 14, 15 << 14, 31 << 14] and len(bounds) == 11
    want = oracle.gbm(100.0, 0.05, 0.2, 1.0, steps, bounds[-1] + 40, seed=21, threads=8)
    for c in bounds:
        lo, hi = c - 40, c + 40
        assert _rel(b[lo:hi], want[lo:hi]) <= PATH_RTOL, c


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_unaligned_output_base(stocha, precision):
    """A caller's device buffer need not start on a 32-byte sector: with the
    output shifted by 1..SE-1 elements every lane-0 row starts mid-sector and
    the writer stores the unshared pieces element by element.  The values
    must equal the aligned launch's bit for bit, and nothing outside the
    array may be written."""
    torch = pytest.importorskip("torch")
    from stocha_gb300 import _lib

    lib = _lib.load()
    se = 4 if precision == "fp64" else 8
    dt = torch.float64 if precision == "fp64" else torch.float32
    prec = _lib.FP64 if precision == "fp64" else _lib.FP32
    n, steps = 1000, 40
    m = stocha.model_struct("heston", dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7,
                                           t=1.0), steps=steps, n_paths=n)
    size = n * (steps + 1)
    base = torch.empty(size + 2 * se, dtype=dt, device="cuda")
    ref = None
    for off in range(se):
        base.fill_(-7.0)
        view = base[off:off + size]
        _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, prec, ctypes.c_void_p(view.data_ptr())))
        _lib.check(lib.stocha_ctx_sync(None))
        host = base.cpu().numpy()
        got = host[off:off + size]
        assert (host[:off] == -7.0).all() and (host[off + size:] == -7.0).all(), off
        if ref is None:
            ref = got.copy()
        else:
            np.testing.assert_array_equal(got.view(np.uint64 if precision == "fp64" else np.uint32),
                                          ref.view(np.uint64 if precision == "fp64" else np.uint32))


def _paths_device(stocha, torch, model, params, steps, n, precision, seed=42):
    from stocha_gb300 import _lib

    lib = _lib.load()
    m = stocha.model_struct(model, params, steps=steps, n_paths=n)
    width = m.n_assets if model == "multi_gbm" else 1
    shape = (n, steps + 1, width) if model == "multi_gbm" else (n, steps + 1)
    dt = torch.float32 if precision == "fp32" else torch.float64
    out = torch.full(shape, float("nan"), dtype=dt, device="cuda")
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), seed, prec, ctypes.c_void_p(out.data_ptr())))
    _lib.check(lib.stocha_ctx_sync(None))
    return out.cpu().numpy()


HESTON = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0)
MERTON = dict(s0=100.0, mu=0.05, sigma=0.2, lambda_=1.0, mu_j=-0.05, sigma_j=0.1, t=1.0)
MULTI = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15],
             corr=np.array([[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], float), t=1.0)
GBM = dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0)


@pytest.mark.parametrize("model,params", [("gbm", GBM), ("heston", HESTON), ("merton", MERTON),
                                          ("multi_gbm", MULTI)])
@pytest.mark.parametrize("steps,n", [(15, 1), (16, 33), (17, 250), (52, 4099), (252, 20_000)])
def test_fp32_rows_written_and_close_to_fp64(stocha, model, params, steps, n):
    torch = pytest.importorskip("torch")
    p32 = _paths_device(stocha, torch, model, params, steps, n, "fp32")
    assert not np.isnan(p32).any()  # every element written exactly where it belongs
    p64 = _paths_device(stocha, torch, model, params, steps, n, "fp64")
    assert _rel(p32, p64) <= F32_RTOL
