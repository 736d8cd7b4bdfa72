"""Device paths and draws against the CPU oracle (FP64 plain form).

Bars (the engine's parity contract):
  * RNG integers, uniforms and normals of the RNG surface: bit-exact.
  * FP64 paths: within PATH_RTOL relative of the oracle; column 0 exact.
    (The only non-basic operation on the path is exp(): CUDA's and glibc's
    differ by at most an ulp now and then, compounded over <= 252 steps.)
  * Full-size runs: the configuration's 1e6-path runs, every row against the
    oracle's run of the same size.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PATH_RTOL = 1e-12


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


# ------------------------------------------------------------------- RNG ---
@pytest.mark.parametrize("seed", [0, 42, 2**64 + 3, 2**128 - 1])
def test_raw_u64_bit_exact(stocha, oracle, seed):
    r = stocha._stocha.RNG(seed=seed)
    st, inc = oracle.pcg_seed(seed)
    a = r.raw_u64(1)
    b = r.raw_u64(1_000_003)
    want = oracle.pcg_u64(st, inc, 1_000_004)
    np.testing.assert_array_equal(np.concatenate([a, b]), want)


def test_uniform_bit_exact_and_continuous(stocha, oracle):
    r = stocha.RNG(seed=7)
    st, inc = oracle.pcg_seed(7)
    got = np.concatenate([r.uniform(100), r.uniform(12345), r.uniform(1)])
    want, _, _ = oracle.stream_fill(st, inc, "uniform", 100 + 12345 + 1)
    np.testing.assert_array_equal(got, want)
    assert got.min() >= 0.0 and got.max() < 1.0


@pytest.mark.parametrize("sizes", [[1], [7, 1000], [100_003], [1_000_000, 5]])
def test_standard_normal_bit_exact(stocha, oracle, sizes):
    r = stocha.RNG(seed=123)
    st, inc = oracle.pcg_seed(123)
    got = np.concatenate([r.standard_normal(n) for n in sizes])
    want, used, st_end = oracle.stream_fill(st, inc, "standard_normal", sum(sizes))
    np.testing.assert_array_equal(got, want)
    # the generator position after the calls is the reference's
    assert f'"state":{st_end},' in r.save_state()


def test_normal_loc_scale_and_state_roundtrip(stocha, oracle):
    r = stocha.RNG(seed=42)
    _ = r.normal(size=500)
    js = r.save_state()
    expected = r.normal(size=100, loc=5.0, scale=2.0)
    restored = stocha.RNG.from_state(js)
    np.testing.assert_array_equal(restored.normal(size=100, loc=5.0, scale=2.0), expected)
    st, inc = oracle.pcg_seed(42)
    _, _, st2 = oracle.stream_fill(st, inc, "standard_normal", 500)
    want, _, _ = oracle.stream_fill(st2, inc, "normal", 100, loc=5.0, scale=2.0)
    np.testing.assert_array_equal(expected, want)


def test_empty_draws(stocha):
    r = stocha.RNG(seed=1)
    js = r.save_state()
    assert r.standard_normal(0).shape == (0,) and r.uniform(0).shape == (0,)
    assert r.save_state() == js


# ----------------------------------------------------------------- paths ---
GBM_CASES = [
    dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=2000, seed=42),
    dict(s0=50.0, mu=0.0, sigma=0.1, t=1.0, steps=10, n_paths=100, seed=0),
    dict(s0=100.0, mu=0.08, sigma=0.2, t=1.0, steps=52, n_paths=1001, seed=7, q=0.03),
    dict(s0=100.0, mu=0.05, sigma=0.9, t=3.0, steps=1, n_paths=333, seed=2**63 + 11),
    dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=1001, seed=42, antithetic=True),
    dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=3, n_paths=1, seed=5, antithetic=True),
]


@pytest.mark.parametrize("kw", GBM_CASES)
def test_gbm_parity(stocha, oracle, kw):
    got = stocha.gbm(**kw)
    want = oracle.gbm(kw["s0"], kw["mu"], kw["sigma"], kw["t"], kw["steps"], kw["n_paths"], seed=kw["seed"],
                      antithetic=kw.get("antithetic", False), q=kw.get("q", 0.0))
    assert got.shape == want.shape and got.dtype == np.float64 and got.flags.c_contiguous
    np.testing.assert_array_equal(got[:, 0], kw["s0"])
    assert _rel(got, want) <= PATH_RTOL


def test_gbm_config1_full_size(stocha, oracle):
    """s0=100, mu=0.05, sigma=0.20, t=1, steps=252, n_paths=100000, seed=42."""
    got = stocha.gbm(100.0, 0.05, 0.2, 1.0, 252, 100_000, seed=42)
    want = oracle.gbm(100.0, 0.05, 0.2, 1.0, 252, 100_000, seed=42)
    assert got.shape == (100_000, 253)
    assert _rel(got, want) <= PATH_RTOL
    assert abs(got[:, -1].mean() / (100 * math.exp(0.05)) - 1) < 5e-3


@pytest.mark.parametrize("na,anti", [(1, False), (2, False), (3, False), (3, True), (5, False)])
def test_multi_gbm_parity(stocha, oracle, na, anti):
    rng = np.random.default_rng(na)
    s0 = list(rng.uniform(50, 200, na))
    mu = list(rng.uniform(0.0, 0.1, na))
    sig = list(rng.uniform(0.1, 0.4, na))
    a = rng.normal(size=(na, na))
    cov = a @ a.T + na * np.eye(na)
    d = np.sqrt(np.diag(cov))
    corr = cov / np.outer(d, d)
    got = stocha.multi_gbm(s0, mu, sig, corr, 1.0, 60, 501, seed=9, antithetic=anti)
    want = oracle.multi_gbm(s0, mu, sig, corr, 1.0, 60, 501, seed=9, antithetic=anti)
    assert got.shape == (501, 61, na)
    assert _rel(got, want) <= PATH_RTOL


@pytest.mark.parametrize("scheme", ["euler", "qe"])
def test_heston_parity(stocha, oracle, scheme):
    kw = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0, steps=252, n_paths=1500,
              seed=42)
    got = stocha.heston(**kw, scheme=scheme)
    want = oracle.heston(*[kw[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t", "steps",
                                           "n_paths")], seed=42, scheme=scheme)
    assert _rel(got, want) <= PATH_RTOL
    # Feller-violating parameters (reference tests: kappa=1 with QE)
    got = stocha.heston(100.0, 0.04, 0.05, 1.0, 0.04, 0.3, -0.7, 1.0, 252, 700, seed=77, scheme=scheme)
    want = oracle.heston(100.0, 0.04, 0.05, 1.0, 0.04, 0.3, -0.7, 1.0, 252, 700, seed=77, scheme=scheme)
    assert _rel(got, want) <= PATH_RTOL and (got > 0).all()


def test_merton_parity(stocha, oracle):
    for lam, mu_j, sj in [(1.0, -0.05, 0.1), (0.0, 0.0, 0.0), (5.0, -0.2, 0.15), (200.0, 0.01, 0.3)]:
        got = stocha.merton_jump_diffusion(100.0, 0.05, 0.2, lam, mu_j, sj, 1.0, 252, 1200, seed=42)
        want = oracle.merton(100.0, 0.05, 0.2, lam, mu_j, sj, 1.0, 252, 1200, seed=42)
        assert _rel(got, want) <= PATH_RTOL, lam


def _rel_blocks(a, b, rows=50_000):
    """_rel over row blocks (bounded temporaries for multi-GB arrays)."""
    return max(_rel(a[i:i + rows], b[i:i + rows]) for i in range(0, len(a), rows))


@pytest.mark.slow
def test_config2_full_size(stocha, oracle):
    """The configuration's three 1e6-path x 252-step FP64 runs (seed 42),
    every row against the oracle's run of the same size on all host cores."""
    n = 1_000_000
    corr = np.array([[1, .6, .3], [.6, 1, .5], [.3, .5, 1]], float)
    got = stocha.multi_gbm([100, 50, 200], [0.05, 0.08, 0.03], [0.2, 0.3, 0.15], corr, 1.0, 252, n, seed=42)
    want = oracle.multi_gbm([100, 50, 200], [0.05, 0.08, 0.03], [0.2, 0.3, 0.15], corr, 1.0, 252, n, seed=42)
    assert got.shape == want.shape == (n, 253, 3)
    assert _rel_blocks(got, want) <= PATH_RTOL
    del got, want
    got = stocha.heston(100, 0.04, 0.05, 2.0, 0.04, 0.3, -0.7, 1.0, 252, n, seed=42)
    want = oracle.heston(100, 0.04, 0.05, 2.0, 0.04, 0.3, -0.7, 1.0, 252, n, seed=42)
    assert _rel_blocks(got, want) <= PATH_RTOL
    del got, want
    got = stocha.merton_jump_diffusion(100, 0.05, 0.2, 1.0, -0.05, 0.1, 1.0, 252, n, seed=42)
    want = oracle.merton(100, 0.05, 0.2, 1.0, -0.05, 0.1, 1.0, 252, n, seed=42)
    assert _rel_blocks(got, want) <= PATH_RTOL


def test_table_exp_accuracy(stocha):
    """The FP64 kernels' exponential (integer pipes: Tang's reduction in fixed
    point, a Q63 2^(j/256) table, one rounding to 53 bits) against exp in
    extended precision: <= 0.6 ulp of the true value for |t| < 16 (0.5 from the
    final rounding, < 0.06 from the truncated fixed-point steps), <= 2 ulp beyond (exp() fallback, compared with numpy's), exact special
    values, subnormal and overflow results."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(7)
    x = np.concatenate([
        rng.uniform(-1, 1, 200_000), rng.uniform(-40, 40, 200_000), rng.uniform(-699.9, 699.9, 100_000),
        rng.normal(0, 1e-3, 50_000),
        # reduction boundaries k ln2/256 and their neighbours (k = floor(t 256/ln2) flips there)
        np.nextafter(np.arange(-2000, 2000) * np.log(2) / 256, -np.inf),
        np.arange(-2000, 2000) * np.log(2) / 256,
        np.nextafter(np.arange(-2000, 2000) * np.log(2) / 256, np.inf),
        np.ldexp(1.0, np.arange(-70, 4)), -np.ldexp(1.0, np.arange(-70, 4)), [15.999999999999998, -15.999999999999998],
        np.array([0.0, -0.0, 1e-300, -1e-300, 0.5, 1.0, -1.0, 699.99, -699.99, 700.0, -700.0, 709.7, 710.0, -708.5,
                  -745.0, -800.0, np.inf, -np.inf, np.nan]),
    ])
    y = np.empty_like(x)
    P = ctypes.POINTER(ctypes.c_double)
    _lib.check(lib.stocha_debug_exp(None, x.ctypes.data_as(P), y.ctypes.data_as(P), x.size))
    want = np.exp(x)
    fin = np.isfinite(want) & (want > np.finfo(float).tiny)
    ulp = np.abs(y[fin] - want[fin]) / np.spacing(want[fin])
    assert ulp.max() <= 2.0, ulp.max()
    work = np.abs(x) < 16.0
    assert work.sum() > 300_000
    if np.finfo(np.longdouble).eps < 1e-18:  # x86 extended or quad precision
        exact = np.exp(x[work].astype(np.longdouble))
        err = np.abs(y[work].astype(np.longdouble) - exact) / np.spacing(exact.astype(np.float64)).astype(np.longdouble)
        assert float(err.max()) <= 0.6, float(err.max())
    else:
        assert (np.abs(y[work] - want[work]) / np.spacing(want[work])).max() <= 1.05
    assert (y[x == 0.0] == 1.0).all()
    # the early-exit form (issue-bound kernels) is the same function
    y4 = np.empty_like(x)
    _lib.check(lib.stocha_debug_f64(None, 4, x.ctypes.data_as(P), y4.ctypes.data_as(P), x.size))
    same = np.isnan(y) & np.isnan(y4)
    assert np.array_equal(y.view(np.uint64)[~same], y4.view(np.uint64)[~same])
    assert np.isinf(y[x == np.inf]).all() and (y[x == -np.inf] == 0).all() and np.isnan(y[np.isnan(x)]).all()
    assert np.isinf(y[x == 710.0]).all()
    sub = (want > 0) & (want < np.finfo(float).tiny)
    assert np.allclose(y[sub], want[sub], rtol=1e-12, atol=2 * np.spacing(0.0))


def test_integer_sqrt_is_correctly_rounded(stocha):
    """The FP64 kernels' integer-pipe square root (Heston's variance recursion)
    returns exactly IEEE sqrt's double, which the reference's f64::sqrt returns:
    random values over the whole exponent range and the working range,
    perfect squares and their neighbours, and the special values."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(19)
    k = rng.integers(1, 2**26, 200_000).astype(np.float64)
    sq = k * k * np.ldexp(1.0, rng.integers(-60, 60, k.size))
    x = np.concatenate([
        rng.uniform(0.0, 0.2, 500_000),
        np.ldexp(rng.uniform(0.5, 1.0, 500_000), rng.integers(-1021, 1023, 500_000)),
        sq, np.nextafter(sq, 0.0), np.nextafter(sq, np.inf),
        [0.0, -0.0, 1.0, 2.0, 4.0, 0.25, np.finfo(float).tiny, np.finfo(float).max, 5e-324, 1e-310,
         np.inf, -1.0, np.nan],
    ])
    y = np.empty_like(x)
    P = ctypes.POINTER(ctypes.c_double)
    _lib.check(lib.stocha_debug_sqrt(None, x.ctypes.data_as(P), y.ctypes.data_as(P), x.size))
    with np.errstate(invalid="ignore"):
        want = np.sqrt(x)
    assert np.array_equal(y.view(np.uint64)[~np.isnan(want)], want.view(np.uint64)[~np.isnan(want)])
    assert np.isnan(y[np.isnan(want)]).all()


def test_integer_normal_product_equals_dmul(stocha):
    """The normal's product (u >> 11) * X[L] 2^-53 on the integer pipes (used by
    the FP64-pipe-bound multi-GBM and Heston kernels) equals the FP64 pipe's
    correctly rounded DMUL bit for bit, over every layer and the whole 53-bit
    range, including 0, 1 and 2^53 - 1."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(23)
    n = 256 * 4000
    m = rng.integers(0, 2**53, n, dtype=np.uint64)
    m[::7] >>= rng.integers(1, 52, m[::7].size).astype(np.uint64)
    m[:256] = 0
    m[256:512] = 1
    m[512:768] = 2**53 - 1
    x = m.astype(np.float64)
    assert (x.astype(np.uint64) == m).all()
    y_int, y_fp = np.empty_like(x), np.empty_like(x)
    P = ctypes.POINTER(ctypes.c_double)
    _lib.check(lib.stocha_debug_f64(None, 2, x.ctypes.data_as(P), y_int.ctypes.data_as(P), n))
    _lib.check(lib.stocha_debug_f64(None, 3, x.ctypes.data_as(P), y_fp.ctypes.data_as(P), n))
    assert np.array_equal(y_int.view(np.uint64), y_fp.view(np.uint64))
    assert (y_fp[:256] == 0).all() and (y_fp[256:] >= 0).all()


def test_fast_tail_value_error(stocha):
    """The path kernels' tail value (hardware logarithm + one Newton step
    through the integer-pipe exponential, 8 FP64 operations) against the FP64
    log-and-divide form the RNG's normals use: within 1e-15 relative over 1e6
    random draws and the extremes of u1 = (draw >> 11) 2^-53 (the smallest
    draws, ln u1 = -36.7, take exp's |t| >= 16 branch)."""
    import ctypes

    from stocha_gb300 import _lib
    lib = _lib.load()
    P = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(77)
    m = rng.integers(1, 1 << 53, size=1_000_000, dtype=np.uint64)
    edge = np.array([1, 2, 3, 1000, 1 << 20, 1 << 30, (1 << 36) + 7, 1 << 52, (1 << 52) - 1, (1 << 52) + 1,
                     (1 << 53) - 1, (1 << 53) - 2, int(0.999999 * 2 ** 53), int(0.5 * 2 ** 53)], dtype=np.uint64)
    m = np.concatenate([m, edge])
    draws = (m << np.uint64(11)) | rng.integers(0, 1 << 11, size=m.size, dtype=np.uint64)
    x = draws.view(np.float64)
    fast = np.empty_like(x)
    exact = np.empty_like(x)
    _lib.check(lib.stocha_debug_f64(None, 5, x.ctypes.data_as(P), fast.ctypes.data_as(P), x.size))
    _lib.check(lib.stocha_debug_f64(None, 6, x.ctypes.data_as(P), exact.ctypes.data_as(P), x.size))
    assert np.isfinite(fast).all() and (exact >= 3.6).all()
    rel = np.abs(fast - exact) / exact
    assert rel.max() <= 1e-15, (rel.max(), m[rel.argmax()])


def test_fast_log_error_bounds(stocha):
    """The ziggurat tail test decides in FP32 with the hardware logarithm
    (__logf) and falls back to FP64 within a margin built from its error
    bounds, kLogAbs = 5e-7 on [0.5, 1) and kLogRel = 3e-7 |ln x| below 0.5
    (csrc/mc_device.cuh).  The bounds are checked here over every normal
    float in (0, 1), the whole domain of the test's arguments, so the FP32
    decision can never disagree with the reference's FP64 one."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    a, r = ctypes.c_double(), ctypes.c_double()
    _lib.check(lib.stocha_debug_fast_log_error(None, ctypes.byref(a), ctypes.byref(r)))
    print(f"__logf: max abs error on [0.5, 1) {a.value:.4g}, max relative error below 0.5 {r.value:.4g}")
    assert 0 < a.value <= 5e-7, a.value
    assert 0 < r.value <= 3e-7, r.value


def test_host_result_cache_reuse(stocha):
    """A released result's buffer serves the next result of the same size: the
    cached byte count rises on release and falls on reuse, and the values are
    those of a fresh array."""
    import ctypes
    import gc

    from stocha_gb300 import _lib

    lib = _lib.load()

    def cached():
        c = ctypes.c_size_t()
        _lib.check(lib.stocha_host_cache_stats(ctypes.byref(c), None))
        return c.value

    kw = dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=20_000, seed=3)
    a = stocha.gbm(**kw)
    first = a.copy()
    base = cached()
    del a
    gc.collect()
    assert cached() >= base + first.nbytes
    b = stocha.gbm(**kw)
    assert cached() <= base + 1
    np.testing.assert_array_equal(b, first)
    c = stocha.gbm(**dict(kw, seed=4))  # b is alive: a different buffer
    assert not np.shares_memory(b, c) and not np.array_equal(b, c)



@pytest.mark.parametrize("antithetic", [False, True])
def test_chunked_copy_overlap_same_result(stocha, antithetic):
    """A large result copied into a cached host buffer is computed in row chunks
    whose copies overlap the next chunk's compute; it must equal the one-launch
    result (the first call, into fresh memory), row for row, including the
    antithetic half and a multi-asset row layout."""
    import gc

    kw = dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=30, n_paths=700_001, seed=11, antithetic=antithetic)
    a = stocha.gbm(**kw)  # > 64 MB, > 2^19 rows
    first = a.copy()
    del a
    gc.collect()
    b = stocha.gbm(**kw)  # into the cached buffer: the chunked form
    np.testing.assert_array_equal(b, first)
    del b, first
    mk = dict(s0=[100.0, 50.0], mu=[0.05, 0.08], sigma=[0.2, 0.3], corr=np.array([[1.0, 0.6], [0.6, 1.0]]), t=1.0,
              steps=20, n_paths=600_000, seed=5, antithetic=antithetic)
    a = stocha.multi_gbm(**mk)
    first = a.copy()
    del a
    gc.collect()
    np.testing.assert_array_equal(stocha.multi_gbm(**mk), first)


@pytest.mark.parametrize("model", ["heston", "heston_qe", "merton", "hull_white"])
def test_chunked_copy_overlap_other_models(stocha, model):
    """The chunked copy/compute overlap for every other materialising model:
    second call (cached buffer, row chunks) equals the first (one launch)."""
    import gc

    calls = {
        "heston": lambda: stocha.heston(100.0, 0.04, 0.05, 2.0, 0.04, 0.3, -0.7, 1.0, 24, 560_001, seed=9),
        "heston_qe": lambda: stocha.heston(100.0, 0.04, 0.05, 2.0, 0.04, 0.3, -0.7, 1.0, 24, 560_001, seed=9,
                                           scheme="qe"),
        "merton": lambda: stocha.merton_jump_diffusion(100.0, 0.05, 0.2, 1.0, -0.05, 0.1, 1.0, 24, 560_001, seed=9),
        "hull_white": lambda: stocha.hull_white(0.03, 0.1, 0.005, 0.01, 1.0, 24, 560_001, seed=9),
    }
    a = calls[model]()
    assert a.nbytes >= 64 << 20
    first = a.copy()
    del a
    gc.collect()
    np.testing.assert_array_equal(calls[model](), first)
