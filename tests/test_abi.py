"""The C ABI and host logic, without a GPU.

* libstocha_gpu.so builds (nvcc cross-compiles for sm_103a) and exports every
  function include/stocha_gpu.h declares.
* Argument validation happens on the host before any CUDA call and raises the
  reference's exceptions and messages (src/lib.rs), checked here the way the
  reference's own tests check them.
* The integer fast-path thresholds equal the reference's FP64 comparison.
"""
import ctypes
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _declared():
    src = open(os.path.join(ROOT, "include", "stocha_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(stocha_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(stocha):
    from stocha_gb300 import _lib

    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_fast_path_thresholds_match_fp64_compare(stocha):
    from stocha_gb300 import _lib

    lib = _lib.load()
    thr = np.zeros(256, np.uint64)
    lib.stocha_debug_zig_thresholds.argtypes = [_lib.P_u64]
    assert lib.stocha_debug_zig_thresholds(thr.ctypes.data_as(_lib.P_u64)) == 0
    from tests.test_oracle import _table_from_inc

    _, X, _ = _table_from_inc()
    rng = np.random.default_rng(5)
    two53 = 2.0**-53
    for L in range(256):
        t = int(thr[L])
        cands = [0, 1, t - 2, t - 1, t, t + 1, 2**53 - 1] + [int(v) for v in rng.integers(0, 2**53, 64)]
        for m in cands:
            if 0 <= m < 2**53:
                fast = (float(m) * two53) * X[L] < X[L + 1]  # normal.rs:25-27
                assert fast == (m < t), (L, m, t)
    assert int(thr[255]) == 0  # X[256] = 0: layer 255 never takes the fast path
    # the kernels compare the raw draw with thr * 2^11, exact only while thr < 2^53
    assert int(thr.max()) < 2**53


def test_validation_messages(stocha):
    s = stocha
    cases = [
        (lambda: s.gbm(-1.0, 0.05, 0.2, 1.0, 10, 10), "s0 must be positive"),
        (lambda: s.gbm(100.0, 0.05, 0.0, 1.0, 10, 5), "sigma must be positive"),
        (lambda: s.gbm(100.0, 0.05, 0.2, -1.0, 10, 10), "t must be positive"),
        (lambda: s.gbm(100.0, 0.05, 0.2, 1.0, 0, 10), "steps and n_paths must be positive"),
        (lambda: s.heston(100, -0.1, 0.05, 2, 0.04, 0.3, -0.7, 1, 10, 10), "v0 must be non-negative"),
        (lambda: s.heston(100, 0.04, 0.05, 0, 0.04, 0.3, -0.7, 1, 10, 10), "kappa must be positive"),
        (lambda: s.heston(100, 0.04, 0.05, 2, 0, 0.3, -0.7, 1, 10, 10), "theta must be positive"),
        (lambda: s.heston(100, 0.04, 0.05, 2, 0.04, 0, -0.7, 1, 10, 10), "xi must be positive"),
        (lambda: s.heston(100, 0.04, 0.05, 2, 0.04, 0.3, 2.0, 1, 10, 10), "rho must be in [-1, 1]"),
        (lambda: s.heston(100, 0.04, 0.05, 2, 0.04, 0.3, -0.7, 1, 10, 10, scheme="bad"),
         "scheme must be 'euler' or 'qe'"),
        (lambda: s.merton_jump_diffusion(100, 0.05, 0.0, 1, -0.05, 0.1, 1, 10, 10), "sigma must be positive"),
        (lambda: s.merton_jump_diffusion(100, 0.05, 0.2, -1, -0.05, 0.1, 1, 10, 10), "lambda_ must be non-negative"),
        (lambda: s.merton_jump_diffusion(100, 0.05, 0.2, 1, -0.05, -0.1, 1, 10, 10), "sigma_j must be non-negative"),
        (lambda: s.multi_gbm([], [], [], np.eye(1), 1.0, 10, 10), "s0 must not be empty"),
        (lambda: s.multi_gbm([100.0], [0.05, 0.08], [0.2], np.eye(1), 1.0, 10, 10),
         "s0, mu, sigma must have the same length"),
        (lambda: s.multi_gbm([-1.0, 50.0], [0.05, 0.08], [0.2, 0.3], np.eye(2), 1.0, 10, 10),
         "all s0 must be positive"),
        (lambda: s.multi_gbm([100.0, 50.0], [0.05, 0.08], [0.2, 0.0], np.eye(2), 1.0, 10, 10),
         "all sigma must be positive"),
        (lambda: s.multi_gbm([100.0, 50.0], [0.05, 0.08], [0.2, 0.3], np.eye(3), 1.0, 10, 10),
         "corr must be (2, 2), got (3, 3)"),
        (lambda: s.multi_gbm([100.0, 50.0], [0.05, 0.08], [0.2, 0.3], np.array([[1.0, 1.5], [1.5, 1.0]]), 1.0,
                             10, 10), "matrix is not positive-definite (diagonal element 1 = -1.25)"),
        (lambda: s.RNG(seed=0).normal(size=10, scale=-1.0), "scale must be positive"),
        (lambda: s.RNG(seed=0, algorithm="mt"), "Unknown algorithm: 'mt'. Supported: 'pcg64dxsm'"),
    ]
    for fn, msg in cases:
        with pytest.raises(ValueError) as ei:
            fn()
        assert str(ei.value) == msg


def test_conversion_errors(stocha):
    with pytest.raises(OverflowError):
        stocha.gbm(100.0, 0.05, 0.2, 1.0, -5, 10)
    with pytest.raises(OverflowError):
        stocha.gbm(100.0, 0.05, 0.2, 1.0, 10, 10, seed=2**64)
    with pytest.raises(TypeError):
        stocha.gbm(100.0, 0.05, 0.2, 1.0, 10.5, 10)
    with pytest.raises(OverflowError):
        stocha.RNG(seed=2**128)


def test_host_buffer_cache_host_logic(stocha):
    """Acquire/release of the host result cache without a GPU: a buffer whose
    pages were never written is unmapped on release (nothing cached), a
    second release and a foreign pointer are errors, the cap is positive."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    cached, cap = ctypes.c_size_t(), ctypes.c_size_t()
    _lib.check(lib.stocha_host_cache_stats(ctypes.byref(cached), ctypes.byref(cap)))
    assert cap.value > 0
    before = cached.value
    p = ctypes.c_void_p()
    _lib.check(lib.stocha_host_buffer_acquire(3 << 20, ctypes.byref(p)))
    assert p.value and p.value % 4096 == 0
    ctypes.memset(p.value, 7, 3 << 20)  # the memory is usable
    _lib.check(lib.stocha_host_buffer_release(p))
    _lib.check(lib.stocha_host_cache_stats(ctypes.byref(cached), None))
    assert cached.value == before  # never filled by a device copy: not kept
    for bad in (p, ctypes.c_void_p(12345)):
        with pytest.raises(ValueError, match="not a buffer from stocha_host_buffer_acquire"):
            _lib.check(lib.stocha_host_buffer_release(bad))
    # the Python layer's arrays: small ones are plain NumPy memory, large ones cached buffers
    small = stocha._stocha._host_array((10, 10))
    big = stocha._stocha._host_array((1000, 253))
    assert small.flags.owndata and not big.flags.owndata and big.flags.writeable and big.flags.c_contiguous
    big[:] = 1.0
    del big
    # concurrent acquire/release from several threads (the cache is process-wide)
    import threading

    errors = []

    def work():
        for _ in range(100):
            q = ctypes.c_void_p()
            if lib.stocha_host_buffer_acquire(2 << 20, ctypes.byref(q)) or not q.value:
                errors.append("acquire")
                return
            ctypes.memset(q.value, 1, 4096)
            if lib.stocha_host_buffer_release(q):
                errors.append("release")

    threads = [threading.Thread(target=work) for _ in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors


def test_rng_state_json_roundtrip(stocha):
    r = stocha.RNG(seed=2**100 + 7)
    assert r.seed == 2**100 + 7 and repr(r) == f"RNG(seed={2**100 + 7}, algorithm='pcg64dxsm')"
    js = r.save_state()
    assert js.startswith('{"version":2,"rng":{"state":') and js.endswith(f',"seed":{2**100 + 7}}}')
    r2 = stocha.RNG.from_state(js)
    assert r2.save_state() == js and r2.seed == r.seed
    legacy = stocha.RNG.from_state('{"seed":42}')
    assert legacy.save_state() == stocha.RNG(seed=42).save_state()
    with pytest.raises(ValueError):
        stocha.RNG.from_state("not-valid-json")


def test_rng_seed_state_matches_oracle(stocha, oracle):
    for seed in (0, 42, 2**64 + 3, 2**128 - 1):
        r = stocha.RNG(seed=seed)
        st, inc = oracle.pcg_seed(seed)
        js = r.save_state()
        assert f'"state":{st},' in js and f'"increment":{inc}}}' in js


def test_greeks_validation_messages(stocha):
    gbm = {"s0": 100.0, "r": 0.05, "sigma": 0.2, "t": 1.0}
    fd = stocha.greeks_fd
    cases = [  # reference tests/test_greeks.py validation + lib.rs messages
        (lambda: fd("invalid", gbm, "call", 100.0, 1000, 10, ["delta"]),
         "Unknown model: 'invalid'. Supported: gbm, heston, merton"),
        (lambda: fd("gbm", gbm, "call", 100.0, 1000, 10, ["invalid"]),
         "Unknown greek: 'invalid'. Supported: delta, gamma, vega, theta, rho"),
        (lambda: fd("gbm", gbm, "binary", 100.0, 1000, 10, ["delta"]),
         "Unknown payoff: 'binary'. Supported: 'call', 'put', or a callable"),
        (lambda: fd("gbm", gbm, 3.5, 100.0, 1000, 10, ["delta"]), "payoff must be 'call', 'put', or a callable"),
        (lambda: fd("gbm", {"s0": 100.0, "sigma": 0.2, "t": 1.0}, "call", 100.0, 1000, 10, ["delta"]),
         "Missing required param: 'r'"),
        (lambda: fd("heston", dict(gbm, v0=0.04, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, scheme="x"), "call", 100.0,
                    1000, 10, ["delta"]), "scheme must be 'euler' or 'qe'"),
        (lambda: stocha.greeks_pathwise(-1.0, 0.05, 0.2, 1.0, 100.0, True, 1000, 10, ["delta"]),
         "s0 must be positive"),
        (lambda: stocha.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, True, 0, 10, ["delta"]),
         "n_paths and n_steps must be positive"),
        (lambda: stocha.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, True, 1000, 10, ["gamma"]),
         "Pathwise method only supports 'delta' and 'vega', got 'gamma'"),
    ]
    for fn, msg in cases:
        with pytest.raises(ValueError) as ei:
            fn()
        assert str(ei.value) == msg


def test_lsmc_validation_messages(stocha):
    f = stocha.lsmc_american_option
    cases = [
        (lambda: f(-1.0, 100.0, 0.05, 0.2, 1.0, 10, 100), "s0 must be positive"),
        (lambda: f(100.0, 0.0, 0.05, 0.2, 1.0, 10, 100), "k must be positive"),
        (lambda: f(100.0, 100.0, 0.05, 0.0, 1.0, 10, 100), "sigma must be positive"),
        (lambda: f(100.0, 100.0, 0.05, 0.2, 0.0, 10, 100), "t must be positive"),
        (lambda: f(100.0, 100.0, 0.05, 0.2, 1.0, 0, 100), "steps and n_paths must be positive"),
        (lambda: f(100.0, 100.0, 0.05, 0.2, 1.0, 10, 1), "n_paths must be at least 2"),
        (lambda: f(100.0, 100.0, 0.05, 0.2, 1.0, 10, 100, poly_degree=0), "poly_degree must be in [1, 4]"),
        (lambda: f(100.0, 100.0, 0.05, 0.2, 1.0, 10, 100, poly_degree=5), "poly_degree must be in [1, 4]"),
    ]
    for fn, msg in cases:
        with pytest.raises(ValueError) as ei:
            fn()
        assert str(ei.value) == msg


def test_serving_arena_host_logic(stocha):
    """The serving loop's device-memory arena (first fit, 256-byte blocks,
    coalescing on release) on host-only scripts: no two live blocks overlap,
    every block is aligned and inside the budget, a full release coalesces
    back to one free block, and a request larger than the largest free block
    is refused."""
    import ctypes

    from stocha_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(5)
    cap = 1 << 20
    for trial in range(20):
        ops, live = [], []
        for i in range(400):
            if live and rng.random() < 0.45:
                k = live.pop(int(rng.integers(len(live))))
                ops.append(-k)
            else:
                ops.append(int(rng.integers(1, 60_000)))
                live.append(i)
        # then release everything still live
        ops += [-k for k in live]
        n = len(ops)
        a = np.array(ops, np.int64)
        res = np.zeros(n + 4, np.int64)
        P = ctypes.POINTER(ctypes.c_int64)
        assert lib.stocha_debug_arena(cap, a.ctypes.data_as(P), n, res.ctypes.data_as(P)) == 0
        blocks = {}
        for i, op in enumerate(ops):
            if op > 0 and res[i] >= 0:
                size = (op + 255) // 256 * 256
                off = int(res[i])
                assert off % 256 == 0 and off + size <= cap
                for o2, s2 in blocks.values():
                    assert off + size <= o2 or o2 + s2 <= off, "overlap"
                blocks[i] = (off, size)
            elif op <= 0:
                blocks.pop(-op, None)
        used, peak, largest, nfree = res[n:]
        assert used == 0 and peak <= cap and largest == cap and nfree == 1
    # refusal: two halves, free the first, a 3/4 request does not fit
    ops = np.array([cap // 2, cap // 2, -0, 3 * cap // 4], np.int64)
    ops[2] = 0  # releases allocation 0
    res = np.zeros(8, np.int64)
    P = ctypes.POINTER(ctypes.c_int64)
    lib.stocha_debug_arena(cap, ops.ctypes.data_as(P), 4, res.ctypes.data_as(P))
    assert res[0] == 0 and res[1] == cap // 2 and res[3] == -1


def test_tune_table_host_logic(stocha):
    """The fused-kernel launch-shape table: valid shapes are installed and read
    back, invalid ones are refused with ValueError (no GPU involved)."""
    before = stocha.tune_get("gbm")
    before_m3 = stocha.tune_get("multi_gbm", 3)
    try:
        stocha.tune_set("gbm", 128, 2, 2, variant=1)
        got = stocha.tune_get("gbm")
        assert (got["block"], got["ilp"], got["waves"], got["variant"]) == (128, 2, 2, 1)
        stocha.tune_set("gbm", 64, 1, 1, variant=2)
        assert stocha.tune_get("gbm")["variant"] == 2
        for bad in [(512, 1, 1, 1), (256, 3, 1, 1), (256, 1, 0, 1), (256, 1, 3, 1), (256, 2, 1, 0), (256, 2, 1, 2),
                    (256, 1, 1, 3), (256, 1, 1, -1)]:
            with pytest.raises(ValueError):
                stocha.tune_set("gbm", bad[0], bad[1], bad[2], variant=bad[3])
        with pytest.raises(ValueError):
            stocha.tune_get("multi_gbm", 9)  # more than 4 assets: generic kernel, no table slot
        stocha.tune_set("multi_gbm", 64, 1, 2, variant=0, n_assets=3)
        assert stocha.tune_get("multi_gbm", 3)["block"] == 64
    finally:
        stocha.tune_set("gbm", before["block"], before["ilp"], before["waves"], variant=before["variant"])
        stocha.tune_set("multi_gbm", before_m3["block"], before_m3["ilp"], before_m3["waves"],
                        variant=before_m3["variant"], n_assets=3)


def test_top_layer_always_rejects(stocha):
    """The warp-uniform FP32 sampler sends a failed attempt in the top layer
    (L = 255) to a state that only consumes its second draw, without a wedge
    test.  That rests on the reference's tables: the layer's fast threshold
    is 0 (X[256] = 0, normal.rs:25-27), so every top-layer attempt leaves the
    fast path, and its wedge test can never accept (Y[255] = Y[256] = 1, so
    y = 1 >= exp(-x^2/2), normal.rs:38-42).  Every other layer has a positive
    threshold."""
    from stocha_gb300 import _lib
    from tests.test_oracle import _table_from_inc

    lib = _lib.load()
    thr = np.zeros(256, np.uint64)
    lib.stocha_debug_zig_thresholds.argtypes = [_lib.P_u64]
    assert lib.stocha_debug_zig_thresholds(thr.ctypes.data_as(_lib.P_u64)) == 0
    _, X, Y = _table_from_inc()
    assert int(thr[255]) == 0 and X[256] == 0.0
    assert Y[255] == 1.0 and Y[256] == 1.0
    assert all(int(thr[L]) > 0 for L in range(255))


def test_greeks_batch_step_limit(stocha):
    """The FP32 batch kernel counts a path's normals in 32 bits: an FP32
    instance with 2^32 steps or more is a value error before any CUDA call."""
    inst = dict(model="gbm", s0=100.0, sigma=0.2, r=0.05, t=1.0, strike=100.0, n_paths=1000, steps=2**32)
    with pytest.raises(ValueError, match=r"instance 0: steps must be below 2\^32 in fp32"):
        stocha.greeks_batch([inst], precision="fp32")


def test_hull_white_validation(stocha):
    """hull_white's argument checks (lib.rs:617-636) happen before any CUDA call."""
    for kw, msg in [(dict(a=0.0), "a must be positive"), (dict(sigma=0.0), "sigma must be positive"),
                    (dict(t=0.0), "t must be positive"), (dict(steps=0), "steps and n_paths must be positive"),
                    (dict(n_paths=0), "steps and n_paths must be positive")]:
        args = dict(r0=0.05, a=0.1, theta=0.005, sigma=0.01, t=1.0, steps=12, n_paths=10)
        args.update(kw)
        with pytest.raises(ValueError, match=msg):
            stocha.hull_white(**args)


def test_var_cvar_validation(stocha):
    """var_cvar's checks on confidence and emptiness (lib.rs:507-517) come
    before any CUDA call; non-float64 input is a TypeError as in PyO3."""
    r = np.array([0.01, -0.02, 0.03])
    for c in (0.0, 1.0, -0.5, 1.5):
        with pytest.raises(ValueError, match=r"confidence must be in \(0, 1\)"):
            stocha.var_cvar(r, c)
    with pytest.raises(ValueError, match="returns must not be empty"):
        stocha.var_cvar(np.array([], np.float64), 0.95)
    with pytest.raises(TypeError):
        stocha.var_cvar(np.array([1, 2, 3], np.int64), 0.95)


def test_oracle_var_cvar_known_values(oracle):
    """The oracle against the reference's own unit tests (var_cvar.rs:50-75)."""
    v, c = oracle.var_cvar(np.array([-(i * 0.01) for i in range(1, 11)]), 0.9)
    assert abs(v - 0.10) < 1e-10 and abs(c - 0.10) < 1e-10
    v, c = oracle.var_cvar(np.array([i * 0.01 for i in range(1, 21)]), 0.95)
    assert v < 0 and c <= v + 1e-10


def test_gaussian_copula_validation(stocha):
    """gaussian_copula's matrix checks (copula/gaussian.rs:21-47, 76-99) with
    the reference's messages, before any CUDA call."""
    with pytest.raises(ValueError, match="correlation matrix must be square"):
        stocha.gaussian_copula(np.ones((2, 3)), 10)
    with pytest.raises(ValueError, match=r"diagonal element \[1\]\[1\] must be 1.0, got 0.9"):
        stocha.gaussian_copula(np.array([[1.0, 0.2], [0.2, 0.9]]), 10)
    with pytest.raises(ValueError, match=r"not symmetric: \[0,1\]=0.2 vs \[1,0\]=0.3"):
        stocha.gaussian_copula(np.array([[1.0, 0.2], [0.3, 1.0]]), 10)
    with pytest.raises(ValueError, match="matrix is not positive-definite"):
        stocha.gaussian_copula(np.array([[1.0, 1.5], [1.5, 1.0]]), 10)
    with pytest.raises(TypeError):
        stocha.gaussian_copula([[1.0, 0.0], [0.0, 1.0]], 10)


def test_student_t_copula_validation(stocha):
    """student_t_copula's checks (lib.rs:570-572, copula/student_t.rs:141-149)."""
    eye = np.eye(2)
    for nu in (2.0, 1.0, -3.0):
        with pytest.raises(ValueError, match="nu must be > 2"):
            stocha.student_t_copula(eye, nu, 10)
    with pytest.raises(ValueError, match="correlation matrix must be square"):
        stocha.student_t_copula(np.ones((2, 3)), 5.0, 10)
    with pytest.raises(ValueError, match="matrix is not positive-definite"):
        stocha.student_t_copula(np.array([[1.0, 1.5], [1.5, 1.0]]), 5.0, 10)
    with pytest.raises(TypeError):
        stocha.student_t_copula([[1.0, 0.0], [0.0, 1.0]], 5.0, 10)


def test_oracle_student_t_known_values(oracle):
    """The oracle against the reference's unit tests (copula/student_t.rs:175-200):
    CDF symmetry, and copula samples of shape (500, 2) inside (0, 1)."""
    assert abs(oracle.student_t_cdf(0.0, 5.0) - 0.5) < 1e-6
    assert abs(oracle.student_t_cdf(1.0, 5.0) + oracle.student_t_cdf(-1.0, 5.0) - 1.0) < 1e-5
    # published t-distribution quantiles: P(T_5 <= 2.015048) = 0.95, P(T_10 <= 2.763769) = 0.99
    assert abs(oracle.student_t_cdf(2.015048, 5.0) - 0.95) < 1e-5
    assert abs(oracle.student_t_cdf(2.763769, 10.0) - 0.99) < 1e-5
    u = oracle.student_t_copula(np.array([[1.0, 0.5], [0.5, 1.0]]), 5.0, 500, 42)
    assert u.shape == (500, 2) and np.all((u > 0) & (u < 1))

