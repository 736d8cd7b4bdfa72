"""ctypes wrapper of the CPU oracle (oracle/stocha_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it as the checker and as the timed CPU restatement of the
reference algorithm; the product package never imports it.

Every function mirrors one function of heki1224/stocha (Rust); see the
citations in stocha_oracle.cpp.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libstocha_oracle.so")
_lock = threading.Lock()
_lib = None

_u64 = ctypes.c_uint64
_dbl = ctypes.c_double
_int = ctypes.c_int
_pdbl = ctypes.POINTER(ctypes.c_double)
_pu64 = ctypes.POINTER(ctypes.c_uint64)
_pint = ctypes.POINTER(ctypes.c_int)

MODEL_CODES = {"gbm": 0, "heston": 1, "merton": 2}
GREEK_CODES = {"delta": 0, "gamma": 1, "vega": 2, "theta": 3, "rho": 4}
# parameter vector layout of oracle_terminal / oracle_greeks_fd
P_INDEX = {"s0": 0, "r": 1, "sigma": 2, "t": 3, "v0": 4, "kappa": 5, "theta": 6,
           "xi": 7, "rho": 8, "lambda_": 9, "mu_j": 10, "sigma_j": 11}


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -ffp-contract=off)."""
    with _lock:
        if force or not os.path.exists(_LIB_PATH):
            subprocess.run(["make", "-s", "-C", _HERE, "libstocha_oracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_pcg_seed.argtypes = [_u64, _u64, _pu64, _pu64]
        L.oracle_pcg_advance.argtypes = [_pu64, _pu64, _u64, _u64]
        L.oracle_pcg_fill_u64.argtypes = [_pu64, _pu64, _u64, _pu64]
        L.oracle_stream_fill.argtypes = [_pu64, _pu64, _int, _dbl, _dbl, _u64, _pdbl]
        L.oracle_stream_fill.restype = _u64
        L.oracle_gbm.argtypes = [_dbl, _dbl, _dbl, _dbl, _dbl, _u64, _u64, _int, _u64, _int, _int, _pdbl, _pu64]
        L.oracle_cholesky.argtypes = [_int, _pdbl, _pdbl, _pdbl]
        L.oracle_cholesky.restype = _int
        L.oracle_multi_gbm.argtypes = [_int, _pdbl, _pdbl, _pdbl, _pdbl, _dbl, _u64, _u64, _int, _u64, _int, _int,
                                       _pdbl, _pu64]
        L.oracle_multi_gbm.restype = _int
        L.oracle_heston.argtypes = [_dbl] * 8 + [_u64, _u64, _int, _u64, _int, _int, _pdbl, _pu64]
        L.oracle_merton.argtypes = [_dbl] * 7 + [_u64, _u64, _u64, _int, _int, _pdbl, _pu64]
        L.oracle_lsmc.argtypes = [_dbl] * 5 + [_u64, _u64, _int, _int, _u64, _int, _int, _pdbl, _pdbl, _pdbl]
        L.oracle_terminal.argtypes = [_int, _pdbl, _int, _u64, _u64, _u64, _int, _pdbl]
        L.oracle_mc_price.argtypes = [_int, _pdbl, _int, _int, _dbl, _u64, _u64, _u64, _int]
        L.oracle_mc_price.restype = _dbl
        L.oracle_greeks_fd.argtypes = [_int, _pdbl, _int, _int, _dbl, _u64, _u64, _pint, _int, _u64, _dbl, _int,
                                       _pdbl]
        L.oracle_greeks_pathwise.argtypes = [_dbl] * 5 + [_int, _u64, _u64, _pint, _int, _u64, _int, _pdbl]
        L.oracle_barrier_mc.argtypes = [_dbl] * 7 + [_int, _int, _int, _dbl, _int, _u64, _u64, _u64, _int]
        L.oracle_barrier_mc.restype = _dbl
        L.oracle_asian_paths.argtypes = [_dbl] * 6 + [_u64, _int, _int, _u64, _u64, _int, _pdbl, _pdbl]
        L.oracle_asian_estimate.argtypes = [_pdbl, _pdbl, _u64, _int, _dbl, _dbl]
        L.oracle_asian_estimate.restype = _dbl
        L.oracle_asian_floating_seasoned.argtypes = [_dbl] * 5 + [_u64, _int, _int, _dbl, _dbl, _u64, _u64, _int]
        L.oracle_asian_floating_seasoned.restype = _dbl
        L.oracle_lookback_mc.argtypes = [_dbl] * 6 + [_u64, _int, _int, _dbl, _dbl, _u64, _u64, _int]
        L.oracle_lookback_mc.restype = _dbl
        L.oracle_hull_white.argtypes = [_dbl] * 5 + [_u64, _u64, _u64, _int, _pdbl]
        L.oracle_var_cvar.argtypes = [_pdbl, _u64, _dbl, _pdbl]
        L.oracle_gaussian_copula.argtypes = [_pdbl, _int, _u64, _u64, _pdbl]
        L.oracle_gaussian_copula.restype = _int
        L.oracle_student_t_copula.argtypes = [_pdbl, _int, _dbl, _u64, _u64, _pdbl]
        L.oracle_student_t_copula.restype = _int
        L.oracle_student_t_cdf.argtypes = [_dbl, _dbl]
        L.oracle_student_t_cdf.restype = _dbl
        _lib = L
    return _lib


def _p(a, t=_pdbl):
    return a.ctypes.data_as(t) if a is not None else None


# ------------------------------------------------------------------ PCG ----
def _split(x: int):
    return x & (2**64 - 1), x >> 64


def _join(a) -> int:
    return int(a[0]) | (int(a[1]) << 64)


def pcg_seed(seed: int):
    """(state, inc) of Pcg64Dxsm::new(seed) (src/prng/pcg64.rs:23-30)."""
    st = np.zeros(2, np.uint64)
    inc = np.zeros(2, np.uint64)
    lo, hi = _split(seed)
    lib().oracle_pcg_seed(lo, hi, _p(st, _pu64), _p(inc, _pu64))
    return _join(st), _join(inc)


def pcg_advance(state: int, inc: int, delta: int) -> int:
    st = np.array(_split(state), np.uint64)
    ic = np.array(_split(inc), np.uint64)
    lo, hi = _split(delta)
    lib().oracle_pcg_advance(_p(st, _pu64), _p(ic, _pu64), lo, hi)
    return _join(st)


def pcg_u64(state: int, inc: int, n: int) -> np.ndarray:
    st = np.array(_split(state), np.uint64)
    ic = np.array(_split(inc), np.uint64)
    out = np.empty(n, np.uint64)
    lib().oracle_pcg_fill_u64(_p(st, _pu64), _p(ic, _pu64), n, _p(out, _pu64))
    return out


def stream_fill(state: int, inc: int, kind: str, n: int, loc=0.0, scale=1.0):
    """Sequential draws of one stream: returns (values, u64 consumed, new state)."""
    st = np.array(_split(state), np.uint64)
    ic = np.array(_split(inc), np.uint64)
    out = np.empty(n, np.float64)
    code = {"uniform": 0, "standard_normal": 1, "normal": 2}[kind]
    used = lib().oracle_stream_fill(_p(st, _pu64), _p(ic, _pu64), code, loc, scale, n, _p(out))
    return out, int(used), _join(st)


# --------------------------------------------------------------- models ----
def gbm(s0, mu, sigma, t, steps, n_paths, seed=42, antithetic=False, q=0.0, threads=0, gather=False,
        with_used=False):
    out = np.empty((n_paths, steps + 1), np.float64)
    used = np.empty(n_paths, np.uint64) if with_used else None
    lib().oracle_gbm(s0, mu, sigma, q, t, steps, n_paths, int(antithetic), seed, threads, int(gather), _p(out),
                     _p(used, _pu64))
    return (out, used) if with_used else out


def cholesky(a):
    a = np.ascontiguousarray(a, np.float64)
    n = a.shape[0]
    l = np.empty_like(a)
    bad = np.zeros(1)
    rc = lib().oracle_cholesky(n, _p(a), _p(l), _p(bad))
    if rc:
        raise ValueError(f"matrix is not positive-definite (diagonal element {rc - 1} = {bad[0]})")
    return l


def multi_gbm(s0, mu, sigma, corr, t, steps, n_paths, seed=42, antithetic=False, threads=0, gather=False,
              with_used=False):
    s0 = np.ascontiguousarray(s0, np.float64)
    mu = np.ascontiguousarray(mu, np.float64)
    sigma = np.ascontiguousarray(sigma, np.float64)
    corr = np.ascontiguousarray(corr, np.float64)
    na = s0.shape[0]
    out = np.empty((n_paths, steps + 1, na), np.float64)
    used = np.empty(n_paths, np.uint64) if with_used else None
    rc = lib().oracle_multi_gbm(na, _p(s0), _p(mu), _p(sigma), _p(corr), t, steps, n_paths, int(antithetic), seed,
                                threads, int(gather), _p(out), _p(used, _pu64))
    if rc:
        raise ValueError("matrix is not positive-definite")
    return (out, used) if with_used else out


def heston(s0, v0, mu, kappa, theta, xi, rho, t, steps, n_paths, seed=42, scheme="euler", threads=0,
           gather=False, with_used=False):
    out = np.empty((n_paths, steps + 1), np.float64)
    used = np.empty(n_paths, np.uint64) if with_used else None
    lib().oracle_heston(s0, v0, mu, kappa, theta, xi, rho, t, steps, n_paths, 0 if scheme == "euler" else 1, seed,
                        threads, int(gather), _p(out), _p(used, _pu64))
    return (out, used) if with_used else out


def merton(s0, mu, sigma, lambda_, mu_j, sigma_j, t, steps, n_paths, seed=42, threads=0, gather=False,
           with_used=False):
    out = np.empty((n_paths, steps + 1), np.float64)
    used = np.empty(n_paths, np.uint64) if with_used else None
    lib().oracle_merton(s0, mu, sigma, lambda_, mu_j, sigma_j, t, steps, n_paths, seed, threads, int(gather),
                        _p(out), _p(used, _pu64))
    return (out, used) if with_used else out


def lsmc(s0, k, r, sigma, t, steps, n_paths, is_put=True, poly_degree=3, seed=42, solver="qr", threads=0,
         paths=None):
    price = np.zeros(1)
    se = np.zeros(1)
    pp = None
    if paths is not None:
        pp = np.ascontiguousarray(paths, np.float64)
        assert pp.shape == (n_paths, steps + 1)
    lib().oracle_lsmc(s0, k, r, sigma, t, steps, n_paths, int(is_put), poly_degree, seed,
                      0 if solver == "qr" else 1, threads, _p(pp), _p(price), _p(se))
    return float(price[0]), float(se[0])


def _pvec(model: str, params: dict) -> np.ndarray:
    p = np.zeros(12, np.float64)
    for key, val in params.items():
        if key in P_INDEX:
            p[P_INDEX[key]] = float(val)
    return p


def terminal(model, params, steps, n_paths, seed=42, threads=0):
    p = _pvec(model, params)
    out = np.empty(n_paths, np.float64)
    scheme = 1 if params.get("scheme", "euler") == "qe" else 0
    lib().oracle_terminal(MODEL_CODES[model], _p(p), scheme, steps, n_paths, seed, threads, _p(out))
    return out


def greeks_fd(model, params, payoff, strike, n_paths, n_steps, greeks, seed=42, bump_size=0.01, threads=0):
    p = _pvec(model, params)
    codes = np.array([GREEK_CODES[g] for g in greeks], np.int32)
    out = np.empty(len(greeks), np.float64)
    scheme = 1 if params.get("scheme", "euler") == "qe" else 0
    lib().oracle_greeks_fd(MODEL_CODES[model], _p(p), scheme, 0 if payoff == "call" else 1, strike, n_paths,
                           n_steps, _p(codes, _pint), len(greeks), seed, bump_size, threads, _p(out))
    return {g: float(v) for g, v in zip(greeks, out)}


def greeks_pathwise(s0, r, sigma, t, strike, is_call, n_paths, n_steps, greeks, seed=42, threads=0):
    codes = np.array([GREEK_CODES[g] for g in greeks], np.int32)
    out = np.empty(len(greeks), np.float64)
    lib().oracle_greeks_pathwise(s0, r, sigma, t, strike, int(is_call), n_paths, n_steps, _p(codes, _pint),
                                 len(greeks), seed, threads, _p(out))
    return {g: float(v) for g, v in zip(greeks, out)}


# ---------------------------------------------------------- exotic MC ---
_DIR = {"up-and-out": (0, 0), "uo": (0, 0), "up-and-in": (0, 1), "ui": (0, 1), "down-and-out": (1, 0),
        "do": (1, 0), "down-and-in": (1, 1), "di": (1, 1)}


def barrier_mc(s, k, r, sigma, t, barrier, barrier_type="up-and-out", option_type="call", q=0.0, n_paths=100_000,
               n_steps=252, seed=42, rebate=0.0, rebate_at_hit=False, threads=0):
    """barrier.rs:286-372 barrier_mc."""
    d, kin = _DIR[barrier_type]
    return lib().oracle_barrier_mc(s, k, r, q, sigma, t, barrier, d, kin, int(option_type == "call"), rebate,
                                   int(rebate_at_hit), n_paths, n_steps, seed, threads)


def asian_paths(s, k, r, sigma, t, n_steps, strike_type="fixed", option_type="call", q=0.0, n_paths=100_000,
                seed=42, threads=0):
    """Per-path (arithmetic, geometric) payoffs of asian.rs:143-268."""
    a = np.empty(n_paths)
    g = np.empty(n_paths)
    lib().oracle_asian_paths(s, k, r, q, sigma, t, n_steps, int(strike_type == "floating"),
                             int(option_type == "call"), n_paths, seed, threads, _p(a), _p(g))
    return a, g


def asian_estimate(arith, geo, use_cv, geo_analytical, discount):
    """asian.rs:270-289: the control-variate (or plain) estimator."""
    a = np.ascontiguousarray(arith, np.float64)
    g = np.ascontiguousarray(geo, np.float64)
    return lib().oracle_asian_estimate(_p(a), _p(g), a.size, int(use_cv), geo_analytical, discount)


def asian_floating_seasoned(s, r, sigma, t, n_steps, average_type, option_type, a_spent, t1, q=0.0,
                            n_paths=100_000, seed=42, threads=0):
    """asian.rs:292-352 asian_mc_floating_seasoned."""
    return lib().oracle_asian_floating_seasoned(s, r, q, sigma, t, n_steps, int(average_type == "geometric"),
                                                int(option_type == "call"), a_spent, t1, n_paths, seed, threads)


def lookback_mc(s, r, sigma, t, n_steps=252, strike_type="floating", option_type="call", k=0.0, q=0.0,
                n_paths=100_000, seed=42, running_max=None, running_min=None, threads=0):
    """lookback.rs:158-210 lookback_mc."""
    nan = float("nan")
    return lib().oracle_lookback_mc(s, k, r, q, sigma, t, n_steps, int(strike_type == "fixed"),
                                    int(option_type == "call"), nan if running_max is None else running_max,
                                    nan if running_min is None else running_min, n_paths, seed, threads)


def hull_white(r0, a, theta, sigma, t, steps, n_paths, seed=42, threads=0):
    """hull_white.rs:26-57 hull_white_paths."""
    out = np.empty((n_paths, steps + 1), np.float64)
    lib().oracle_hull_white(r0, a, theta, sigma, t, steps, n_paths, seed, threads, _p(out))
    return out


def var_cvar(returns, confidence):
    """var_cvar.rs:7-43 (sort by total_cmp, VaR at rank ceil(c n), CVaR = tail mean)."""
    r = np.ascontiguousarray(returns, np.float64)
    out = np.zeros(2)
    lib().oracle_var_cvar(_p(r), r.size, confidence, _p(out))
    return float(out[0]), float(out[1])


def gaussian_copula(corr, n_samples, seed=42):
    """copula/gaussian.rs:15-73 gaussian_copula_samples."""
    c = np.ascontiguousarray(corr, np.float64)
    out = np.empty((n_samples, c.shape[0]))
    assert lib().oracle_gaussian_copula(_p(c), c.shape[0], n_samples, seed, _p(out)) == 0
    return out


def student_t_copula(corr, nu, n_samples, seed=42):
    """copula/student_t.rs:135-170 student_t_copula_samples."""
    c = np.ascontiguousarray(corr, np.float64)
    out = np.empty((n_samples, c.shape[0]))
    assert lib().oracle_student_t_copula(_p(c), c.shape[0], nu, n_samples, seed, _p(out)) == 0
    return out


def student_t_cdf(x, nu):
    """copula/student_t.rs:8-16 (incomplete beta by modified Lentz, Lanczos log-gamma)."""
    return lib().oracle_student_t_cdf(float(x), float(nu))

