"""The extension-module surface of stocha (`stocha._stocha`, src/lib.rs) over
the C ABI of libstocha_gpu.so.

Each function keeps the reference's name, keyword signature, defaults, return
type and error behaviour: argument conversion errors are TypeError /
OverflowError as PyO3 raises them, and invalid values raise ValueError with
the reference's message (the message comes from the C++ host library).
The GIL is released during every call (ctypes does that), as `py.detach`
does in the reference.
"""
from __future__ import annotations

import ctypes
import operator
import weakref

import numpy as np

from . import _lib
from ._lib import check, dptr, load

__version__ = "1.7.1"  # lib.rs:1879

_U64_MAX = 2**64 - 1
_U128_MAX = 2**128 - 1


# --------------------------------------------------------- result arrays --
_CACHE_MIN = 1 << 20  # smaller results go to plain NumPy memory


def _release(addr):
    try:
        load().stocha_host_buffer_release(ctypes.c_void_p(addr))
    except Exception:  # interpreter shutdown: the process unmaps everything anyway
        pass


def _host_array(shape, dtype=np.float64):
    """A result array in the library's host-buffer cache: when it dies, its
    pages (which exist by then) are kept for a later result of a similar size,
    so that result's copy from the device skips the page faults of fresh memory
    (stocha_host_buffer_acquire in stocha_gpu.h)."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
    if nbytes < _CACHE_MIN:
        return np.empty(shape, dt)
    p = ctypes.c_void_p()
    check(load().stocha_host_buffer_acquire(nbytes, ctypes.byref(p)))
    raw = (ctypes.c_char * nbytes).from_address(p.value)
    weakref.finalize(raw, _release, p.value).atexit = False
    return np.frombuffer(raw, dtype=dt).reshape(shape)


# ---------------------------------------------------- PyO3-like conversion --
def _f64(x, name="argument"):
    if isinstance(x, (str, bytes)):
        raise TypeError(f"argument '{name}': must be real number, not {type(x).__name__}")
    return float(x)


def _uint(x, limit, name="argument"):
    if isinstance(x, bool):
        x = int(x)
    try:
        v = operator.index(x)
    except TypeError:
        raise TypeError(f"argument '{name}': '{type(x).__name__}' object cannot be interpreted as an integer")
    if v < 0:
        raise OverflowError(f"argument '{name}': can't convert negative int to unsigned")
    if v > limit:
        raise OverflowError(f"argument '{name}': int too big to convert")
    return v


def _usize(x, name="argument"):
    return _uint(x, _U64_MAX, name)


def _bool(x, name="argument"):
    if isinstance(x, (bool, np.bool_)):
        return bool(x)
    raise TypeError(f"argument '{name}': '{type(x).__name__}' object cannot be converted to 'PyBool'")


def _str(x, name="argument"):
    if not isinstance(x, str):
        raise TypeError(f"argument '{name}': '{type(x).__name__}' object cannot be converted to 'PyString'")
    return x


# ---------------------------------------------------------------- RNG ------
class RNG:
    """Python-accessible random number generator backed by PCG64DXSM
    (lib.rs:74-184).  The 48-byte state lives on the host; draws are
    generated on the GPU and the state advances exactly as the reference's
    sequential generator does."""

    def __init__(self, seed=0, algorithm="pcg64dxsm"):
        seed = _uint(seed, _U128_MAX, "seed")
        algorithm = _str(algorithm, "algorithm")
        self._st = _lib.StochaRng()
        check(load().stocha_rng_new(seed & _U64_MAX, seed >> 64, algorithm.encode(), ctypes.byref(self._st)))

    @property
    def seed(self) -> int:
        return self._st.seed_lo | (self._st.seed_hi << 64)

    def _fill(self, fn, size, *extra):
        size = _usize(size, "size")
        out = _host_array(size, np.float64)
        check(fn(None, ctypes.byref(self._st), size, *extra, dptr(out)))
        return out

    def uniform(self, size):
        return self._fill(load().stocha_rng_uniform, size)

    def standard_normal(self, size):
        return self._fill(load().stocha_rng_standard_normal, size)

    def normal(self, size, loc=0.0, scale=1.0):
        return self._fill(load().stocha_rng_normal, size, _f64(loc, "loc"), _f64(scale, "scale"))

    def raw_u64(self, size):
        """Raw generator words (no counterpart in the reference API)."""
        size = _usize(size, "size")
        out = _host_array(size, np.uint64)
        check(load().stocha_rng_raw_u64(None, ctypes.byref(self._st), size, out.ctypes.data_as(_lib.P_u64)))
        return out

    def save_state(self) -> str:
        n = ctypes.c_size_t(0)
        buf = ctypes.create_string_buffer(256)
        check(load().stocha_rng_save_state(ctypes.byref(self._st), buf, 256, ctypes.byref(n)))
        return buf.value.decode()

    @staticmethod
    def from_state(json) -> "RNG":
        json = _str(json, "json")
        obj = RNG.__new__(RNG)
        obj._st = _lib.StochaRng()
        check(load().stocha_rng_from_state(json.encode(), ctypes.byref(obj._st)))
        return obj

    def __repr__(self) -> str:
        return f"RNG(seed={self.seed}, algorithm='pcg64dxsm')"


# ------------------------------------------------------------- models ------
def gbm(s0, mu, sigma, t, steps, n_paths, seed=42, antithetic=False, q=0.0):
    """lib.rs:205-252: (n_paths, steps + 1) float64 GBM paths."""
    args = (_f64(s0, "s0"), _f64(mu, "mu"), _f64(sigma, "sigma"), _f64(t, "t"))
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    seed, anti, q = _usize(seed, "seed"), _bool(antithetic, "antithetic"), _f64(q, "q")
    out = _alloc(n_paths, steps + 1, args[0] > 0 and args[2] > 0 and args[3] > 0)
    check(load().stocha_gbm(None, *args, steps, n_paths, seed, int(anti), q, dptr(out)))
    return out


def heston(s0, v0, mu, kappa, theta, xi, rho, t, steps, n_paths, seed=42, scheme="euler"):
    """lib.rs:327-408: (n_paths, steps + 1) float64 Heston paths."""
    vals = [_f64(v, n) for v, n in zip((s0, v0, mu, kappa, theta, xi, rho, t),
                                       ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t"))]
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    seed, scheme = _usize(seed, "seed"), _str(scheme, "scheme")
    out = _alloc(n_paths, steps + 1, True)
    check(load().stocha_heston(None, *vals, steps, n_paths, seed, scheme.encode(), dptr(out)))
    return out


def merton_jump_diffusion(s0, mu, sigma, lambda_, mu_j, sigma_j, t, steps, n_paths, seed=42):
    """lib.rs:430-489: (n_paths, steps + 1) float64 Merton paths."""
    vals = [_f64(v, n) for v, n in zip((s0, mu, sigma, lambda_, mu_j, sigma_j, t),
                                       ("s0", "mu", "sigma", "lambda_", "mu_j", "sigma_j", "t"))]
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    seed = _usize(seed, "seed")
    out = _alloc(n_paths, steps + 1, True)
    check(load().stocha_merton_jump_diffusion(None, *vals, steps, n_paths, seed, dptr(out)))
    return out


def hull_white(r0, a, theta, sigma, t, steps, n_paths, seed=42):
    """lib.rs:604-649: (n_paths, steps + 1) float64 Hull-White short-rate paths
    by the exact transition; column 0 is r0."""
    vals = [_f64(v, n) for v, n in zip((r0, a, theta, sigma, t), ("r0", "a", "theta", "sigma", "t"))]
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    seed = _usize(seed, "seed")
    out = _alloc(n_paths, steps + 1, vals[1] > 0 and vals[3] > 0 and vals[4] > 0)
    check(load().stocha_hull_white(None, *vals, steps, n_paths, seed, dptr(out)))
    return out


def multi_gbm(s0, mu, sigma, corr, t, steps, n_paths, seed=42, antithetic=False):
    """lib.rs:759-827: (n_paths, steps + 1, n_assets) float64 paths."""
    s0 = np.ascontiguousarray([_f64(v, "s0") for v in s0], np.float64)
    mu = np.ascontiguousarray([_f64(v, "mu") for v in mu], np.float64)
    sigma = np.ascontiguousarray([_f64(v, "sigma") for v in sigma], np.float64)
    if not isinstance(corr, np.ndarray) or corr.ndim != 2 or corr.dtype != np.float64:
        raise TypeError("argument 'corr': must be a 2-D float64 numpy.ndarray")
    corr_c = np.ascontiguousarray(corr)
    t = _f64(t, "t")
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    seed, anti = _usize(seed, "seed"), _bool(antithetic, "antithetic")
    n = s0.shape[0]
    if n > 0 and (mu.shape[0] != n or sigma.shape[0] != n):
        raise ValueError("s0, mu, sigma must have the same length")  # lib.rs:777-781
    ok = n > 0 and corr_c.shape == (n, n)
    out = _alloc(n_paths, steps + 1, ok, n)
    check(load().stocha_multi_gbm(None, n, dptr(s0), dptr(mu), dptr(sigma), dptr(corr_c), corr_c.shape[0],
                                  corr_c.shape[1], t, steps, n_paths, seed, int(anti), dptr(out)))
    return out


def lsmc_american_option(s0, k, r, sigma, t, steps, n_paths, is_put=True, poly_degree=3, seed=42,
                         precision="fp64"):
    """lib.rs:854-918: (price, std_err) of an American option by LSMC.
    ``precision="fp32"`` (no counterpart in the reference) runs the paths in
    FP32; the regression stays FP64."""
    vals = [_f64(v, nm) for v, nm in zip((s0, k, r, sigma, t), ("s0", "k", "r", "sigma", "t"))]
    steps, n_paths = _usize(steps, "steps"), _usize(n_paths, "n_paths")
    is_put, deg, seed = _bool(is_put, "is_put"), _usize(poly_degree, "poly_degree"), _usize(seed, "seed")
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    price, se = ctypes.c_double(0.0), ctypes.c_double(0.0)
    if precision == "fp64":
        check(load().stocha_lsmc_american_option(None, *vals, steps, n_paths, int(is_put), deg, seed,
                                                 ctypes.byref(price), ctypes.byref(se)))
    else:
        check(load().stocha_lsmc(None, *vals, steps, n_paths, int(is_put), deg, seed,
                                 _lib.FP32 if precision == "fp32" else -1, ctypes.byref(price), ctypes.byref(se)))
    return float(price.value), float(se.value)


_GREEK_NAMES = ("delta", "gamma", "vega", "theta", "rho")
_PARAM_KEYS = ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j")
_MODEL_KEYS = {  # lib.rs:964-1033, in extraction order
    "gbm": ("s0", "r", "sigma", "t"),
    "heston": ("s0", "v0", "r", "kappa", "theta", "xi", "rho", "t"),
    "merton": ("s0", "r", "sigma", "lambda_", "mu_j", "sigma_j", "t"),
}


def _greek_list(greeks):
    if not isinstance(greeks, list):
        raise TypeError(f"argument 'greeks': '{type(greeks).__name__}' object cannot be converted to 'PyList'")
    names = [_str(g, "greeks") for g in greeks]
    for g in names:  # lib.rs:920-938
        if g not in _GREEK_NAMES:
            raise ValueError(f"Unknown greek: '{g}'. Supported: delta, gamma, vega, theta, rho")
    arr = (ctypes.c_char_p * max(len(names), 1))(*[g.encode() for g in names])
    return names, arr


def _greek_params(model, params):
    if not isinstance(params, dict):
        raise TypeError(f"argument 'params': '{type(params).__name__}' object cannot be converted to 'PyDict'")
    p = _lib.StochaGreeksParams()
    p.present = 0
    p.scheme = 0
    for key in _MODEL_KEYS.get(model, ()):  # lib.rs:951-956 extract_f64
        if key not in params:
            raise ValueError(f"Missing required param: '{key}'")
        setattr(p, key, _f64(params[key], key))
        p.present |= 1 << _PARAM_KEYS.index(key)
    if model == "heston" and "scheme" in params:
        s = _str(params["scheme"], "scheme")
        p.scheme = 0 if s == "euler" else 1 if s == "qe" else -1
    return p


def greeks_fd(model, params, payoff, strike, n_paths, n_steps, greeks, seed=42, bump_size=0.01, precision="fp64"):
    """lib.rs:1064-1156: dict of bump-and-revalue Greeks with common random
    numbers.  ``payoff`` is "call", "put" or a callable f(terminals) -> values
    (called once per scenario with the terminal prices, as the reference
    does).  ``precision="fp32"`` (no counterpart in the reference) prices all
    scenarios of each path in one FP32 pass."""
    model = _str(model, "model")
    strike = _f64(strike, "strike")
    n_paths, n_steps = _usize(n_paths, "n_paths"), _usize(n_steps, "n_steps")
    seed, bump_size = _usize(seed, "seed"), _f64(bump_size, "bump_size")
    if not isinstance(params, dict):
        raise TypeError(f"argument 'params': '{type(params).__name__}' object cannot be converted to 'PyDict'")
    names, arr = _greek_list(greeks)
    p = _greek_params(model, params)
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    out = np.zeros(max(len(names), 1), np.float64)
    pay_name, cb, err = None, _lib.PAYOFF_FN(), []
    if isinstance(payoff, str):
        pay_name = payoff.encode()
    elif callable(payoff):
        def _cb(user, terms, n, sum_out, len_out):
            try:
                t = np.ctypeslib.as_array(terms, shape=(n,)).copy() if n else np.empty(0, np.float64)
                vals = np.asarray([float(v) for v in payoff(t)], np.float64)
                sum_out[0] = float(np.cumsum(vals)[-1]) if vals.size else 0.0  # sequential sum
                len_out[0] = int(vals.size)
                return 0
            except BaseException as e:  # re-raised below
                err.append(e)
                return 1
        cb = _lib.PAYOFF_FN(_cb)
    rc = load().stocha_greeks_fd(None, model.encode(), ctypes.byref(p), pay_name, cb, None, strike, n_paths, n_steps,
                                 arr, len(names), seed, bump_size, _lib.FP32 if precision == "fp32" else _lib.FP64,
                                 dptr(out))
    if err:
        raise err[0]
    check(rc)
    return {g: float(v) for g, v in zip(names, out)}


def greeks_pathwise(s0, r, sigma, t, strike, is_call, n_paths, n_steps, greeks, seed=42):
    """lib.rs:1177-1242: pathwise (IPA) delta and vega for GBM."""
    vals = [_f64(v, nm) for v, nm in zip((s0, r, sigma, t, strike), ("s0", "r", "sigma", "t", "strike"))]
    is_call = _bool(is_call, "is_call")
    n_paths, n_steps, seed = _usize(n_paths, "n_paths"), _usize(n_steps, "n_steps"), _usize(seed, "seed")
    if not isinstance(greeks, list):
        raise TypeError(f"argument 'greeks': '{type(greeks).__name__}' object cannot be converted to 'PyList'")
    names = [_str(g, "greeks") for g in greeks]
    arr = (ctypes.c_char_p * max(len(names), 1))(*[g.encode() for g in names])
    out = np.zeros(max(len(names), 1), np.float64)
    check(load().stocha_greeks_pathwise(None, *vals, int(is_call), n_paths, n_steps, arr, len(names), seed, dptr(out)))
    return {g: float(v) for g, v in zip(names, out)}


def _alloc(n_paths, cols, plausible, n_assets=None):
    """Output array; tiny placeholder when validation is about to fail."""
    if not plausible or n_paths == 0 or cols <= 1:
        shape = (0, 0) if n_assets is None else (0, 0, 0)
        return np.empty(shape, np.float64)
    shape = (n_paths, cols) if n_assets is None else (n_paths, cols, n_assets)
    return _host_array(shape, np.float64)


# ------------------------------------------------------- exotic options ---
def _opt_f64(x, name):
    return float("nan") if x is None else _f64(x, name)


def _exotic_precision(precision):
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    return _lib.FP32 if precision == "fp32" else _lib.FP64


def barrier_price(s, k, r, sigma, t, barrier, barrier_type="up-and-out", option_type="call", q=0.0,
                  n_paths=100_000, n_steps=252, seed=42, method="auto", n_monitoring=None, rebate=0.0,
                  rebate_at_hit=False, precision="fp64"):
    """lib.rs:1549-1641: barrier option price (analytical or Monte Carlo).
    ``precision="fp32"`` (no counterpart in the reference) runs the Monte
    Carlo paths in FP32 log space on the same draws."""
    prec = _exotic_precision(precision)
    vals = [_f64(v, nm) for v, nm in zip((s, k, r, sigma, t, barrier), ("s", "k", "r", "sigma", "t", "barrier"))]
    barrier_type, option_type = _str(barrier_type, "barrier_type"), _str(option_type, "option_type")
    q = _f64(q, "q")
    n_paths, n_steps, seed = _usize(n_paths, "n_paths"), _usize(n_steps, "n_steps"), _usize(seed, "seed")
    method = _str(method, "method")
    n_mon = -1 if n_monitoring is None else _uint(n_monitoring, 2**32 - 1, "n_monitoring")
    rebate, rebate_at_hit = _f64(rebate, "rebate"), _bool(rebate_at_hit, "rebate_at_hit")
    out = ctypes.c_double(0.0)
    check(load().stocha_barrier_price(None, *vals, barrier_type.encode(), option_type.encode(), q, n_paths, n_steps,
                                      seed, method.encode(), n_mon, rebate, int(rebate_at_hit), prec,
                                      ctypes.byref(out)))
    return float(out.value)


def asian_price(s, k, r, sigma, t, n_steps=252, average_type="arithmetic", strike_type="fixed", option_type="call",
                q=0.0, n_paths=100_000, seed=42, method="auto", running_avg=None, time_elapsed=None,
                precision="fp64"):
    """lib.rs:1643-1757: Asian option price (Kemna-Vorst or Monte Carlo).
    ``precision="fp32"``: the Monte Carlo paths in FP32 (a GB300 addition)."""
    prec = _exotic_precision(precision)
    vals = [_f64(v, nm) for v, nm in zip((s, k, r, sigma, t), ("s", "k", "r", "sigma", "t"))]
    n_steps = _usize(n_steps, "n_steps")
    average_type, strike_type = _str(average_type, "average_type"), _str(strike_type, "strike_type")
    option_type, q = _str(option_type, "option_type"), _f64(q, "q")
    n_paths, seed, method = _usize(n_paths, "n_paths"), _usize(seed, "seed"), _str(method, "method")
    out = ctypes.c_double(0.0)
    check(load().stocha_asian_price(None, *vals, n_steps, average_type.encode(), strike_type.encode(),
                                    option_type.encode(), q, n_paths, seed, method.encode(),
                                    _opt_f64(running_avg, "running_avg"), _opt_f64(time_elapsed, "time_elapsed"),
                                    prec, ctypes.byref(out)))
    return float(out.value)


def lookback_price(s, r, sigma, t, n_steps=252, strike_type="floating", option_type="call", k=0.0, q=0.0,
                   n_paths=100_000, seed=42, method="auto", running_max=None, running_min=None, precision="fp64"):
    """lib.rs:1759-1870: lookback option price (GSG / Conze-Viswanathan or Monte Carlo).
    ``precision="fp32"``: the Monte Carlo paths in FP32 (a GB300 addition)."""
    prec = _exotic_precision(precision)
    vals = [_f64(v, nm) for v, nm in zip((s, r, sigma, t), ("s", "r", "sigma", "t"))]
    n_steps = _usize(n_steps, "n_steps")
    strike_type, option_type = _str(strike_type, "strike_type"), _str(option_type, "option_type")
    k, q = _f64(k, "k"), _f64(q, "q")
    n_paths, seed, method = _usize(n_paths, "n_paths"), _usize(seed, "seed"), _str(method, "method")
    out = ctypes.c_double(0.0)
    check(load().stocha_lookback_price(None, *vals, n_steps, strike_type.encode(), option_type.encode(), k, q, n_paths,
                                       seed, method.encode(), _opt_f64(running_max, "running_max"),
                                       _opt_f64(running_min, "running_min"), prec, ctypes.byref(out)))
    return float(out.value)


# ------------------------------------------------------------ copulas ------
def gaussian_copula(corr, n_samples, seed=42):
    """lib.rs:522-549: (n_samples, dim) uniforms of a Gaussian copula."""
    if not isinstance(corr, np.ndarray) or corr.ndim != 2 or corr.dtype != np.float64:
        raise TypeError("argument 'corr': must be a 2-D float64 numpy.ndarray")
    n_samples, seed = _usize(n_samples, "n_samples"), _usize(seed, "seed")
    c = np.ascontiguousarray(corr)
    rows, cols = c.shape
    out = _host_array((n_samples, rows) if rows == cols else (0, 0), np.float64)
    check(load().stocha_gaussian_copula(None, dptr(c) if c.size else None, rows, cols, n_samples, seed,
                                        dptr(out) if out.size else None))
    return out


def student_t_copula(corr, nu, n_samples, seed=42):
    """lib.rs:551-578: (n_samples, dim) uniforms of a Student-t copula."""
    if not isinstance(corr, np.ndarray) or corr.ndim != 2 or corr.dtype != np.float64:
        raise TypeError("argument 'corr': must be a 2-D float64 numpy.ndarray")
    nu = _f64(nu, "nu")
    n_samples, seed = _usize(n_samples, "n_samples"), _usize(seed, "seed")
    c = np.ascontiguousarray(corr)
    rows, cols = c.shape
    out = _host_array((n_samples, rows) if rows == cols and not nu <= 2.0 else (0, 0), np.float64)
    check(load().stocha_student_t_copula(None, dptr(c) if c.size else None, rows, cols, nu, n_samples, seed,
                                         dptr(out) if out.size else None))
    return out


# -------------------------------------------------------------- risk -------
def var_cvar(returns, confidence):
    """lib.rs:505-520: (VaR, CVaR) of the losses -returns at `confidence`."""
    if not isinstance(returns, np.ndarray) or returns.ndim != 1 or returns.dtype != np.float64:
        raise TypeError("argument 'returns': must be a 1-D float64 numpy.ndarray")
    confidence = _f64(confidence, "confidence")
    r = np.ascontiguousarray(returns)
    out = np.zeros(2, np.float64)
    check(load().stocha_var_cvar(None, dptr(r) if r.size else None, r.size, confidence, dptr(out)))
    return float(out[0]), float(out[1])

