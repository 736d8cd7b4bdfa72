"""stocha_gb300 — GB300-native Monte Carlo engine behind stocha's Python API.

Drop-in for the Monte Carlo part of heki1224/stocha (python/stocha/__init__.py):
`RNG`, `gbm`, `heston`, `merton_jump_diffusion`, `multi_gbm`,
`lsmc_american_option`, `greeks_fd`, `greeks_pathwise` keep the reference's
names, signatures, defaults, return types and error messages.  All of them run
on the GPU through the C ABI of libstocha_gpu.so (include/stocha_gpu.h);
there is no CPU fallback.

GB300-only additions: `price_european` (fused in-kernel payoff, FP64 or FP32),
`paths_device` (device-resident paths), `greeks_batch` (many instances in one
persistent launch) and `serve` (continuous-batching request loop).

Example:
    >>> import stocha_gb300 as stocha
    >>> paths = stocha.gbm(s0=100.0, mu=0.05, sigma=0.2, t=1.0, steps=252, n_paths=10000)
"""
from __future__ import annotations

import ctypes
from typing import Literal

import numpy as np

from . import _lib, _stocha
from ._stocha import __version__
from .serve import Server

__all__ = [
    "RNG",
    "gbm",
    "heston",
    "merton_jump_diffusion",
    "multi_gbm",
    "hull_white",
    "lsmc_american_option",
    "greeks_fd",
    "greeks_pathwise",
    "barrier_price",
    "asian_price",
    "lookback_price",
    "var_cvar",
    "gaussian_copula",
    "student_t_copula",
    "greeks_batch",
    "price_european",
    "model_struct",
    "autotune",
    "tune_get",
    "tune_set",
    "Server",
    "__version__",
]


class RNG:
    """PCG64DXSM generator (python/stocha/__init__.py:75-177).

    Args:
        seed:      Integer seed (default 0), up to 128 bits.
        algorithm: Only ``"pcg64dxsm"`` is supported.
    """

    def __init__(self, seed: int = 0, algorithm: Literal["pcg64dxsm"] = "pcg64dxsm") -> None:
        self._inner = _stocha.RNG(seed=seed, algorithm=algorithm)

    @property
    def seed(self) -> int:
        return self._inner.seed

    def uniform(self, size: int = 1) -> np.ndarray:
        return self._inner.uniform(size)

    def standard_normal(self, size: int = 1) -> np.ndarray:
        return self._inner.standard_normal(size)

    def normal(self, size: int = 1, loc: float = 0.0, scale: float = 1.0) -> np.ndarray:
        return self._inner.normal(size=size, loc=loc, scale=scale)

    def save_state(self) -> str:
        return self._inner.save_state()

    @classmethod
    def from_state(cls, json: str) -> "RNG":
        inner = _stocha.RNG.from_state(json)
        obj = cls.__new__(cls)
        obj._inner = inner
        return obj

    def __repr__(self) -> str:
        return f"RNG(seed={self.seed}, algorithm='pcg64dxsm')"


def gbm(s0: float, mu: float, sigma: float, t: float, steps: int, n_paths: int, seed: int = 42,
        antithetic: bool = False, q: float = 0.0) -> np.ndarray:
    """GBM paths, shape ``(n_paths, steps + 1)`` (python/stocha/__init__.py:180-231)."""
    return _stocha.gbm(s0=s0, mu=mu, sigma=sigma, t=t, steps=steps, n_paths=n_paths, seed=seed,
                       antithetic=antithetic, q=q)


def heston(s0: float, v0: float, mu: float, kappa: float, theta: float, xi: float, rho: float, t: float,
           steps: int, n_paths: int, seed: int = 42, scheme: Literal["euler", "qe"] = "euler") -> np.ndarray:
    """Heston paths, shape ``(n_paths, steps + 1)`` (python/stocha/__init__.py:276-324)."""
    return _stocha.heston(s0=s0, v0=v0, mu=mu, kappa=kappa, theta=theta, xi=xi, rho=rho, t=t, steps=steps,
                          n_paths=n_paths, seed=seed, scheme=scheme)


def merton_jump_diffusion(s0: float, mu: float, sigma: float, lambda_: float, mu_j: float, sigma_j: float,
                          t: float, steps: int, n_paths: int, seed: int = 42) -> np.ndarray:
    """Merton jump-diffusion paths (python/stocha/__init__.py:327-373)."""
    return _stocha.merton_jump_diffusion(s0=s0, mu=mu, sigma=sigma, lambda_=lambda_, mu_j=mu_j, sigma_j=sigma_j,
                                         t=t, steps=steps, n_paths=n_paths, seed=seed)


def multi_gbm(s0: list, mu: list, sigma: list, corr: np.ndarray, t: float, steps: int, n_paths: int,
              seed: int = 42, antithetic: bool = False) -> np.ndarray:
    """Correlated multi-asset GBM, shape ``(n_paths, steps + 1, n_assets)``
    (python/stocha/__init__.py:574-627)."""
    return _stocha.multi_gbm(s0=list(s0), mu=list(mu), sigma=list(sigma), corr=np.asarray(corr, dtype=np.float64),
                             t=t, steps=steps, n_paths=n_paths, seed=seed, antithetic=antithetic)


def hull_white(r0: float, a: float, theta: float, sigma: float, t: float, steps: int, n_paths: int,
               seed: int = 42) -> np.ndarray:
    """Hull-White one-factor short-rate paths by the exact transition, shape ``(n_paths, steps + 1)``
    (python/stocha/__init__.py hull_white)."""
    return _stocha.hull_white(r0=r0, a=a, theta=theta, sigma=sigma, t=t, steps=steps, n_paths=n_paths, seed=seed)


def lsmc_american_option(s0: float, k: float, r: float, sigma: float, t: float, steps: int, n_paths: int,
                         is_put: bool = True, poly_degree: int = 3, seed: int = 42,
                         precision: str = "fp64") -> tuple[float, float]:
    """American option by Longstaff-Schwartz, ``(price, std_err)``
    (python/stocha/__init__.py:630-671).  ``precision="fp32"`` is a GB300
    addition: FP32 paths with the FP64 regression."""
    return _stocha.lsmc_american_option(s0=s0, k=k, r=r, sigma=sigma, t=t, steps=steps, n_paths=n_paths,
                                        is_put=is_put, poly_degree=poly_degree, seed=seed, precision=precision)


def greeks_fd(model: str, params: dict, payoff, strike: float, n_paths: int, n_steps: int, greeks: list,
              seed: int = 42, bump_size: float = 0.01, precision: str = "fp64") -> dict:
    """Bump-and-revalue Greeks with common random numbers
    (python/stocha/__init__.py:674-722).  ``precision="fp32"`` is a GB300
    addition: every scenario of a path in one FP32 pass."""
    return _stocha.greeks_fd(model=model, params=params, payoff=payoff, strike=strike, n_paths=n_paths,
                             n_steps=n_steps, greeks=greeks, seed=seed, bump_size=bump_size, precision=precision)


def greeks_pathwise(s0: float, r: float, sigma: float, t: float, strike: float, is_call: bool, n_paths: int,
                    n_steps: int, greeks: list, seed: int = 42) -> dict:
    """Pathwise (IPA) delta and vega for GBM (python/stocha/__init__.py:725-769)."""
    return _stocha.greeks_pathwise(s0=s0, r=r, sigma=sigma, t=t, strike=strike, is_call=is_call, n_paths=n_paths,
                                   n_steps=n_steps, greeks=greeks, seed=seed)


def barrier_price(s: float, k: float, r: float, sigma: float, t: float, barrier: float,
                  barrier_type: str = "up-and-out", option_type: str = "call", q: float = 0.0, n_paths: int = 100_000,
                  n_steps: int = 252, seed: int = 42, method: str = "auto", n_monitoring: int | None = None,
                  rebate: float = 0.0, rebate_at_hit: bool = False, precision: str = "fp64") -> float:
    """Barrier option price (python/stocha/__init__.py:983-1060): Reiner-Rubinstein closed form
    ("auto"/"analytical") or Monte Carlo on the GPU ("mc").  ``precision="fp32"`` is a GB300
    addition: the Monte Carlo paths in FP32 log space on the same draws."""
    return _stocha.barrier_price(s, k, r, sigma, t, barrier, barrier_type=barrier_type, option_type=option_type,
                                 q=q, n_paths=n_paths, n_steps=n_steps, seed=seed, method=method,
                                 n_monitoring=n_monitoring, rebate=rebate, rebate_at_hit=rebate_at_hit,
                                 precision=precision)


def asian_price(s: float, k: float, r: float, sigma: float, t: float, n_steps: int = 252,
                average_type: str = "arithmetic", strike_type: str = "fixed", option_type: str = "call", q: float = 0.0,
                n_paths: int = 100_000, seed: int = 42, method: str = "auto", running_avg: float | None = None,
                time_elapsed: float | None = None, precision: str = "fp64") -> float:
    """Asian option price (python/stocha/__init__.py:1063-1127): Kemna-Vorst closed form for the
    geometric fixed-strike case, Monte Carlo on the GPU (geometric control variate) otherwise.
    ``precision="fp32"``: the Monte Carlo paths in FP32 (a GB300 addition)."""
    return _stocha.asian_price(s, k, r, sigma, t, n_steps=n_steps, average_type=average_type,
                               strike_type=strike_type, option_type=option_type, q=q, n_paths=n_paths, seed=seed,
                               method=method, running_avg=running_avg, time_elapsed=time_elapsed,
                               precision=precision)


def lookback_price(s: float, r: float, sigma: float, t: float, n_steps: int = 252, strike_type: str = "floating",
                   option_type: str = "call", k: float = 0.0, q: float = 0.0, n_paths: int = 100_000, seed: int = 42,
                   method: str = "auto", running_max: float | None = None,
                   running_min: float | None = None, precision: str = "fp64") -> float:
    """Lookback option price (python/stocha/__init__.py:1130-1190): Goldman-Sosin-Gatto / Conze-Viswanathan
    closed forms or Monte Carlo on the GPU.  ``precision="fp32"``: the Monte Carlo paths in FP32
    (a GB300 addition)."""
    return _stocha.lookback_price(s, r, sigma, t, n_steps=n_steps, strike_type=strike_type, option_type=option_type,
                                  k=k, q=q, n_paths=n_paths, seed=seed, method=method, running_max=running_max,
                                  running_min=running_min, precision=precision)


def gaussian_copula(corr: np.ndarray, n_samples: int, seed: int = 42) -> np.ndarray:
    """Samples of a Gaussian copula, shape ``(n_samples, dim)`` in (0, 1) (python/stocha/__init__.py
    gaussian_copula): one sequential stream, normals generated on the GPU by a parallel parse."""
    return _stocha.gaussian_copula(corr, n_samples, seed=seed)


def student_t_copula(corr: np.ndarray, nu: float, n_samples: int, seed: int = 42) -> np.ndarray:
    """Samples of a Student-t copula, shape ``(n_samples, dim)`` in (0, 1) (python/stocha/__init__.py
    student_t_copula): one sequential stream, parsed in parallel on the GPU."""
    return _stocha.student_t_copula(corr, nu, n_samples, seed=seed)


def var_cvar(returns: np.ndarray, confidence: float) -> tuple[float, float]:
    """Value-at-Risk and Conditional VaR of a return series (python/stocha/__init__.py var_cvar):
    losses are -returns; VaR is the loss at rank ceil(confidence * n) of the sorted losses and CVaR
    the mean of the losses from there on.  Computed on the GPU by a radix select (no sort)."""
    return _stocha.var_cvar(returns, confidence)


# ------------------------------------------------------- GB300 additions ---
_BATCH_FIELDS = ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j")


def greeks_batch(instances: list, precision: str = "fp32"):
    """Price and all five Greeks of many instances in one persistent launch.

    Each instance is a dict: ``model`` ("gbm"/"heston"/"merton"), the
    model's parameters as for greeks_fd (``r`` is the drift), ``strike``,
    ``payoff`` ("call"/"put", default call), ``n_paths``, ``steps``,
    optional ``seed`` (42), ``bump_size`` (0.01), ``scheme`` (Heston).
    ``precision="fp32"``: FP32 paths with common random numbers across
    scenarios and FP64 reductions; ``"fp64"``: the reference's scenario
    revaluation per instance.  Returns an array (n, 7): price, std_err,
    delta, gamma, vega, theta, rho."""
    n = len(instances)
    arr = (_lib.StochaGreeksInstance * max(n, 1))()
    for i, d in enumerate(instances):
        x = arr[i]
        x.model = _KINDS[d["model"]]
        x.payoff = _lib.PAYOFF_CALL if d.get("payoff", "call") == "call" else _lib.PAYOFF_PUT
        x.scheme = 1 if d.get("scheme", "euler") == "qe" else 0
        for k in _BATCH_FIELDS:
            setattr(x, k, float(d.get(k, 0.0)))
        x.strike = float(d["strike"])
        x.bump_size = float(d.get("bump_size", 0.01))
        x.n_paths, x.steps, x.seed = int(d["n_paths"]), int(d["steps"]), int(d.get("seed", 42))
    out = np.zeros((max(n, 1), 7), np.float64)
    if precision not in _PRECISION:
        raise ValueError("precision must be 'fp64' or 'fp32'")
    _lib.check(_lib.load().stocha_greeks_batch(None, arr, n, _PRECISION[precision], _lib.dptr(out)))
    return out[:n]
_KINDS = {"gbm": _lib.MODEL_GBM, "heston": _lib.MODEL_HESTON, "merton": _lib.MODEL_MERTON,
          "multi_gbm": _lib.MODEL_MULTI_GBM}
_PRECISION = {"fp64": _lib.FP64, "fp32": _lib.FP32}


def model_struct(model: str, params: dict, steps: int, n_paths: int, antithetic: bool = False):
    """The C-ABI ``stocha_model`` for a model name and parameter dict.

    Keys: gbm ``s0, mu, sigma, t[, q]``; heston ``s0, v0, mu, kappa, theta,
    xi, rho, t[, scheme]``; merton ``s0, mu, sigma, lambda_, mu_j, sigma_j,
    t``; multi_gbm ``s0, mu, sigma`` (lists), ``corr``, ``t``.  ``r`` is
    accepted for ``mu`` (the risk-neutral drift, as greeks_fd names it)."""
    if model not in _KINDS:
        raise ValueError(f"Unknown model: '{model}'. Supported: gbm, heston, merton, multi_gbm")
    m = _lib.StochaModel()
    m.kind = _KINDS[model]
    p = dict(params)
    if "r" in p and "mu" not in p:
        p["mu"] = p["r"]
    m.steps, m.n_paths, m.antithetic = int(steps), int(n_paths), int(bool(antithetic))
    if model == "multi_gbm":
        keep = [np.ascontiguousarray(p[k], np.float64) for k in ("s0", "mu", "sigma")]
        corr = np.ascontiguousarray(p["corr"], np.float64)
        m.n_assets = keep[0].shape[0]
        m.s0_v, m.mu_v, m.sigma_v, m.corr = (_lib.dptr(a) for a in (*keep, corr))
        m._keep = (keep, corr)
        m.t = float(p["t"])
        return m
    for k in ("s0", "mu", "sigma", "q", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j"):
        if k in p:
            setattr(m, k, float(p[k]))
    scheme = p.get("scheme", "euler")
    m.scheme = 0 if scheme == "euler" else 1 if scheme == "qe" else -1
    return m


def price_european(model: str, params: dict, strike: float, payoff: str = "call", steps: int = 252,
                   n_paths: int = 100_000, seed: int = 42, precision: str = "fp64", rate=None,
                   antithetic: bool = False):
    """European call/put price and standard error with the payoff reduced in
    the path kernel (no path array is materialised).

    Same draws and discretisation as the path functions: ``fp64`` equals
    ``exp(-rate*t) * mean(payoff(paths[:, -1]))`` of ``gbm``/``heston``/...
    to summation order; ``fp32`` runs the paths in FP32 with FP64 block
    totals.  ``rate`` defaults to the model drift (risk-neutral pricing).
    Returns ``(price, std_err)``, or a list of them per asset for multi_gbm."""
    m = model_struct(model, params, steps, n_paths, antithetic)
    if payoff not in ("call", "put"):
        raise ValueError(f"Unknown payoff: '{payoff}'. Supported: 'call', 'put'")
    if precision not in _PRECISION:
        raise ValueError("precision must be 'fp64' or 'fp32'")
    if rate is None:
        rate = params.get("r", params.get("mu", 0.0)) if model != "multi_gbm" else params.get("r", 0.0)
    na = m.n_assets if model == "multi_gbm" else 1
    out = np.zeros(2 * max(na, 1), np.float64)
    _lib.check(_lib.load().stocha_price(None, ctypes.byref(m), int(seed), _PRECISION[precision],
                                        _lib.PAYOFF_CALL if payoff == "call" else _lib.PAYOFF_PUT, float(strike),
                                        float(rate), _lib.dptr(out)))
    res = [(float(out[2 * a]), float(out[2 * a + 1])) for a in range(na)]
    return res if model == "multi_gbm" else res[0]


def _tune_dict(r) -> dict:
    return {"variant": r.variant, "block": r.block, "ilp": r.ilp, "waves": r.waves, "candidates": r.candidates,
            "ms_best": r.ms_best, "ms_default": r.ms_default}


def autotune(model: str, params: dict, steps: int = 252, n_paths: int = 1_000_000, reps: int = 3) -> dict:
    """Times every launch shape of the fused FP32 pricing kernel of ``model``
    (kernel form: one path per thread at a time, 1 or 2 paths per thread
    in lockstep, or one path per thread with the sampler fed one draw per
    warp-wide iteration; threads per block 64/128/256; 1 or 2 waves of
    resident blocks) on this size and installs the fastest for the model kind
    (process-wide).  Returns the chosen shape with its time and the default
    shape's time (ms per launch)."""
    m = model_struct(model, params, steps, n_paths)
    r = _lib.StochaTuneResult()
    _lib.check(_lib.load().stocha_autotune(None, ctypes.byref(m), int(reps), ctypes.byref(r)))
    return _tune_dict(r)


def tune_get(model: str, n_assets: int = 0) -> dict:
    """The installed launch shape of ``model``'s fused FP32 kernel."""
    r = _lib.StochaTuneResult()
    _lib.check(_lib.load().stocha_tune_get(_KINDS[model], int(n_assets), ctypes.byref(r)))
    return _tune_dict(r)


def tune_set(model: str, block: int, ilp: int, waves: int, variant: int = 1, n_assets: int = 0) -> None:
    """Installs a launch shape (e.g. one saved from an earlier autotune)."""
    _lib.check(_lib.load().stocha_tune_set(_KINDS[model], int(n_assets), int(block), int(ilp), int(waves),
                                           int(variant)))

