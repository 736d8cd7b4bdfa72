"""Serving loop over the C ABI (stocha_server_* in include/stocha_gpu.h).

A :class:`Server` owns one device-memory budget, a set of CUDA streams and a
native dispatcher thread that admits requests as their bytes fit and batches
small pricing/Greeks requests into one launch as they arrive.  Requests are
dicts:

``kind``
    ``"price"`` (European price and standard error), ``"greeks"`` (price and
    all five Greeks, as ``greeks_fd`` with the bump-and-revalue scenarios of
    src/finance/greeks.rs) or ``"lsmc"`` (``lsmc_american_option``).
``model``
    ``"gbm"``, ``"heston"`` (Euler) or ``"merton"`` (price / greeks).
parameters
    ``s0, r, sigma, t`` and the model's own (``v0, kappa, theta, xi, rho``;
    ``lambda_, mu_j, sigma_j``), ``strike``, ``payoff`` (``"call"``/``"put"``),
    ``n_paths``, ``steps``, ``seed`` (42), ``bump_size`` (0.01),
    ``poly_degree`` (LSMC, 3).

Results are dicts with ``price``, ``std_err``, ``greeks`` (for ``"greeks"``)
and the server-clock times ``t_submit``, ``t_admit``, ``t_done`` (seconds).
A result depends only on its request, not on what else was in flight.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

# Streams share the device's hardware work queues (8 by default); a small
# launch queued behind a large one on a shared queue waits for the large one
# to dispatch.  Takes effect if set before the process's CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import _lib

_KIND = {"price": _lib.REQ_PRICE, "greeks": _lib.REQ_GREEKS, "lsmc": _lib.REQ_LSMC}
_MODEL = {"gbm": _lib.MODEL_GBM, "heston": _lib.MODEL_HESTON, "merton": _lib.MODEL_MERTON}
_FIELDS = ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j", "sigma_j")
GREEK_NAMES = ("delta", "gamma", "vega", "theta", "rho")


def _fill(x: _lib.StochaRequest, d: dict) -> None:
    kind = d.get("kind", "price")
    if kind not in _KIND:
        raise ValueError(f"Unknown request kind: '{kind}'. Supported: price, greeks, lsmc")
    x.kind = _KIND[kind]
    x.poly_degree = int(d.get("poly_degree", 3))
    i = x.inst
    model = d.get("model", "gbm")
    if kind != "lsmc" and model not in _MODEL:
        raise ValueError(f"Unknown model: '{model}'. Supported: gbm, heston, merton")
    i.model = _MODEL.get(model, _lib.MODEL_GBM)
    payoff = d.get("payoff", "put" if kind == "lsmc" else "call")
    if payoff not in ("call", "put"):
        raise ValueError(f"Unknown payoff: '{payoff}'. Supported: 'call', 'put'")
    i.payoff = _lib.PAYOFF_CALL if payoff == "call" else _lib.PAYOFF_PUT
    i.scheme = 0
    for k in _FIELDS:
        setattr(i, k, float(d.get(k, 0.0)))
    i.strike = float(d["strike"])
    i.bump_size = float(d.get("bump_size", 0.01))
    i.n_paths, i.steps, i.seed = int(d["n_paths"]), int(d["steps"]), int(d.get("seed", 42))


def _result(r: _lib.StochaResult, kind: int) -> dict:
    status = {1: "done", 0: "pending", -_lib.STOCHA_ERR_CANCELLED: "cancelled"}.get(r.status, "failed")
    out = {"status": status,
           "price": r.price, "std_err": r.std_err,
           "t_submit": r.t_submit, "t_admit": r.t_admit, "t_done": r.t_done}
    if r.status < 0:
        out["error_code"] = -r.status
    if kind == _lib.REQ_GREEKS:
        out["greeks"] = {n: r.greeks[j] for j, n in enumerate(GREEK_NAMES)}
    return out


class Server:
    """Continuous-batching server on one GPU.

    Args:
        budget_bytes: device memory the server may hold (admission budget).
        lanes: CUDA streams: an eighth at the highest priority (small pricing
            and Greeks batches), a quarter at a middle one (LSMC), the rest at
            the lowest (large pricing and Greeks requests).
        device: CUDA device index.
    """

    def __init__(self, budget_bytes: int = 40 << 30, lanes: int = 32, device: int = 0) -> None:
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.stocha_server_create(int(device), int(budget_bytes), int(lanes), ctypes.byref(h)))
        self._h = h
        self._kinds: dict[int, int] = {}

    def close(self) -> None:
        """Finishes every submitted request, then releases the server."""
        if self._h:
            _lib.check(self._lib.stocha_server_destroy(self._h))
            self._h = None

    def __enter__(self) -> "Server":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def submit(self, request: dict) -> int:
        x = _lib.StochaRequest()
        _fill(x, request)
        t = ctypes.c_uint64()
        _lib.check(self._lib.stocha_server_submit(self._h, ctypes.byref(x), ctypes.byref(t)))
        self._kinds[t.value] = x.kind
        return t.value

    def poll(self, ticket: int) -> dict:
        r = _lib.StochaResult()
        _lib.check(self._lib.stocha_server_poll(self._h, int(ticket), ctypes.byref(r)))
        return _result(r, self._kinds.get(ticket, -1))

    def cancel(self, ticket: int) -> bool:
        """Cancels a request that is still waiting for admission (a lane or
        device memory); True if it is (now) cancelled, False if it was already
        admitted, in which case it runs to completion."""
        c = ctypes.c_int32()
        _lib.check(self._lib.stocha_server_cancel(self._h, int(ticket), ctypes.byref(c)))
        return bool(c.value)

    def wait(self, ticket: int, timeout: float | None = None) -> dict:
        r = _lib.StochaResult()
        _lib.check(self._lib.stocha_server_wait(self._h, int(ticket), -1.0 if timeout is None else float(timeout),
                                                 ctypes.byref(r)))
        return _result(r, self._kinds.get(ticket, -1))

    def replay(self, requests: list, arrival_s) -> list:
        """Submits requests[i] at arrival_s[i] seconds after the call starts
        (native open-loop driver), waits for all, returns their results."""
        n = len(requests)
        arr = (_lib.StochaRequest * max(n, 1))()
        for i, d in enumerate(requests):
            _fill(arr[i], d)
        t = np.ascontiguousarray(arrival_s, np.float64)
        if t.shape != (n,):
            raise ValueError("arrival_s must have one entry per request")
        res = (_lib.StochaResult * max(n, 1))()
        _lib.check(self._lib.stocha_server_replay(self._h, arr, _lib.dptr(t), n, res))
        return [_result(res[i], arr[i].kind) for i in range(n)]

    def stats(self) -> dict:
        c = _lib.StochaServerCounters()
        _lib.check(self._lib.stocha_server_stats(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in _lib.StochaServerCounters._fields_}


def latency_summary(results: list, requests: list | None = None, small_paths: int = 100_000) -> dict:
    """p50/p99 of submit-to-done latency (ms), overall and for requests of at
    most ``small_paths`` paths, and the completion rate."""
    lat = np.array([r["t_done"] - r["t_submit"] for r in results]) * 1e3
    out = {"requests": len(results), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "max_ms": float(lat.max())}
    if requests is not None:
        small = np.array([int(q["n_paths"]) <= small_paths for q in requests])
        if small.any():
            out["small_p50_ms"] = float(np.percentile(lat[small], 50))
            out["small_p99_ms"] = float(np.percentile(lat[small], 99))
            out["small_requests"] = int(small.sum())
    t0 = min(r["t_submit"] for r in results)
    t1 = max(r["t_done"] for r in results)
    out["req_per_s"] = len(results) / (t1 - t0) if t1 > t0 else float("inf")
    return out
