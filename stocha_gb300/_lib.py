"""Loads libstocha_gpu.so (built in-tree by stocha_gb300/build.py) and declares
the C ABI of include/stocha_gpu.h for ctypes.

There is no CPU fallback: if the library is missing or no GPU is present the
calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstocha_gpu.so")

STOCHA_OK = 0
STOCHA_ERR_VALUE = 1
STOCHA_ERR_CUDA = 2
STOCHA_ERR_NOMEM = 3
STOCHA_ERR_DEVICE = 4
STOCHA_ERR_CALLBACK = 5
STOCHA_ERR_BUSY = 6
STOCHA_ERR_TIMEOUT = 7
STOCHA_ERR_CANCELLED = 8
REQ_PRICE, REQ_GREEKS, REQ_LSMC = 0, 1, 2

FP64, FP32 = 0, 1
MODEL_GBM, MODEL_HESTON, MODEL_MERTON, MODEL_MULTI_GBM, MODEL_HULL_WHITE = 0, 1, 2, 3, 4
PAYOFF_CALL, PAYOFF_PUT = 0, 1

c_u64 = ctypes.c_uint64
c_i32 = ctypes.c_int32
c_dbl = ctypes.c_double
c_size = ctypes.c_size_t
c_void_p = ctypes.c_void_p
c_char_p = ctypes.c_char_p
P_dbl = ctypes.POINTER(ctypes.c_double)
P_u64 = ctypes.POINTER(ctypes.c_uint64)


class StochaModel(ctypes.Structure):
    _fields_ = [
        ("kind", c_i32), ("scheme", c_i32),
        ("s0", c_dbl), ("mu", c_dbl), ("sigma", c_dbl), ("q", c_dbl), ("t", c_dbl),
        ("v0", c_dbl), ("kappa", c_dbl), ("theta", c_dbl), ("xi", c_dbl), ("rho", c_dbl),
        ("lambda_", c_dbl), ("mu_j", c_dbl), ("sigma_j", c_dbl),
        ("steps", c_u64), ("n_paths", c_u64),
        ("antithetic", c_i32), ("n_assets", c_i32),
        ("s0_v", P_dbl), ("mu_v", P_dbl), ("sigma_v", P_dbl), ("corr", P_dbl),
    ]


class StochaGreeksParams(ctypes.Structure):
    _fields_ = [(k, c_dbl) for k in ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j",
                                     "sigma_j")] + [("present", ctypes.c_uint32), ("scheme", c_i32)]


class StochaGreeksInstance(ctypes.Structure):
    _fields_ = [("model", c_i32), ("payoff", c_i32), ("scheme", c_i32), ("pad", c_i32)] + \
        [(k, c_dbl) for k in ("s0", "r", "sigma", "t", "v0", "kappa", "theta", "xi", "rho", "lambda_", "mu_j",
                              "sigma_j", "strike", "bump_size")] + \
        [("n_paths", c_u64), ("steps", c_u64), ("seed", c_u64)]


class StochaRequest(ctypes.Structure):
    _fields_ = [("kind", c_i32), ("poly_degree", c_i32), ("inst", StochaGreeksInstance)]


class StochaResult(ctypes.Structure):
    _fields_ = [("status", c_i32), ("pad", c_i32), ("price", c_dbl), ("std_err", c_dbl),
                ("greeks", c_dbl * 5), ("t_submit", c_dbl), ("t_admit", c_dbl), ("t_done", c_dbl)]


class StochaServerCounters(ctypes.Structure):
    _fields_ = [(k, c_u64) for k in ("submitted", "completed", "failed", "jobs", "batched_requests",
                                     "budget_bytes", "peak_bytes", "in_use_bytes")] + \
        [("lanes", c_i32), ("high_lanes", c_i32), ("cancelled", c_u64)]


class StochaTuneResult(ctypes.Structure):
    _fields_ = [(k, c_i32) for k in ("model", "n_assets", "block", "ilp", "waves", "variant", "candidates", "pad")] + \
        [("ms_best", c_dbl), ("ms_default", c_dbl)]


PAYOFF_FN = ctypes.CFUNCTYPE(c_i32, c_void_p, P_dbl, c_u64, P_dbl, ctypes.POINTER(c_u64))
P_charp = ctypes.POINTER(ctypes.c_char_p)


class StochaRng(ctypes.Structure):
    _fields_ = [("state_lo", c_u64), ("state_hi", c_u64), ("inc_lo", c_u64), ("inc_hi", c_u64),
                ("seed_lo", c_u64), ("seed_hi", c_u64)]


# (name, restype, argtypes) of every exported function
SIGNATURES = [
    ("stocha_ctx_create", c_i32, [c_i32, ctypes.POINTER(c_void_p)]),
    ("stocha_ctx_destroy", None, [c_void_p]),
    ("stocha_ctx_stream", c_void_p, [c_void_p]),
    ("stocha_ctx_set_stream", c_i32, [c_void_p, c_void_p]),
    ("stocha_ctx_sync", c_i32, [c_void_p]),
    ("stocha_last_error", c_char_p, []),
    ("stocha_version", c_char_p, []),
    ("stocha_host_buffer_acquire", c_i32, [c_size, ctypes.POINTER(c_void_p)]),
    ("stocha_host_buffer_release", c_i32, [c_void_p]),
    ("stocha_host_cache_stats", c_i32, [ctypes.POINTER(c_size), ctypes.POINTER(c_size)]),
    ("stocha_gbm", c_i32, [c_void_p, c_dbl, c_dbl, c_dbl, c_dbl, c_u64, c_u64, c_u64, c_i32, c_dbl, P_dbl]),
    ("stocha_heston", c_i32, [c_void_p] + [c_dbl] * 8 + [c_u64, c_u64, c_u64, c_char_p, P_dbl]),
    ("stocha_merton_jump_diffusion", c_i32, [c_void_p] + [c_dbl] * 7 + [c_u64, c_u64, c_u64, P_dbl]),
    ("stocha_gaussian_copula", c_i32, [c_void_p, P_dbl, c_size, c_size, c_u64, c_u64, P_dbl]),
    ("stocha_student_t_copula", c_i32, [c_void_p, P_dbl, c_size, c_size, c_dbl, c_u64, c_u64, P_dbl]),
    ("stocha_hull_white", c_i32, [c_void_p] + [c_dbl] * 5 + [c_u64, c_u64, c_u64, P_dbl]),
    ("stocha_multi_gbm", c_i32, [c_void_p, c_size, P_dbl, P_dbl, P_dbl, P_dbl, c_size, c_size, c_dbl, c_u64, c_u64,
                                 c_u64, c_i32, P_dbl]),
    ("stocha_paths_device", c_i32, [c_void_p, ctypes.POINTER(StochaModel), c_u64, c_i32, c_void_p]),
    ("stocha_price", c_i32, [c_void_p, ctypes.POINTER(StochaModel), c_u64, c_i32, c_i32, c_dbl, c_dbl, P_dbl]),
    ("stocha_price_device", c_i32, [c_void_p, ctypes.POINTER(StochaModel), c_u64, c_i32, c_i32, c_dbl, c_dbl,
                                    c_void_p]),
    ("stocha_rng_new", c_i32, [c_u64, c_u64, c_char_p, ctypes.POINTER(StochaRng)]),
    ("stocha_rng_uniform", c_i32, [c_void_p, ctypes.POINTER(StochaRng), c_u64, P_dbl]),
    ("stocha_rng_standard_normal", c_i32, [c_void_p, ctypes.POINTER(StochaRng), c_u64, P_dbl]),
    ("stocha_rng_normal", c_i32, [c_void_p, ctypes.POINTER(StochaRng), c_u64, c_dbl, c_dbl, P_dbl]),
    ("stocha_rng_save_state", c_i32, [ctypes.POINTER(StochaRng), ctypes.c_char_p, c_size, ctypes.POINTER(c_size)]),
    ("stocha_rng_from_state", c_i32, [c_char_p, ctypes.POINTER(StochaRng)]),
    ("stocha_rng_raw_u64", c_i32, [c_void_p, ctypes.POINTER(StochaRng), c_u64, P_u64]),
    ("stocha_lsmc_american_option", c_i32, [c_void_p] + [c_dbl] * 5 + [c_u64, c_u64, c_i32, c_u64, c_u64, P_dbl,
                                                                   P_dbl]),
    ("stocha_lsmc", c_i32, [c_void_p] + [c_dbl] * 5 + [c_u64, c_u64, c_i32, c_u64, c_u64, c_i32, P_dbl, P_dbl]),
    ("stocha_greeks_fd", c_i32, [c_void_p, c_char_p, ctypes.POINTER(StochaGreeksParams), c_char_p, PAYOFF_FN, c_void_p,
                                 c_dbl, c_u64, c_u64, P_charp, c_u64, c_u64, c_dbl, c_i32, P_dbl]),
    ("stocha_greeks_pathwise", c_i32, [c_void_p] + [c_dbl] * 5 + [c_i32, c_u64, c_u64, P_charp, c_u64, c_u64, P_dbl]),
    ("stocha_greeks_batch", c_i32, [c_void_p, ctypes.POINTER(StochaGreeksInstance), c_u64, c_i32, P_dbl]),
    ("stocha_price_noalloc", c_i32, [ctypes.POINTER(StochaModel), c_u64, c_i32, c_i32, c_dbl, c_void_p, c_void_p]),
    ("stocha_barrier_price", c_i32, [c_void_p] + [c_dbl] * 6 + [c_char_p, c_char_p, c_dbl, c_u64, c_u64, c_u64,
                                                                 c_char_p, c_i32, c_dbl, c_i32, c_i32, P_dbl]),
    ("stocha_asian_price", c_i32, [c_void_p] + [c_dbl] * 5 + [c_u64, c_char_p, c_char_p, c_char_p, c_dbl, c_u64,
                                                               c_u64, c_char_p, c_dbl, c_dbl, c_i32, P_dbl]),
    ("stocha_lookback_price", c_i32, [c_void_p] + [c_dbl] * 4 + [c_u64, c_char_p, c_char_p, c_dbl, c_dbl, c_u64,
                                                                  c_u64, c_char_p, c_dbl, c_dbl, c_i32, P_dbl]),
    ("stocha_var_cvar", c_i32, [c_void_p, P_dbl, c_u64, c_dbl, P_dbl]),
    ("stocha_var_cvar_device", c_i32, [c_void_p, c_void_p, c_u64, c_dbl, P_dbl]),
    ("stocha_autotune", c_i32, [c_void_p, ctypes.POINTER(StochaModel), c_i32, ctypes.POINTER(StochaTuneResult)]),
    ("stocha_tune_get", c_i32, [c_i32, c_i32, ctypes.POINTER(StochaTuneResult)]),
    ("stocha_tune_set", c_i32, [c_i32, c_i32, c_i32, c_i32, c_i32, c_i32]),
    ("stocha_server_create", c_i32, [c_i32, c_u64, c_i32, ctypes.POINTER(c_void_p)]),
    ("stocha_server_destroy", c_i32, [c_void_p]),
    ("stocha_server_submit", c_i32, [c_void_p, ctypes.POINTER(StochaRequest), ctypes.POINTER(c_u64)]),
    ("stocha_server_poll", c_i32, [c_void_p, c_u64, ctypes.POINTER(StochaResult)]),
    ("stocha_server_cancel", c_i32, [c_void_p, c_u64, ctypes.POINTER(c_i32)]),
    ("stocha_server_wait", c_i32, [c_void_p, c_u64, c_dbl, ctypes.POINTER(StochaResult)]),
    ("stocha_server_replay", c_i32, [c_void_p, ctypes.POINTER(StochaRequest), P_dbl, c_u64,
                                     ctypes.POINTER(StochaResult)]),
    ("stocha_server_stats", c_i32, [c_void_p, ctypes.POINTER(StochaServerCounters)]),
    ("stocha_debug_arena", c_i32, [c_u64, ctypes.POINTER(ctypes.c_int64), c_u64, ctypes.POINTER(ctypes.c_int64)]),
    ("stocha_debug_zig_thresholds", c_i32, [P_u64]),
    ("stocha_debug_exp", c_i32, [c_void_p, P_dbl, P_dbl, c_u64]),
    ("stocha_debug_sqrt", c_i32, [c_void_p, P_dbl, P_dbl, c_u64]),
    ("stocha_debug_f64", c_i32, [c_void_p, c_i32, P_dbl, P_dbl, c_u64]),
    ("stocha_debug_capped_draws", c_i32, [c_void_p, c_i32, c_i32, c_u64, c_u64, P_dbl]),
    ("stocha_debug_zigfeed", c_i32, [c_void_p, c_i32, c_u64, c_u64, ctypes.c_uint32, c_void_p, c_void_p]),
    ("stocha_debug_fast_log_error", c_i32, [c_void_p, P_dbl, P_dbl]),
    ("stocha_measure_peak", c_i32, [c_void_p, c_i32, P_dbl]),
]

_lock = threading.Lock()
_lib = None


def load():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with `python -m stocha_gb300.build` "
                                  "(there is no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, res, args in SIGNATURES:
                fn = getattr(L, name, None)
                if fn is None:
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class StochaError(RuntimeError):
    """A CUDA or device-side failure reported by the engine."""


def check(rc: int) -> None:
    if rc == STOCHA_OK:
        return
    msg = load().stocha_last_error().decode("utf-8", "replace")
    if rc == STOCHA_ERR_VALUE:
        raise ValueError(msg)
    if rc == STOCHA_ERR_NOMEM:
        raise MemoryError(msg)
    raise StochaError(msg)


def dptr(a):
    return a.ctypes.data_as(P_dbl)
