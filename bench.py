"""Benchmark: path-steps/s of the correlated and stochastic-volatility
workload (1e6 paths x 252 steps of each of: 3-asset multi-GBM, Heston
(Euler), Merton; seed 42), FP64 plain and FP32 fused.

One "step" = one pass of all three models.  Path-steps per step = 3 * 2.52e8
(one path-step = one time step of one path, all assets for multi-GBM).

  value     FP64 plain (the reference's method and precision): the three
            models' FP64 paths materialised into device memory (10.1 GB per
            step), timed with CUDA events on the launching stream.
  e2e       the same through the public API stocha_gb300.multi_gbm / heston /
            merton_jump_diffusion into host NumPy arrays (copies included).
  roofline  the dominant FP64 plain kernel against the FP64 pipe (measured
            DFMA rate), with its HBM write rate beside it.
  fp32_fused         FP32 paths reduced in-kernel to a European call (K=100):
            device rate, e2e through price_european, autotuned launch shapes,
            the speed-up over FP64 plain, and the generator-bound roofline.
  fp64_fused, fp32_materialised   the configuration's other two cells.
  cpu_baseline  the C++ oracle (restatement of the reference's Rayon
            algorithm) on the host cores, bounded sample.
  config5_serving  20 000 pricing / Greeks / LSMC requests, Poisson arrivals
            at 2000/s, through stocha_gb300.Server (40 GB budget): p50/p99
            latency overall and for requests of <= 1e5 paths, requests/s, and
            the per-request error against the FP64 plain form.
  config1_gbm_fp64, config3_lsmc, config4_greeks_batch, exotics_mc,
  rates_copulas_risk, api_rows   the other configurations and rows through
            the public API, each beside the oracle on a bounded sample.

--impl reference runs the C++ oracle (the reference itself is Rust and cannot
be built here) on all host cores over the identical headline workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# the serving loop runs many concurrent streams: give them hardware queues of
# their own (read when the CUDA context is created, i.e. before torch starts it)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

N_PATHS = 1_000_000  # --paths overrides (small cases for profiling only)
STEPS = 252
SEED = 42
STRIKE = 100.0
CORR3 = [[1.0, 0.6, 0.3], [0.6, 1.0, 0.5], [0.3, 0.5, 1.0]]
MULTI = dict(s0=[100.0, 50.0, 200.0], mu=[0.05, 0.08, 0.03], sigma=[0.2, 0.3, 0.15], corr=CORR3, t=1.0)
HESTON = dict(s0=100.0, v0=0.04, mu=0.05, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7, t=1.0)
MERTON = dict(s0=100.0, mu=0.05, sigma=0.2, lambda_=1.0, mu_j=-0.05, sigma_j=0.1, t=1.0)
WORKLOAD = [("multi_gbm", MULTI), ("heston", HESTON), ("merton", MERTON)]
# PCG64DXSM draws per path-step (1.0296 u64 per normal from the ziggurat tables)
DRAWS_PER_PATH_STEP = {"multi_gbm": 3 * 1.0296, "heston": 2 * 1.0296,
                       "merton": 1.0296 + 1.0 + (1.0 / 252) * 1.0296}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def hbm_peak_gbs():
    """Measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json,
    written per machine), else the fallback 6800 GB/s."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi SM clock / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(threads: int, sample_paths: int):
    """Oracle (C++ restatement of the reference's algorithm) on host cores:
    FP64 paths of the three models gathered into host arrays, sample_paths
    each."""
    import numpy as np

    from oracle import oracle as O

    O.build()
    corr = np.array(CORR3)
    t0 = time.perf_counter()
    p = O.multi_gbm(MULTI["s0"], MULTI["mu"], MULTI["sigma"], corr, 1.0, STEPS, sample_paths, seed=SEED,
                    threads=threads, gather=True)
    del p
    p = O.heston(*[HESTON[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t")], STEPS, sample_paths,
                 seed=SEED, threads=threads, gather=True)
    del p
    p = O.merton(*[MERTON[k] for k in ("s0", "mu", "sigma", "lambda_", "mu_j", "sigma_j", "t")], STEPS,
                 sample_paths, seed=SEED, threads=threads, gather=True)
    del p
    dt = time.perf_counter() - t0
    return 3 * sample_paths * STEPS / dt


def greeks_instances(n=512, seed=20261203):
    """The 512 seeded Greeks instances: s0~U[80,120], sigma~U[.1,.5],
    r~U[0,.06], t~U[.1,2], K=s0*U[.8,1.2], model uniform over gbm / heston
    (kappa=2, theta=.04, xi=.3, rho=-.7, v0=sigma^2) / merton (lambda=1,
    mu_j=-.05, sigma_j=.1), n_paths=10^U[4,6], steps in {12, 52, 252}, call."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s0 = float(rng.uniform(80, 120))
        d = dict(model=["gbm", "heston", "merton"][int(rng.integers(0, 3))], s0=s0,
                 sigma=float(rng.uniform(0.1, 0.5)), r=float(rng.uniform(0.0, 0.06)), t=float(rng.uniform(0.1, 2.0)))
        d["strike"] = s0 * float(rng.uniform(0.8, 1.2))
        d["n_paths"] = int(round(10 ** rng.uniform(4, 6)))
        d["steps"] = int(rng.choice([12, 52, 252]))
        d["payoff"] = "call"
        d["seed"] = 42
        if d["model"] == "heston":
            d.update(v0=d["sigma"] ** 2, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7)
        if d["model"] == "merton":
            d.update(lambda_=1.0, mu_j=-0.05, sigma_j=0.1)
        out.append(d)
    return out


def serving_requests(n=20_000, seed=20261204, rate=2000.0):
    """The serving mix: each request draws model, parameters and payoff from
    the Greeks-instance distributions (s0~U[80,120], sigma~U[.1,.5],
    r~U[0,.06], t~U[.1,2], K=s0*U[.8,1.2], model uniform over gbm / heston /
    merton with the fixed model parameters), kind uniform over price and
    greeks, call/put uniform; with probability 0.2 it is an LSMC put (degree
    3) instead.  n_paths = 10^U[4, log10 2e6], steps in {12, 50, 252}, seeds
    drawn per request; Poisson arrivals at `rate` per second."""
    import numpy as np

    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n):
        s0 = float(rng.uniform(80, 120))
        d = dict(s0=s0, sigma=float(rng.uniform(0.1, 0.5)), r=float(rng.uniform(0.0, 0.06)),
                 t=float(rng.uniform(0.1, 2.0)))
        d["strike"] = s0 * float(rng.uniform(0.8, 1.2))
        d["n_paths"] = int(round(10 ** rng.uniform(4, math.log10(2e6))))
        d["steps"] = int(rng.choice([12, 50, 252]))
        d["seed"] = int(rng.integers(1 << 63))
        if rng.random() < 0.2:
            d.update(kind="lsmc", payoff="put", poly_degree=3)
        else:
            d["model"] = ["gbm", "heston", "merton"][int(rng.integers(0, 3))]
            d["kind"] = ["price", "greeks"][int(rng.integers(0, 2))]
            d["payoff"] = ["call", "put"][int(rng.integers(0, 2))]
            if d["model"] == "heston":
                d.update(v0=d["sigma"] ** 2, kappa=2.0, theta=0.04, xi=0.3, rho=-0.7)
            if d["model"] == "merton":
                d.update(lambda_=1.0, mu_j=-0.05, sigma_j=0.1)
        reqs.append(d)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    return reqs, arrivals


def _fp64_plain(stocha, q):
    """The FP64 plain form (the reference's arithmetic) of one served request:
    its price, and its five Greeks for a Greeks request."""
    if q["kind"] == "lsmc":
        p, se = stocha.lsmc_american_option(q["s0"], q["strike"], q["r"], q["sigma"], q["t"], q["steps"],
                                            q["n_paths"], is_put=True, poly_degree=q["poly_degree"], seed=q["seed"])
        return {"price": p}
    keys = {"gbm": ("s0", "sigma", "t"), "heston": ("s0", "v0", "kappa", "theta", "xi", "rho", "t"),
            "merton": ("s0", "sigma", "lambda_", "mu_j", "sigma_j", "t")}[q["model"]]
    params = {k: q[k] for k in keys}
    params["mu"] = q["r"]
    p, se = stocha.price_european(q["model"], params, q["strike"], payoff=q["payoff"], steps=q["steps"],
                                  n_paths=q["n_paths"], seed=q["seed"], precision="fp64", rate=q["r"])
    out = {"price": p}
    if q["kind"] == "greeks":
        params.pop("mu")
        params["r"] = q["r"]
        out["greeks"] = stocha.greeks_fd(q["model"], params, q["payoff"], q["strike"], q["n_paths"], q["steps"],
                                         ["delta", "gamma", "vega", "theta", "rho"], seed=q["seed"], bump_size=0.01)
    return out


def bench_serving(stocha, n=20_000, rate=2000.0, budget=40 << 30, lanes=32, sample=1000):
    """Configuration 5: open-loop serving of the mix; latency, throughput and
    the error of a sample of requests against the FP64 plain form."""
    import numpy as np
    from stocha_gb300.serve import latency_summary

    reqs, arrivals = serving_requests(n, rate=rate)
    with stocha.Server(budget_bytes=budget, lanes=lanes) as srv:
        srv.replay(reqs[:64], np.zeros(64))  # warm-up: code paths, graph instantiation
        t0 = time.perf_counter()
        res = srv.replay(reqs, arrivals)
        wall = time.perf_counter() - t0
        st = srv.stats()
    out = latency_summary(res, reqs)
    lat = np.array([r["t_done"] - r["t_submit"] for r in res]) * 1e3
    kinds = np.array([q["kind"] for q in reqs])
    small = np.array([q["n_paths"] <= 100_000 for q in reqs])
    out["by_kind_p99_ms"] = {f"{k}_{'small' if s else 'large'}": float(np.percentile(lat[(kinds == k) & (small == s)], 99))
                             for k in ("price", "greeks", "lsmc") for s in (True, False)
                             if ((kinds == k) & (small == s)).any()}
    path_steps = sum(q["n_paths"] * q["steps"] for q in reqs)
    out.update(failed=int(sum(r["status"] != "done" for r in res)), wall_s=wall,
               offered_req_per_s=rate, path_steps_per_s=path_steps / wall,
               budget_bytes=budget, peak_bytes=st["peak_bytes"], lanes=lanes, jobs=st["jobs"],
               batched_requests=st["batched_requests"])
    # per-request error against the FP64 plain form, on an even sample
    idx = np.linspace(0, n - 1, sample).astype(int)
    eu, gk, ls, ls_se, ls_n = [], [], [], [], []
    for i in idx:
        q, r = reqs[i], res[i]
        ref = _fp64_plain(stocha, q)
        d = abs(r["price"] - ref["price"])
        if q["kind"] == "lsmc":
            ls.append(d / abs(ref["price"]))
            ls_se.append(d / r["std_err"])
            ls_n.append(q["n_paths"])
            continue
        eu.append(d / abs(ref["price"]))
        if "greeks" in ref:  # each Greek relative to max(|greek|, 1% of the price)
            gk.extend(abs(r["greeks"][k] - v) / max(abs(v), 0.01 * abs(ref["price"])) for k, v in ref["greeks"].items())
    f = lambda v, fn: float(fn(v)) if v else None
    out["error_vs_fp64_plain"] = {
        "sample": int(sample),
        "european_price_rel_err_max": f(eu, max), "european_price_rel_err_median": f(eu, np.median),
        "european_price_over_1e-4": int(sum(e > 1e-4 for e in eu)), "european_n": len(eu),
        "greeks_rel_err_max": f(gk, max), "greeks_rel_err_median": f(gk, np.median),
        "lsmc_price_rel_err_max": f(ls, max), "lsmc_price_rel_err_median": f(ls, np.median),
        "lsmc_price_rel_err_p99": f(ls, lambda v: np.percentile(v, 99)),
        "lsmc_price_over_1e-4": int(sum(e > 1e-4 for e in ls)),
        "lsmc_abs_err_over_std_err_max": f(ls_se, max),
        "lsmc_abs_err_over_std_err_p99": f(ls_se, lambda v: np.percentile(v, 99)), "lsmc_n": len(ls),
        "lsmc_rel_err_max_by_paths": {
            lab: f([e for e, m in zip(ls, ls_n) if lo <= m < hi], max)
            for lab, lo, hi in (("1e4-1e5", 1e4, 1e5), ("1e5-1e6", 1e5, 1e6), ("1e6-2e6", 1e6, 3e6))},
        "note": "LSMC: FP32 paths and regression move exercise decisions at near-ties; the difference to the "
                "FP64 plain form is statistical (a fraction of one standard error)"}
    out["workload"] = (f"{n} requests, Poisson {rate:.0f}/s; price/greeks on gbm/heston/merton (Greeks-instance "
                       "distributions) + 20% LSMC puts; n_paths=10^U[4,log10 2e6], steps in {12,50,252}; FP32 forms")
    return out


def bench_extras(stocha, torch, cores, skip_cpu):
    """The other configurations and rows beside the headline (each a few
    seconds).  A section that fails records its error instead of ending the
    run, so the headline line is always printed."""
    import numpy as np

    from oracle import oracle as O

    res = {}

    # -- config 1: GBM FP64, 1e5 x 252, seed 42 (the reference's own benchmark case)
    def _section0():
        steps1, n1 = 252, 100_000
        m = stocha.model_struct("gbm", dict(s0=100.0, mu=0.05, sigma=0.2, t=1.0), steps1, n1)
        from stocha_gb300 import _lib

        lib = _lib.load()
        buf = torch.empty((n1, steps1 + 1), dtype=torch.float64, device="cuda")
        for _ in range(3):
            _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, _lib.FP64, ctypes.c_void_p(buf.data_ptr())))
        _lib.check(lib.stocha_ctx_sync(None))
        k = 20
        t0 = time.perf_counter()
        for _ in range(k):
            _lib.check(lib.stocha_paths_device(None, ctypes.byref(m), 42, _lib.FP64, ctypes.c_void_p(buf.data_ptr())))
        _lib.check(lib.stocha_ctx_sync(None))
        dev_s = (time.perf_counter() - t0) / k
        stocha.gbm(100.0, 0.05, 0.2, 1.0, steps1, n1, seed=42)
        t0 = time.perf_counter()
        for _ in range(5):
            stocha.gbm(100.0, 0.05, 0.2, 1.0, steps1, n1, seed=42)
        e2e_s = (time.perf_counter() - t0) / 5
        c1 = {"workload": "gbm fp64 1e5 paths x 252 steps, seed 42", "value": n1 * steps1 / dev_s,
              "unit": "path-steps/s", "e2e": {"value": n1 * steps1 / e2e_s, "unit": "path-steps/s",
                                              "d2h_bytes_per_step": n1 * (steps1 + 1) * 8}}
        if not skip_cpu:
            O.gbm(100.0, 0.05, 0.2, 1.0, steps1, 20_000, seed=42, threads=cores, gather=True)
            t0 = time.perf_counter()
            O.gbm(100.0, 0.05, 0.2, 1.0, steps1, n1, seed=42, threads=cores, gather=True)
            c1["cpu_baseline"] = {"value": n1 * steps1 / (time.perf_counter() - t0), "cores": cores, "kind": "port"}
        res["config1_gbm_fp64"] = c1
        del buf

    # -- config 3: LSMC American put, s0=k=100, r=.05, sigma=.2, t=1, 50 steps, degree 3
    def _section1():
        c3 = {"workload": "lsmc put s0=k=100 r=.05 sigma=.2 t=1 steps=50 deg=3 seed=42"}
        for n in (50_000, 4_000_000):
            row = {}
            for prec in ("fp64", "fp32"):
                stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.2, 1.0, 50, n, precision=prec)
                t0 = time.perf_counter()
                reps = 5 if n < 1e6 else 3
                for _ in range(reps):
                    p, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.2, 1.0, 50, n, precision=prec)
                row[prec] = {"price": p, "std_err": se, "ms": 1e3 * (time.perf_counter() - t0) / reps,
                             "path_steps_per_s": n * 50 / ((time.perf_counter() - t0) / reps)}
            row["fp32_minus_fp64"] = row["fp32"]["price"] - row["fp64"]["price"]
            c3[str(n)] = row
        if not skip_cpu:
            t0 = time.perf_counter()
            p, se = O.lsmc(100.0, 100.0, 0.05, 0.2, 1.0, 50, 50_000, seed=42, threads=cores)
            c3["cpu_baseline_50000"] = {"price": p, "std_err": se, "ms": 1e3 * (time.perf_counter() - t0),
                                        "cores": cores, "kind": "port",
                                        "note": "paths on all cores, backward sweep single-threaded as in lsmc.rs"}
            c3["50000"]["fp64_minus_cpu_qr"] = c3["50000"]["fp64"]["price"] - p
        res["config3_lsmc"] = c3

    # -- config 4: 512 Greeks instances, one persistent FP32 launch
    def _section2():
        insts = greeks_instances()
        draw_steps = sum(d["n_paths"] * d["steps"] for d in insts)
        stocha.greeks_batch(insts[:8])
        t0 = time.perf_counter()
        g32 = stocha.greeks_batch(insts, precision="fp32")
        dt = time.perf_counter() - t0
        sample = list(range(0, 512, 4))  # 128 instances
        g64 = stocha.greeks_batch([insts[i] for i in sample], precision="fp64")
        rel = np.abs(g32[sample][:, [0, 2, 3, 4, 5, 6]] - g64[:, [0, 2, 3, 4, 5, 6]]) / np.maximum(
            np.abs(g64[:, [0, 2, 3, 4, 5, 6]]), 1e-3)
        names = ["price", "delta", "gamma", "vega", "theta", "rho"]
        res["config4_greeks_batch"] = {
            "instances": 512, "seconds": dt, "draw_steps": draw_steps,
            "scenario_path_steps_per_s": 7 * draw_steps / dt, "draw_steps_per_s": draw_steps / dt,
            "fp32_vs_fp64_rel_err_median": dict(zip(names, np.median(rel, axis=0).tolist())),
            "fp32_vs_fp64_rel_err_max": dict(zip(names, np.max(rel, axis=0).tolist())),
            "fp64_sample": f"{len(sample)} instances (every 4th) revalued scenario by scenario in FP64",
            "error_measure": "|fp32 - fp64| / max(|fp64|, 1e-3) per Greek"}

    # -- exotic Monte Carlo (barrier / Asian / lookback), FP64, 1e6 x 252
    def _section3():
        ex = {"workload": "1e6 paths x 252 steps, s=k=100 r=.05 sigma=.2 t=1, FP64 Monte Carlo (reference arithmetic)"}
        cases = [("barrier_uo_call_h120", lambda n: stocha.barrier_price(100, 100, .05, .2, 1., 120, method="mc",
                                                                         n_paths=n, n_steps=252),
                  lambda n: O.barrier_mc(100, 100, .05, .2, 1., 120, n_paths=n, n_steps=252, threads=cores)),
                 ("asian_arith_fixed_call_cv", lambda n: stocha.asian_price(100, 100, .05, .2, 1., method="mc", n_paths=n),
                  None),
                 ("lookback_floating_call", lambda n: stocha.lookback_price(100, .05, .2, 1., method="mc", n_paths=n),
                  lambda n: O.lookback_mc(100, .05, .2, 1., n_paths=n, threads=cores)),
                 # the FP32 forms (a GB300 addition: same draws, log-space FP32 paths)
                 ("barrier_uo_call_h120_fp32", lambda n: stocha.barrier_price(100, 100, .05, .2, 1., 120, method="mc",
                                                                              n_paths=n, n_steps=252,
                                                                              precision="fp32"), None),
                 ("asian_arith_fixed_call_cv_fp32", lambda n: stocha.asian_price(100, 100, .05, .2, 1., method="mc",
                                                                                n_paths=n, precision="fp32"), None),
                 ("lookback_floating_call_fp32", lambda n: stocha.lookback_price(100, .05, .2, 1., method="mc",
                                                                                n_paths=n, precision="fp32"), None)]
        for name, gpu, cpu in cases:
            gpu(10_000)
            t0 = time.perf_counter()
            price = gpu(1_000_000)
            dt = time.perf_counter() - t0
            row = {"price": price, "ms": dt * 1e3, "path_steps_per_s": 1e6 * 252 / dt}
            if cpu is not None and not skip_cpu:
                t0 = time.perf_counter()
                cpu(50_000)
                row["cpu_path_steps_per_s"] = 5e4 * 252 / (time.perf_counter() - t0)
                row["cpu_cores"] = cores
            ex[name] = row
        res["exotics_mc"] = ex

    # -- Hull-White paths, copulas, VaR / CVaR (host arrays in and out, as the API returns them)
    def _section4():
        rr = {}
        corr4 = np.full((4, 4), 0.4) + 0.6 * np.eye(4)
        returns = np.random.default_rng(7).standard_normal(10_000_000) * 0.02
        cases = [("hull_white_1e5x252", 1e5 * 252, "path-steps/s",
                  lambda: stocha.hull_white(0.05, 0.1, 0.005, 0.01, 1.0, 252, 100_000),
                  lambda: O.hull_white(0.05, 0.1, 0.005, 0.01, 1.0, 252, 100_000, threads=cores), 1e5 * 252),
                 ("gaussian_copula_1e6x4", 1e6, "samples/s", lambda: stocha.gaussian_copula(corr4, 1_000_000),
                  lambda: O.gaussian_copula(corr4, 100_000), 1e5),
                 ("student_t_copula_1e6x4_nu5", 1e6, "samples/s", lambda: stocha.student_t_copula(corr4, 5.0, 1_000_000),
                  lambda: O.student_t_copula(corr4, 5.0, 100_000), 1e5),
                 ("var_cvar_1e7_returns", 1e7, "returns/s", lambda: stocha.var_cvar(returns, 0.99),
                  lambda: O.var_cvar(returns[:1_000_000], 0.99), 1e6)]
        for name, units, unit, gpu, cpu, cpu_units in cases:
            gpu()
            t0 = time.perf_counter()
            for _ in range(3):
                gpu()
            dt = (time.perf_counter() - t0) / 3
            row = {"e2e_value": units / dt, "unit": unit, "ms": dt * 1e3}
            if not skip_cpu:
                t0 = time.perf_counter()
                cpu()
                row["cpu_value"] = cpu_units / (time.perf_counter() - t0)
                # Hull-White paths are per-path parallel (Rayon in the reference); the
                # copulas are one sequential stream and VaR one sort, single-threaded there
                row["cpu_cores"] = cores if name.startswith("hull_white") else 1
            rr[name] = row
        res["rates_copulas_risk"] = rr

    # -- the rest of the reference API on the path: RNG class, greeks_fd (FP64), greeks_pathwise
    def _section5():
        api = {}
        gbm_p = dict(s0=100.0, r=0.05, sigma=0.2, t=1.0)
        five = ["delta", "gamma", "vega", "theta", "rho"]
        st0, inc0 = O.pcg_seed(42)
        cases = [("rng_standard_normal_1e7", 1e7, "normals/s", lambda: stocha.RNG(seed=42).standard_normal(10_000_000),
                  lambda: O.stream_fill(st0, inc0, "standard_normal", 1_000_000), 1e6, 1),
                 ("rng_uniform_1e7", 1e7, "uniforms/s", lambda: stocha.RNG(seed=42).uniform(10_000_000),
                  lambda: O.stream_fill(st0, inc0, "uniform", 1_000_000), 1e6, 1),
                 ("greeks_fd_gbm_5greeks_1e5x252_fp64", 1e5 * 252, "path-steps/s (7 scenarios each)",
                  lambda: stocha.greeks_fd("gbm", gbm_p, "call", 100.0, 100_000, 252, five),
                  lambda: O.greeks_fd("gbm", gbm_p, "call", 100.0, 100_000, 252, five, threads=cores), 1e5 * 252, cores),
                 ("greeks_pathwise_gbm_1e6x252", 1e6 * 252, "path-steps/s",
                  lambda: stocha.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, True, 1_000_000, 252, ["delta", "vega"]),
                  lambda: O.greeks_pathwise(100.0, 0.05, 0.2, 1.0, 100.0, True, 100_000, 252, ["delta", "vega"],
                                            threads=cores), 1e5 * 252, cores)]
        for name, units, unit, gpu, cpu, cpu_units, cpu_cores in cases:
            gpu()
            t0 = time.perf_counter()
            for _ in range(3):
                gpu()
            dt = (time.perf_counter() - t0) / 3
            row = {"e2e_value": units / dt, "unit": unit, "ms": dt * 1e3}
            if not skip_cpu:
                t0 = time.perf_counter()
                cpu()
                row["cpu_value"] = cpu_units / (time.perf_counter() - t0)
                row["cpu_cores"] = cpu_cores
            api[name] = row
        res["api_rows"] = api

    # -- config 5: the serving loop
    def _section6():
        res["config5_serving"] = bench_serving(stocha)

    for fn in (_section0, _section1, _section2, _section3, _section4, _section5, _section6,):
        try:
            fn()
        except Exception as e:  # keep the headline line; record what failed
            res.setdefault("errors", []).append(f"{fn.__name__}: {e!r}")
            log(f"bench extras: {fn.__name__} failed: {e!r}")
    return res


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def rank_max(x: float, world: int, device: str = "cuda") -> float:
    """The maximum of x over the ranks of the process group (x itself for one
    rank): the job's time is its slowest rank's."""
    if world <= 1:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Seed of rank `rank`'s replica: every rank prices its own independent
    paths of the same workload (weak scaling; no data-path collective)."""
    return SEED + rank


# The headline configuration, written identically into both arms' lines
def headline_config(seed=SEED):
    return {"workload": "multi_gbm(3 assets, corr [[1,.6,.3],[.6,1,.5],[.3,.5,1]]) + heston(euler) + "
                        f"merton(lambda=1, mu_j=-0.05, sigma_j=0.1); {STEPS} steps; {N_PATHS:.0e} paths each; "
                        "seed 42; FP64 paths materialised (n_paths, steps+1[, n_assets]), the reference's method",
            "paths_per_model": N_PATHS, "steps": STEPS, "seed": seed, "precision": "fp64", "mode": "materialised",
            "l2": "no input data (parameters only); the 10.1 GB of FP64 paths written per step exceed L2"}


# Algorithmic FLOPs per path-step (exp, sqrt and ln counted as 1 each; RNG
# integer work excluded), frozen with the workload definition: multi-GBM(3)
# 6 lower-triangular MACs (12) + 3 x (FMA 2, exp 1, mul 1); Heston Euler ~21;
# Merton ~7; GBM 4.
FLOPS_PER_PATH_STEP = {"multi_gbm": 24.0, "heston": 21.0, "merton": 7.0, "gbm": 4.0}

# dram__bytes_read.sum + dram__bytes_write.sum per path row of the materialised
# FP64 kernels, from ncu captures of 2e5-path launches (the ncu summaries of
# this repository); the traffic is the written rows, so it scales with the
# row count.  Dirty data still in L2 when a
# capture ends is not counted, so these sit slightly below the algorithmic
# 8 * 253 * width bytes a row.
DRAM_BYTES_PER_ROW = {"multi_gbm": (0.112640e6 + 1164.697e6) / 2e5, "heston": (0.118528e6 + 354.099e6) / 2e5,
                      "merton": (1.749760e6 + 354.970e6) / 2e5}

# FP64 pipe operations per path-step that each FP64 plain kernel issues
# (DMUL, DADD, DFMA counted once), read from the kernels: the exponential,
# the sqrt, the conversions and (multi-GBM, Heston) the normals' products run
# on the integer pipes.
#   multi-GBM(3): the 3 normals' products (DMUL); per asset the exponent as a DFMA
#                 chain over row i of diffusion*L (1 + 2 + 3) and the price product (3 DMUL)
#   Heston Euler: sqrt(v+ dt) 1; xi dW2 2; variance update 3; log increment 2; product 1
#   Merton: normal product, exponent DFMA, price product (+3 on the ~0.4 % jump steps)
FP64_OPS_PER_PATH_STEP = {"multi_gbm": 12.0, "heston": 9.0, "merton": 3.0 + 3.0 / 252}

# Hardware-pipe figures of the FP32 fused kernels (warp-uniform form, default
# launch shape), from one ncu --set full capture of 2e5-path launches: issue
# slots busy, ALU and FMA pipe instruction rates (of their peaks), warp
# instructions per PCG64DXSM draw and threads active per warp instruction.
# They change only with the kernels; the capture's summary in this repository
# is profiles/k_uf_fp32_fused_200k.md.
FP32_FUSED_NCU = {
    "multi_gbm": {"issue_active": 0.728, "alu": 0.523, "fma": 0.310, "warp_inst_per_draw": 62.1, "simt": 28.2},
    "heston": {"issue_active": 0.721, "alu": 0.582, "fma": 0.303, "warp_inst_per_draw": 75.7, "simt": 28.0},
    "merton": {"issue_active": 0.689, "alu": 0.503, "fma": 0.319, "warp_inst_per_draw": 56.4, "simt": 28.7},
}


def oracle_headline_step(cores, n_paths=None):
    """One step of the headline workload on the host cores by the oracle (the
    C++ restatement of the reference's Rayon algorithm): the three models'
    FP64 paths (n_paths each, the full 1e6 unless given), each gathered
    serially into a new array as gbm.rs:99-105 does.  Returns the seconds
    taken."""
    import numpy as np

    from oracle import oracle as O

    n = N_PATHS if n_paths is None else n_paths
    corr = np.array(CORR3)
    t0 = time.perf_counter()
    p = O.multi_gbm(MULTI["s0"], MULTI["mu"], MULTI["sigma"], corr, 1.0, STEPS, n, seed=SEED, threads=cores,
                    gather=True)
    del p
    p = O.heston(*[HESTON[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t")], STEPS, n,
                 seed=SEED, threads=cores, gather=True)
    del p
    p = O.merton(*[MERTON[k] for k in ("s0", "mu", "sigma", "lambda_", "mu_j", "sigma_j", "t")], STEPS, n,
                 seed=SEED, threads=cores, gather=True)
    del p
    return time.perf_counter() - t0


# Seconds the reference arm's timed steps may take in all: past this, each
# step prices the first paths of the workload only (path-steps/s is the
# per-path rate, so the sample does not change it), so that any --steps ends
# within a few minutes.
REFERENCE_TIMED_BUDGET_S = 150.0


def run_reference(args, rank, world):
    """The reference's own CPU algorithm on the headline configuration.  The
    reference is Rust and cannot be built here, so this is the oracle, its
    C++ restatement, on all host cores, over the same 3 x 1e6 x 252 FP64
    paths as the GPU arm's headline (same config, same seed)."""
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    cores = host_cores()
    # the warm-up steps run the full workload; the first one sizes the timed steps
    n_step = N_PATHS
    for w in range(args.warmup):
        t_full = oracle_headline_step(cores)
        if w == 0 and args.steps * t_full > REFERENCE_TIMED_BUDGET_S:
            n_step = max(10_000, int(N_PATHS * REFERENCE_TIMED_BUDGET_S / (args.steps * t_full)) // 1000 * 1000)
    times = [oracle_headline_step(cores, n_step) for _ in range(args.steps)]
    total = sum(times)
    path_steps = 3 * n_step * STEPS
    value = path_steps * len(times) / total
    sample = (f"the full workload: 3 models x {N_PATHS} paths x {STEPS} steps" if n_step == N_PATHS else
              f"the first {n_step} of the {N_PATHS} paths of each model x {STEPS} steps per step (the timed "
              f"steps kept within {REFERENCE_TIMED_BUDGET_S:.0f} s)")
    line = {
        "impl": "reference", "metric": "path-steps/s", "value": value, "unit": "path-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference parameters)",
        "config": headline_config(),
        "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": cores, "kind": "port",
                         "sample": sample + ", FP64 paths gathered into host arrays"},
        "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C++ restatement of stocha's Rayon algorithm (the Rust reference cannot be built here)",
    }
    print(json.dumps(line), flush=True)


def _events(stream, fn, reps):
    """Average ms of fn() over reps, CUDA events on `stream`."""
    import torch

    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / reps


def run_ours(args, rank, world):
    import numpy as np
    import torch

    import stocha_gb300 as stocha
    from stocha_gb300 import _lib
    from stocha_gb300 import build as sbuild

    sbuild.build()
    lib = _lib.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    ctx = ctypes.c_void_p()
    _lib.check(lib.stocha_ctx_create(dev, ctypes.byref(ctx)))
    stream = torch.cuda.Stream()
    _lib.check(lib.stocha_ctx_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)))
    seed = replica_seed(rank)  # weak scaling: each rank its own independent 1e6 paths per model

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x):
        return rank_max(x, world, "cuda")

    models = [(name, stocha.model_struct(name, p, STEPS, N_PATHS)) for name, p in WORKLOAD]
    width = {"multi_gbm": 3, "heston": 1, "merton": 1}
    path_steps = 3 * N_PATHS * STEPS
    hbm, hbm_src = hbm_peak_gbs()

    # ---- headline: FP64 plain, materialised into device memory ----------
    bufs64 = [torch.empty((N_PATHS, STEPS + 1, width[n]) if width[n] > 1 else (N_PATHS, STEPS + 1),
                          dtype=torch.float64, device="cuda") for n, _ in models]
    bytes64 = sum(b.numel() * 8 for b in bufs64)

    def paths_launch(i, prec, buf):
        _lib.check(lib.stocha_paths_device(ctx, ctypes.byref(models[i][1]), seed, prec, ctypes.c_void_p(buf.data_ptr())))

    def fp64_step():
        for i in range(3):
            paths_launch(i, _lib.FP64, bufs64[i])

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            fp64_step()
        stream.synchronize()
        _lib.check(lib.stocha_ctx_sync(ctx))
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(dev) as clocks:
            ms = _events(stream, fp64_step, args.steps)
            barrier()
            torch.cuda.synchronize()
        _lib.check(lib.stocha_ctx_sync(ctx))
        ms = max_over_ranks(ms)
        value = world * path_steps / (ms * 1e-3)
        # per-model kernel time (3 launches each) for the roofline
        kms64 = {n: _events(stream, lambda i=i: paths_launch(i, _lib.FP64, bufs64[i]), 3)
                 for i, (n, _) in enumerate(models)}
    del bufs64
    torch.cuda.empty_cache()
    peak_dfma = ctypes.c_double(0)
    _lib.check(lib.stocha_measure_peak(ctx, 1, ctypes.byref(peak_dfma)))
    peak_fp64_ops = peak_dfma.value / 2  # DFMA/s (the kernel reports flop/s, 2 per DFMA)
    dom = max(kms64, key=kms64.get)
    flops = FLOPS_PER_PATH_STEP[dom] * N_PATHS * STEPS
    ops = FP64_OPS_PER_PATH_STEP[dom] * N_PATHS * STEPS
    roofline = {
        "bound": "fp64 pipe (and issue)", "kernel": f"k_{dom}_f64 (materialised)",
        "achieved": flops / (kms64[dom] * 1e-3) / 1e9, "peak": peak_dfma.value / 1e9, "unit": "GFLOP/s",
        "frac": flops / (kms64[dom] * 1e-3) / peak_dfma.value,
        "peak_source": "measured live (stocha_measure_peak kind 1: DFMA chains, 2 FLOP each)",
        "flops_per_path_step": FLOPS_PER_PATH_STEP[dom],
        # the FP64-pipe operations the kernel issues (the exponential, the
        # conversions and the normals' products run on the integer pipes)
        "issued_fp64_ops_per_path_step": FP64_OPS_PER_PATH_STEP[dom],
        "issued_fp64_pipe_frac": ops / (kms64[dom] * 1e-3) / peak_fp64_ops,
        "kernel_ms": kms64,
        # the bytes the dominant kernel writes, against the measured HBM copy rate
        "hbm": {"achieved_gbs": N_PATHS * (STEPS + 1) * width[dom] * 8 / (kms64[dom] * 1e-3) / 1e9,
                "peak_gbs": hbm, "peak_source": hbm_src},
        # dram__bytes_read.sum + dram__bytes_write.sum per launch (ncu on 2e5 rows, scaled by rows)
        "traffic": DRAM_BYTES_PER_ROW[dom] * N_PATHS,
        "traffic_unit": "bytes per launch",
        "algorithmic_bytes": 8.0 * (STEPS + 1) * width[dom] * N_PATHS,
    }
    roofline["hbm"]["frac"] = roofline["hbm"]["achieved_gbs"] / hbm

    # ---- e2e: FP64 plain through the public API into NumPy --------------
    e2e = None
    if not args.skip_e2e:
        corr = np.array(CORR3)

        def e2e_step():
            # each result is dropped before the next call, as a caller that
            # reduces the paths and moves on would
            x = stocha.multi_gbm(MULTI["s0"], MULTI["mu"], MULTI["sigma"], corr, 1.0, STEPS, N_PATHS, seed=seed)
            s = float(x[-1, -1, 0])  # a host read of the result
            del x
            x = stocha.heston(*[HESTON[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t")],
                              STEPS, N_PATHS, seed=seed)
            s += float(x[-1, -1])
            del x
            x = stocha.merton_jump_diffusion(*[MERTON[k] for k in ("s0", "mu", "sigma", "lambda_", "mu_j",
                                                                   "sigma_j", "t")], STEPS, N_PATHS, seed=seed)
            s += float(x[-1, -1])
            del x
            return s

        t0 = time.perf_counter()
        e2e_step()  # the first call writes into fresh host memory
        first_s = time.perf_counter() - t0
        for _ in range(max(0, args.warmup - 1)):
            e2e_step()
        barrier()
        k_e2e = max(1, args.steps // 2) if N_PATHS >= 1_000_000 else args.steps
        t0 = time.perf_counter()
        marks = [t0]
        for _ in range(k_e2e):
            e2e_step()
            marks.append(time.perf_counter())
        e2e_s = max_over_ranks((marks[-1] - t0) / k_e2e)
        per_step = np.diff(marks) * 1e3
        # the device-to-host link: 1 GiB from device memory into pinned host memory
        dsrc = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")
        hdst = torch.empty(1 << 30, dtype=torch.uint8, pin_memory=True)
        rates = []
        for _ in range(5):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            hdst.copy_(dsrc, non_blocking=True)
            torch.cuda.synchronize()
            rates.append((1 << 30) / (time.perf_counter() - t1) / 1e9)
        link_gbs = float(np.median(rates[1:]))
        del dsrc, hdst
        e2e = {"value": world * path_steps / e2e_s, "unit": "path-steps/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": bytes64, "steps": k_e2e, "ms_per_step": e2e_s * 1e3,
               # rank 0's steps one by one: the link's occasional slow steps
               # show as max >> median
               "step_ms": {"median": float(np.median(per_step)), "min": float(per_step.min()),
                           "max": float(per_step.max())},
               "link_gbs": link_gbs, "link_floor_ms": bytes64 / (link_gbs * 1e9) * 1e3,
               "first_call_value": world * path_steps / first_s,
               "api": "stocha_gb300.multi_gbm / heston / merton_jump_diffusion -> NumPy float64 arrays",
               "note": "inputs are scalar parameters (kernel arguments); d2h = the three path arrays. The "
                       "device-to-host link (link_gbs, measured here with a 1 GiB pinned copy) bounds "
                       "the step: 10.1 GB take link_floor_ms"}

    # ---- FP32 fused pricing (GB300 precision form) ------------------------
    tuning = {}
    if not args.no_tune:
        for name, p in WORKLOAD:
            tuning[name] = stocha.autotune(name, p, steps=STEPS, n_paths=N_PATHS, reps=3)
    sums = torch.zeros(64, dtype=torch.float64, device="cuda")

    def price_launch(i, prec):
        _lib.check(lib.stocha_price_device(ctx, ctypes.byref(models[i][1]), seed, prec, _lib.PAYOFF_CALL, STRIKE,
                                           0.05, ctypes.c_void_p(sums.data_ptr())))

    fp32f = {}
    with torch.cuda.stream(stream):
        for _ in range(3):
            for i in range(3):
                price_launch(i, _lib.FP32)
        ms32 = _events(stream, lambda: [price_launch(i, _lib.FP32) for i in range(3)], args.steps)
        kms32 = {n: _events(stream, lambda i=i: price_launch(i, _lib.FP32), 3) for i, (n, _) in enumerate(models)}
    ms32 = max_over_ranks(ms32)
    peak_draws = ctypes.c_double(0)
    _lib.check(lib.stocha_measure_peak(ctx, 3, ctypes.byref(peak_draws)))
    peaks = {}
    for kind, nm in ((0, "ffma_flops"), (2, "imad_ops")):
        v = ctypes.c_double(0)
        _lib.check(lib.stocha_measure_peak(ctx, kind, ctypes.byref(v)))
        peaks[nm] = v.value
    draws = sum(DRAWS_PER_PATH_STEP[n] * N_PATHS * STEPS for n, _ in WORKLOAD)
    achieved_draws = draws / (sum(kms32.values()) * 1e-3)
    fp32f = {"value": world * path_steps / (ms32 * 1e-3), "unit": "path-steps/s", "ms_per_step": ms32,
             "speedup_vs_fp64_plain": (world * path_steps / (ms32 * 1e-3)) / value,
             "kernel_ms": kms32, "autotune": tuning,
             "roofline": {"bound": "issue, ALU and FMA-heavy pipes (PCG64DXSM generator and sampler)",
                          "achieved": achieved_draws / 1e9, "unit": "G draws/s",
                          "generator_alone_peak": peak_draws.value / 1e9,
                          "frac_of_generator_alone": achieved_draws / peak_draws.value,
                          "peak_source": "measured live (stocha_measure_peak kind 3)",
                          "measured_pipe_peaks": {"ffma_gflops": peaks["ffma_flops"] / 1e9,
                                                  "imad_gops": peaks["imad_ops"] / 1e9,
                                                  "dfma_gflops": peak_dfma.value / 1e9},
                          "traffic": 77824, "traffic_unit": "bytes per launch (multi-GBM kernel: tables only)",
                          "ncu_pipes": dict(FP32_FUSED_NCU, source="ncu --set full on 2e5-path launches of the "
                                            "warp-uniform kernels (profiles/k_uf_fp32_fused_200k.md)")},
             "config": "same three models, 1e6 paths x 252 steps, European call K=100 reduced in-kernel, FP32 "
                       "paths (<= 1e-4 relative price error vs FP64)"}
    if not args.skip_e2e:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for name, p in WORKLOAD:
                stocha.price_european(name, p, STRIKE, steps=STEPS, n_paths=N_PATHS, seed=seed, precision="fp32",
                                      rate=0.05)
        e2e32 = max_over_ranks((time.perf_counter() - t0) / args.steps)
        fp32f["e2e"] = {"value": world * path_steps / e2e32, "unit": "path-steps/s", "h2d_bytes_per_step": 3 * 4096,
                        "d2h_bytes_per_step": 8 * (6 + 2 + 2),
                        "api": "stocha_gb300.price_european(precision='fp32') -> (price, std_err)"}

    # ---- the other two cells of the configuration: FP64 fused, FP32 materialised
    with torch.cuda.stream(stream):
        for i in range(3):
            price_launch(i, _lib.FP64)
        k64f = max(1, min(args.steps, 5))
        ms64f = _events(stream, lambda: [price_launch(i, _lib.FP64) for i in range(3)], k64f)
        kms64f = {n: _events(stream, lambda i=i: price_launch(i, _lib.FP64), 2) for i, (n, _) in enumerate(models)}
    ms64f = max_over_ranks(ms64f)
    d64f = max(kms64f, key=kms64f.get)
    flops_f = FLOPS_PER_PATH_STEP[d64f] * N_PATHS * STEPS
    ops_f = FP64_OPS_PER_PATH_STEP[d64f] * N_PATHS * STEPS
    fp64_fused = {"value": world * path_steps / (ms64f * 1e-3), "unit": "path-steps/s", "ms_per_step": ms64f,
                  "steps": k64f, "kernel_ms": kms64f,
                  "roofline": {"bound": "fp64 pipe (and issue)", "kernel": f"k_{d64f}_f64 (fused)",
                               "achieved": flops_f / (kms64f[d64f] * 1e-3) / 1e9, "peak": peak_dfma.value / 1e9,
                               "unit": "GFLOP/s", "frac": flops_f / (kms64f[d64f] * 1e-3) / peak_dfma.value,
                               "issued_fp64_pipe_frac": ops_f / (kms64f[d64f] * 1e-3) / peak_fp64_ops}}
    bufs32 = [torch.empty((N_PATHS, STEPS + 1, width[n]) if width[n] > 1 else (N_PATHS, STEPS + 1),
                          dtype=torch.float32, device="cuda") for n, _ in models]
    bytes32 = sum(b.numel() * 4 for b in bufs32)
    with torch.cuda.stream(stream):
        for i in range(3):
            paths_launch(i, _lib.FP32, bufs32[i])
        k32m = max(1, min(args.steps, 5))
        ms32m = _events(stream, lambda: [paths_launch(i, _lib.FP32, bufs32[i]) for i in range(3)], k32m)
        kms32m = {n: _events(stream, lambda i=i: paths_launch(i, _lib.FP32, bufs32[i]), 2)
                  for i, (n, _) in enumerate(models)}
    _lib.check(lib.stocha_ctx_sync(ctx))
    ms32m = max_over_ranks(ms32m)
    del bufs32
    torch.cuda.empty_cache()
    gbs32 = bytes32 / (ms32m * 1e-3) / 1e9
    fp32_mat = {"value": world * path_steps / (ms32m * 1e-3), "unit": "path-steps/s", "ms_per_step": ms32m,
                "steps": k32m, "kernel_ms": kms32m, "bytes_written_per_step": bytes32,
                "roofline": {"bound": "integer pipes and issue (generator); HBM is not reached",
                             "hbm_achieved_gbs": gbs32, "hbm_peak_gbs": hbm, "hbm_frac": gbs32 / hbm,
                             "peak_source": hbm_src,
                             "generator_floor_ms": draws / peak_draws.value * 1e3,
                             "hbm_floor_ms": bytes32 / (hbm * 1e9) * 1e3}}

    extras = {}
    if rank == 0 and not args.skip_extras:
        extras = bench_extras(stocha, torch, host_cores(), args.skip_cpu)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        cores = host_cores()
        sample = 20_000
        cpu_baseline(cores, 2000)
        cpu = {"value": cpu_baseline(cores, sample), "unit": "path-steps/s", "cores": cores, "kind": "port",
               "sample": f"{sample} paths x {STEPS} steps per model (3 models), FP64 paths gathered into host "
                         "arrays (the oracle, all host cores)"}

    if rank == 0:
        line = {
            "metric": "path-steps/s", "value": value, "unit": "path-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference parameters)",
            "config": headline_config(seed),
            "e2e": e2e,
            "gpu_launches": 3 * args.steps,
            "roofline": roofline,
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
            "fp32_fused": fp32f,
            "fp64_fused": fp64_fused,
            "fp32_materialised": fp32_mat,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-extras", action="store_true", help="only the headline workload")
    ap.add_argument("--paths", type=int, default=N_PATHS, help="paths per model (profiling cases)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no autotune)")
    args = ap.parse_args()
    globals()["N_PATHS"] = args.paths
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
