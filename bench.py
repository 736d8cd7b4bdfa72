"""Benchmark: path-steps/s, FP32 fused vs FP64 plain, on the correlated and
stochastic-volatility workload (1e6 paths x 252 steps of each of: 3-asset
multi-GBM, Heston (Euler), Merton; seed 42; European call at K=100).

One "step" = one pass of all three models.  Path-steps per step = 3 * 2.52e8
(one path-step = one time step of one path, all assets for multi-GBM).

  value   FP32 fused pricing, device-resident (parameters only, no inputs),
          timed with CUDA events on the launching stream.
  e2e     the same through the public API stocha_gb300.price_european
          (host call: parameters in, (price, se) out, copies included).
  autotune  the fused FP32 kernels' launch shapes (threads per block, paths
          per thread in lockstep, grid waves), timed on this workload before
          the timed region; the chosen shape and its gain over the default.
  fp64_plain   FP64 materialised paths (reference arithmetic) of the same
          workload into device memory (10.1 GB per step) and, end to end,
          through stocha_gb300.multi_gbm/heston/merton_jump_diffusion into
          host NumPy arrays.
  roofline  dominant kernel = FP32 fused; bound = the PCG64DXSM generator
          (integer pipes): achieved draws/s vs the measured draw rate of the
          generator alone (stocha_measure_peak kind 3).
  cpu_baseline  the C++ oracle (restatement of the reference's Rayon
          algorithm) on the host cores, bounded sample.
  config5_serving  20 000 pricing / Greeks / LSMC requests, Poisson arrivals
          at 2000/s, through stocha_gb300.Server (40 GB budget): p50/p99
          latency overall and for requests of <= 1e5 paths, requests/s, and
          the per-request error of a sample against the FP64 plain form.
  exotics_mc, rates_copulas_risk, api_rows  barrier / Asian / lookback
          Monte Carlo, Hull-White paths, Gaussian and Student-t copulas,
          VaR/CVaR, the RNG class, greeks_fd and greeks_pathwise through the
          public API (host arrays), each beside the oracle on a bounded
          sample.

--impl reference runs the C++ oracle (the reference itself is Rust and cannot
be built here) on all host cores for the same workload, each step a sample of
1e5 paths per model.
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
    FP64 materialised paths + payoff of the three models, sample_paths each."""
    import numpy as np

    from oracle import oracle as O

    O.build()
    corr = np.array(CORR3)
    t0 = time.perf_counter()
    p = O.multi_gbm(MULTI["s0"], MULTI["mu"], MULTI["sigma"], corr, 1.0, STEPS, sample_paths, seed=SEED,
                    threads=threads, gather=True)
    _ = np.maximum(p[:, -1, :] - STRIKE, 0).mean(axis=0)
    del p
    p = O.heston(*[HESTON[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t")], STEPS, sample_paths,
                 seed=SEED, threads=threads, gather=True)
    _ = np.maximum(p[:, -1] - STRIKE, 0).mean()
    del p
    p = O.merton(*[MERTON[k] for k in ("s0", "mu", "sigma", "lambda_", "mu_j", "sigma_j", "t")], STEPS,
                 sample_paths, seed=SEED, threads=threads, gather=True)
    _ = np.maximum(p[:, -1] - STRIKE, 0).mean()
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


def bench_serving(stocha, n=20_000, rate=2000.0, budget=40 << 30, lanes=32, sample=60):
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
    eu, gk, ls, ls_se = [], [], [], []
    for i in idx:
        q, r = reqs[i], res[i]
        ref = _fp64_plain(stocha, q)
        d = abs(r["price"] - ref["price"])
        if q["kind"] == "lsmc":
            ls.append(d / abs(ref["price"]))
            ls_se.append(d / r["std_err"])
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
        "lsmc_abs_err_over_std_err_max": f(ls_se, max), "lsmc_n": len(ls),
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
        sample = list(range(0, 512, 32))
        g64 = stocha.greeks_batch([insts[i] for i in sample], precision="fp64")
        rel = np.abs(g32[sample][:, [0, 2, 3, 4, 5, 6]] - g64[:, [0, 2, 3, 4, 5, 6]]) / np.maximum(
            np.abs(g64[:, [0, 2, 3, 4, 5, 6]]), 1e-3)
        names = ["price", "delta", "gamma", "vega", "theta", "rho"]
        res["config4_greeks_batch"] = {
            "instances": 512, "seconds": dt, "draw_steps": draw_steps,
            "scenario_path_steps_per_s": 7 * draw_steps / dt, "draw_steps_per_s": draw_steps / dt,
            "fp32_vs_fp64_rel_err_median": dict(zip(names, np.median(rel, axis=0).tolist())),
            "fp32_vs_fp64_rel_err_max": dict(zip(names, np.max(rel, axis=0).tolist())),
            "fp64_sample": f"{len(sample)} instances (every 32nd) revalued scenario by scenario in FP64"}

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


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = host_cores()
    sample = 100_000
    for _ in range(args.warmup):
        cpu_baseline(cores, sample)
    vals = [cpu_baseline(cores, sample) for _ in range(args.steps)]
    total_time = sum(3 * sample * STEPS / v for v in vals)
    value = 3 * sample * STEPS * len(vals) / total_time
    line = {
        "impl": "reference", "metric": "path-steps/s", "value": value, "unit": "path-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_time / len(vals), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference parameters)",
        "config": {"workload": "multi_gbm(3 assets)+heston(euler)+merton, 252 steps, european call K=100",
                   "paths_per_model_per_step": sample, "full_paths_per_model": N_PATHS},
        "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} paths x {STEPS} steps per model, FP64 materialised + payoff"},
        "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C++ restatement of stocha's Rayon algorithm (the Rust reference cannot be built here)",
    }
    print(json.dumps(line), flush=True)


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
    seed = replica_seed(rank)  # weak scaling: each rank prices its own independent 1e6 paths per model

    models = [(name, stocha.model_struct(name, p, STEPS, N_PATHS)) for name, p in WORKLOAD]
    # launch shapes of the fused FP32 kernels, tuned on this workload before any timing
    tuning = {}
    if not args.no_tune:
        for name, p in WORKLOAD:
            tuning[name] = stocha.autotune(name, p, steps=STEPS, n_paths=N_PATHS, reps=3)
    sums = torch.zeros(64, dtype=torch.float64, device="cuda")

    def fused_step():
        for name, m in models:
            _lib.check(lib.stocha_price_device(ctx, ctypes.byref(m), seed, _lib.FP32, _lib.PAYOFF_CALL, STRIKE,
                                               0.05, ctypes.c_void_p(sums.data_ptr())))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x):
        return rank_max(x, world, "cuda")

    path_steps = 3 * N_PATHS * STEPS
    # ---- headline: FP32 fused, device resident
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            fused_step()
        stream.synchronize()
        _lib.check(lib.stocha_ctx_sync(ctx))
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(dev) as clocks:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                fused_step()
            e1.record(stream)
            e1.synchronize()
            barrier()
            torch.cuda.synchronize()
        _lib.check(lib.stocha_ctx_sync(ctx))
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = world * path_steps / (ms * 1e-3)

    # per-model kernel time (average of 3 launches) for the roofline
    per_model = {}
    with torch.cuda.stream(stream):
        for name, m in models:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(3):
                _lib.check(lib.stocha_price_device(ctx, ctypes.byref(m), seed, _lib.FP32, _lib.PAYOFF_CALL, STRIKE,
                                                   0.05, ctypes.c_void_p(sums.data_ptr())))
            b.record(stream)
            b.synchronize()
            per_model[name] = a.elapsed_time(b) / 3
    peak_draws = ctypes.c_double(0)
    _lib.check(lib.stocha_measure_peak(ctx, 3, ctypes.byref(peak_draws)))
    draws = sum(DRAWS_PER_PATH_STEP[n] * N_PATHS * STEPS for n, _ in WORKLOAD)
    achieved = draws / (sum(per_model.values()) * 1e-3)

    # ---- e2e FP32 fused through the public API
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(0 if args.skip_e2e else args.steps):
        for name, p in WORKLOAD:
            stocha.price_european(name, p, STRIKE, steps=STEPS, n_paths=N_PATHS, seed=seed, precision="fp32",
                                  rate=0.05)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e = world * path_steps / e2e_s if not args.skip_e2e else None

    # ---- FP64 plain: materialised paths, device resident and end to end
    fp64 = {}
    if not args.skip_fp64:
        bufs = [torch.empty((N_PATHS, STEPS + 1, 3), dtype=torch.float64, device="cuda"),
                torch.empty((N_PATHS, STEPS + 1), dtype=torch.float64, device="cuda"),
                torch.empty((N_PATHS, STEPS + 1), dtype=torch.float64, device="cuda")]

        def fp64_step():
            for (name, m), b in zip(models, bufs):
                _lib.check(lib.stocha_paths_device(ctx, ctypes.byref(m), seed, _lib.FP64, ctypes.c_void_p(b.data_ptr())))

        k64 = max(1, min(args.steps, 3))
        with torch.cuda.stream(stream):
            fp64_step()
            stream.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(k64):
                fp64_step()
            b.record(stream)
            b.synchronize()
            _lib.check(lib.stocha_ctx_sync(ctx))
        ms64 = max_over_ranks(a.elapsed_time(b) / k64)
        del bufs
        torch.cuda.empty_cache()
        fp64 = {"value": world * path_steps / (ms64 * 1e-3), "ms_per_step": ms64, "steps": k64,
                "bytes_written_per_step": 8 * N_PATHS * (STEPS + 1) * 5}
        if not args.skip_e2e64:
            corr = np.array(CORR3)

            def e2e64_pass():
                # each result is dropped before the next call, as a caller that
                # reduces the paths and moves on would
                t0 = time.perf_counter()
                x = stocha.multi_gbm(MULTI["s0"], MULTI["mu"], MULTI["sigma"], corr, 1.0, STEPS, N_PATHS, seed=seed)
                del x
                x = stocha.heston(*[HESTON[k] for k in ("s0", "v0", "mu", "kappa", "theta", "xi", "rho", "t")],
                                  STEPS, N_PATHS, seed=seed)
                del x
                x = stocha.merton_jump_diffusion(*[MERTON[k] for k in ("s0", "mu", "sigma", "lambda_", "mu_j",
                                                                       "sigma_j", "t")], STEPS, N_PATHS, seed=seed)
                del x
                return max_over_ranks(time.perf_counter() - t0)

            # the first pass writes into fresh host memory; later passes reuse the
            # host result cache's buffers, whose pages already exist
            cold = e2e64_pass()
            warm = min(e2e64_pass() for _ in range(2))
            fp64["e2e"] = {"value": world * path_steps / warm, "unit": "path-steps/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8 * N_PATHS * (STEPS + 1) * 5,
                           "first_call_value": world * path_steps / cold}
        fp64["fp32_fused_speedup"] = value / fp64["value"]
        hbm, hbm_src = hbm_peak_gbs()
        gbs = fp64["bytes_written_per_step"] / (ms64 * 1e-3) / 1e9
        fp64["roofline"] = {"bound": "FP64 pipe (Heston) and issue (the others); not HBM, see profiles/",
                            "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                            "peak_source": hbm_src, "note": "algorithmic bytes = the materialised paths written"}
        fp64["form"] = ("reference algorithm in FP64 (paths within 1e-12 of the oracle); its exponential, the "
                        "Heston sqrt and the normals' products run on the integer pipes (GB300 issues FP64 at "
                        "1/64 of FP32), 2.7x the FP64-pipe form against which the FP32 fused form was 9.7x")

    extras = {}
    if rank == 0 and not args.skip_extras:
        extras = bench_extras(stocha, torch, host_cores(), args.skip_cpu)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        cores = host_cores()
        sample = 20_000
        cpu_baseline(cores, 2000)
        cpu = {"value": cpu_baseline(cores, sample), "unit": "path-steps/s", "cores": cores, "kind": "port",
               "sample": f"{sample} paths x {STEPS} steps per model (3 models), FP64 materialised + payoff"}

    if rank == 0:
        line = {
            "metric": "path-steps/s", "value": value, "unit": "path-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; reference parameters)",
            "config": {"workload": "multi_gbm(3 assets, corr [[1,.6,.3],[.6,1,.5],[.3,.5,1]]) + heston(euler) + "
                                   "merton(lambda=1, mu_j=-0.05, sigma_j=0.1); 252 steps; 1e6 paths each; "
                                   "european call K=100; FP32 fused",
                       "paths_per_model": N_PATHS, "steps": STEPS, "seed": seed,
                       "l2": "no input data (parameters only); FP64 outputs (10.1 GB/step) exceed L2"},
            "e2e": {"value": e2e, "unit": "path-steps/s", "h2d_bytes_per_step": 3 * 4096,
                    "d2h_bytes_per_step": 8 * (6 + 2 + 2)},
            "gpu_launches": 6 * args.steps,
            "roofline": {"bound": "int (PCG64DXSM generator)", "achieved": achieved / 1e9, "peak": peak_draws.value / 1e9,
                         "unit": "Gdraws/s", "frac": achieved / peak_draws.value,
                         # dram__bytes_read.sum + dram__bytes_write.sum of one k_gbm_uf<3> launch
                         # (ncu, profiles/k_gbm_uf3_fused_200k.md): the staged ziggurat tables only,
                         # the same at any path count (no path data leaves the registers)
                         "traffic": 77824, "traffic_unit": "bytes per launch (multi-GBM kernel)",
                         # that traffic over the kernel's time, against the measured HBM rate: the
                         # fused form is not memory-bound
                         "hbm_frac": 77824 / (per_model["multi_gbm"] * 1e-3) / (hbm_peak_gbs()[0] * 1e9),
                         "kernel_ms": per_model, "peak_source": "measured live (stocha_measure_peak kind 3)"},
            "fp64_plain": fp64,
            "autotune": tuning,
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
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
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e64", action="store_true")
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
