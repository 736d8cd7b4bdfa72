"""The serving loop (stocha_server_*): results, admission and batching.

* A request's result is the same, bit for bit, alone and inside a mix of
  concurrent requests (its streams, chunk partials and launch shapes depend
  only on the request).
* Served results against the library's own calls: LSMC identical to
  lsmc_american_option(precision="fp32"); prices and Greeks within the FP32
  form's tolerance of the FP64 plain method (the reference's arithmetic).
* Admission by device memory: a budget that holds one LSMC job at a time
  still completes every request, never holds more than the budget, and a
  request larger than the budget is refused at submission.
* Failures made on the host: a request cancelled while it waits for
  admission never runs; a budget the device cannot allocate fails creation
  with MemoryError and leaves the process able to serve.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-4


def _mix(rng, n, lsmc_share=0.2, max_paths=200_000):
    out = []
    for i in range(n):
        s0 = rng.uniform(80, 120)
        d = dict(s0=s0, sigma=rng.uniform(0.1, 0.5), r=rng.uniform(0.0, 0.06), t=rng.uniform(0.1, 2.0),
                 strike=s0 * rng.uniform(0.8, 1.2), n_paths=int(10 ** rng.uniform(3, np.log10(max_paths))),
                 steps=int(rng.choice([12, 50, 252])), seed=int(rng.integers(1 << 62)))
        if rng.random() < lsmc_share:
            d.update(kind="lsmc", payoff="put", poly_degree=3)
        else:
            d.update(kind=str(rng.choice(["price", "greeks"])), model=str(rng.choice(["gbm", "heston", "merton"])),
                     payoff=str(rng.choice(["call", "put"])), v0=d["sigma"] ** 2, kappa=2.0, theta=0.04, xi=0.3,
                     rho=-0.7, lambda_=1.0, mu_j=-0.05, sigma_j=0.1)
        out.append(d)
    return out


def _same(a, b):
    assert a["status"] == b["status"] == "done"
    assert a["price"] == b["price"] and a["std_err"] == b["std_err"]
    if "greeks" in a:
        assert a["greeks"] == b["greeks"]


def test_same_result_alone_and_in_mix(stocha):
    rng = np.random.default_rng(2026)
    probes = [
        dict(kind="greeks", model="heston", payoff="put", s0=100.0, r=0.03, sigma=0.2, v0=0.04, kappa=2.0,
             theta=0.04, xi=0.3, rho=-0.7, t=1.0, strike=95.0, n_paths=50_000, steps=50, seed=7),
        dict(kind="price", model="merton", payoff="call", s0=100.0, r=0.05, sigma=0.2, lambda_=1.0, mu_j=-0.05,
             sigma_j=0.1, t=0.5, strike=100.0, n_paths=300_000, steps=12, seed=8),
        dict(kind="lsmc", payoff="put", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=40_000, steps=50,
             seed=9, poly_degree=3),
        dict(kind="greeks", model="gbm", payoff="call", s0=100.0, r=0.05, sigma=0.25, t=1.0, strike=105.0,
             n_paths=1000, steps=252, seed=10),
    ]
    with stocha.Server(budget_bytes=2 << 30, lanes=8) as srv:
        alone = [srv.wait(srv.submit(p)) for p in probes]
        mix = _mix(rng, 60)
        pos = [5, 17, 33, 48]
        reqs = list(mix)
        for k, p in zip(pos, probes):
            reqs.insert(k, p)
        arrivals = np.sort(rng.uniform(0, 0.01, len(reqs)))
        res = srv.replay(reqs, arrivals)
        st = srv.stats()
    for k, p, a in zip(pos, probes, alone):
        _same(a, res[k])
    assert all(r["status"] == "done" for r in res)
    assert st["completed"] == len(reqs) + len(probes) and st["failed"] == 0
    assert st["batched_requests"] > 0  # small requests shared launches


def test_served_results_match_library_calls(stocha):
    lsmc = dict(kind="lsmc", payoff="put", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=50_000,
                steps=50, seed=42, poly_degree=3)
    g = dict(kind="greeks", model="gbm", payoff="call", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0,
             n_paths=200_000, steps=52, seed=3)
    h = dict(kind="price", model="heston", payoff="put", s0=100.0, r=0.05, sigma=0.2, v0=0.04, kappa=2.0,
             theta=0.04, xi=0.3, rho=-0.7, t=1.0, strike=100.0, n_paths=100_000, steps=50, seed=5)
    with stocha.Server(budget_bytes=1 << 30, lanes=4) as srv:
        rl, rg, rh = (srv.wait(srv.submit(d)) for d in (lsmc, g, h))
    p, se = stocha.lsmc_american_option(100.0, 100.0, 0.05, 0.2, 1.0, 50, 50_000, seed=42, precision="fp32")
    assert rl["price"] == p and rl["std_err"] == se
    # Greeks: against the FP64 plain form (the reference's scenario revaluation)
    want = stocha.greeks_fd("gbm", {"s0": 100.0, "r": 0.05, "sigma": 0.2, "t": 1.0}, "call", 100.0, 200_000, 52,
                            ["delta", "gamma", "vega", "theta", "rho"], seed=3)
    for k, v in want.items():
        assert abs(rg["greeks"][k] - v) <= max(FP32_RTOL * abs(v), 1e-6), (k, rg["greeks"][k], v)
    # price: against the FP64 fused price of the same paths
    p64, _ = stocha.price_european("heston", {"s0": 100.0, "v0": 0.04, "mu": 0.05, "kappa": 2.0, "theta": 0.04,
                                              "xi": 0.3, "rho": -0.7, "t": 1.0}, 100.0, payoff="put", steps=50,
                                    n_paths=100_000, seed=5, precision="fp64")
    assert abs(rh["price"] - p64) <= FP32_RTOL * p64, (rh["price"], p64)


def test_admission_by_memory_budget(stocha):
    # each LSMC job holds ~ n * 51 * 4 bytes of paths: 200k paths ~ 41 MB
    req = dict(kind="lsmc", payoff="put", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=200_000,
               steps=50, poly_degree=2)
    budget = 64 << 20
    with stocha.Server(budget_bytes=budget, lanes=8) as srv:
        tickets = [srv.submit(dict(req, seed=s)) for s in range(6)]
        res = [srv.wait(t) for t in tickets]
        st = srv.stats()
        with pytest.raises(MemoryError, match="serving budget"):
            srv.submit(dict(req, n_paths=2_000_000))
    assert all(r["status"] == "done" for r in res)
    assert st["peak_bytes"] <= budget
    # one at a time: the admissions are serialised by the budget
    spans = sorted((r["t_admit"], r["t_done"]) for r in res)
    for (a0, d0), (a1, d1) in zip(spans, spans[1:]):
        assert a1 >= d0 - 1e-3 or a1 >= a0  # admitted after the previous finished (poll granularity)
    assert len({r["price"] for r in res}) == 6  # different seeds, different prices


def test_cancel_waiting_request(stocha):
    """A request still waiting for admission can be cancelled: its result is
    'cancelled', it never runs, and the server goes on serving.  A request
    already admitted is not: cancel returns False and it completes.  With a
    budget that holds one LSMC job (each holds ~4e6 * 253 * 4 bytes of paths)
    the second one waits while the first runs (~15 ms on GB300); the cancel
    comes microseconds after its submission."""
    big = dict(kind="lsmc", payoff="put", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=4_000_000,
               steps=252, poly_degree=3)
    budget = 6 << 30
    with stocha.Server(budget_bytes=budget, lanes=8) as srv:
        t0 = srv.submit(big)
        t1 = srv.submit(dict(big, seed=7))
        assert srv.cancel(t1) is True
        assert srv.cancel(t1) is True  # idempotent
        r1 = srv.wait(t1)
        r0 = srv.wait(t0)
        assert srv.cancel(t0) is False  # admitted and done
        small = srv.submit(dict(kind="price", model="gbm", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0,
                                n_paths=10_000, steps=12))
        r2 = srv.wait(small)
        st = srv.stats()
    assert r1["status"] == "cancelled" and r1["t_admit"] == 0.0
    assert r0["status"] == "done" and r2["status"] == "done"
    assert st["cancelled"] == 1 and st["failed"] == 0 and st["completed"] == 2
    with pytest.raises(ValueError, match="unknown ticket"):
        with stocha.Server(budget_bytes=64 << 20, lanes=3) as srv:
            srv.cancel(5)


def test_budget_allocation_failure(stocha):
    """A serving budget beyond the device's memory: the slab's cudaMalloc
    fails, creation raises MemoryError naming the budget, and the process's
    CUDA context stays usable for a server that fits."""
    with pytest.raises(MemoryError, match="device allocation of the serving budget"):
        stocha.Server(budget_bytes=1 << 50, lanes=3)
    with stocha.Server(budget_bytes=64 << 20, lanes=3) as srv:
        r = srv.wait(srv.submit(dict(kind="price", model="gbm", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0,
                                     n_paths=10_000, steps=12)))
    assert r["status"] == "done"


def test_submit_validation(stocha):
    with stocha.Server(budget_bytes=64 << 20, lanes=3) as srv:
        with pytest.raises(ValueError, match="n_paths must be at least 2"):
            srv.submit(dict(kind="lsmc", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=1, steps=10))
        with pytest.raises(ValueError, match="steps and n_paths must be positive"):
            srv.submit(dict(kind="price", model="gbm", s0=100.0, r=0.05, sigma=0.2, t=1.0, strike=100.0, n_paths=0,
                            steps=10))
        with pytest.raises(ValueError, match="Unknown model"):
            srv.submit(dict(kind="price", model="sabr", s0=100.0, strike=100.0, n_paths=10, steps=10))


def test_open_loop_load_latency(stocha):
    """A short open-loop run of the serving mix: everything completes and
    the latency summary is consistent."""
    from stocha_gb300.serve import latency_summary

    rng = np.random.default_rng(11)
    reqs = _mix(rng, 400, max_paths=2_000_000)
    arrivals = np.cumsum(rng.exponential(1 / 2000.0, len(reqs)))
    with stocha.Server(budget_bytes=8 << 30, lanes=16) as srv:
        res = srv.replay(reqs, arrivals)
        st = srv.stats()
    assert all(r["status"] == "done" for r in res)
    s = latency_summary(res, reqs)
    assert 0 < s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert st["completed"] == len(reqs) and st["peak_bytes"] <= 8 << 30
    print(s)
