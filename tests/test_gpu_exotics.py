"""Exotic Monte Carlo (barrier_mc, asian_mc, lookback_mc) on the device
against the oracle's restatement (same streams, same GBM step).

Bars: FP64 prices within MC_RTOL of the oracle (summation order and the
kernels' exponential: paths agree to ~1e-14 relative; a barrier decision
could flip only for a path within that of the barrier); the Asian
geometric average's log sum is n ln s0 + sum_i (n - i + 1) x_i over the step
exponents x_i, one weighted FMA a step (the oracle keeps the reference's
running log and its running sum), within ASIAN_RTOL.  The reference's own MC expectations
(agreement with the closed forms, reproducibility) are restated.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MC_RTOL = 1e-12
ASIAN_RTOL = 1e-11


@pytest.mark.parametrize("btype,h", [("up-and-out", 115.0), ("up-and-in", 115.0), ("down-and-out", 90.0),
                                     ("down-and-in", 90.0), ("uo", 99.0), ("di", 101.0)])
@pytest.mark.parametrize("opt", ["call", "put"])
def test_barrier_mc_matches_oracle(stocha, oracle, btype, h, opt):
    kw = dict(s=100.0, k=100.0, r=0.05, sigma=0.25, t=1.0, barrier=h, barrier_type=btype, option_type=opt, q=0.01,
              n_paths=20_000, n_steps=100, seed=11)
    got = stocha.barrier_price(**kw, method="mc")
    want = oracle.barrier_mc(**kw)
    assert abs(got - want) <= MC_RTOL * max(abs(want), 1e-300), (got, want)


@pytest.mark.parametrize("btype", ["up-and-out", "up-and-in", "down-and-out", "down-and-in"])
@pytest.mark.parametrize("at_hit", [False, True])
def test_barrier_mc_rebates_match_oracle(stocha, oracle, btype, at_hit):
    h = 120.0 if btype.startswith("up") else 85.0
    kw = dict(s=100.0, k=100.0, r=0.05, sigma=0.2, t=1.0, barrier=h, barrier_type=btype, n_paths=20_000,
              n_steps=252, seed=3, rebate=5.0, rebate_at_hit=at_hit)
    got = stocha.barrier_price(**kw, method="mc")
    want = oracle.barrier_mc(**kw)
    assert abs(got - want) <= MC_RTOL * abs(want), (got, want)


def test_barrier_mc_reference_expectations(stocha):
    base = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, barrier=120)
    ana = stocha.barrier_price(**base)
    mc = stocha.barrier_price(**base, method="mc", n_paths=200_000, n_steps=252)
    assert abs(mc - ana) / ana < 0.15  # discrete monitoring knocks out less often
    assert stocha.barrier_price(**base, method="mc", seed=5) == stocha.barrier_price(**base, method="mc", seed=5)
    # the Monte Carlo monitors the given barrier and ignores n_monitoring
    assert stocha.barrier_price(**base, method="mc", n_monitoring=12) == stocha.barrier_price(**base, method="mc")
    ana_r = stocha.barrier_price(**base, rebate=5, rebate_at_hit=True)
    mc_r = stocha.barrier_price(**base, rebate=5, rebate_at_hit=True, method="mc", n_paths=100_000, n_steps=2000,
                                seed=1)
    assert abs(mc_r - ana_r) / ana_r < 0.05


def _geo_analytical(stocha, s, k, r, sigma, t, q):
    return stocha.asian_price(s, k, r, sigma, t, average_type="geometric", method="analytical", q=q)


@pytest.mark.parametrize("avg,strike,opt", [("arithmetic", "fixed", "call"), ("arithmetic", "fixed", "put"),
                                            ("geometric", "fixed", "call"), ("arithmetic", "floating", "call"),
                                            ("geometric", "floating", "put")])
def test_asian_mc_matches_oracle(stocha, oracle, avg, strike, opt):
    s, k, r, sigma, t, q, n, steps = 100.0, 100.0, 0.05, 0.2, 1.0, 0.01, 20_000, 252
    got = stocha.asian_price(s, k, r, sigma, t, n_steps=steps, average_type=avg, strike_type=strike,
                             option_type=opt, q=q, n_paths=n, seed=21, method="mc")
    a, g = oracle.asian_paths(s, k, r, sigma, t, steps, strike_type=strike, option_type=opt, q=q, n_paths=n, seed=21)
    use_cv = avg == "arithmetic" and strike == "fixed"
    geo = _geo_analytical(stocha, s, k, r, sigma, t, q) if use_cv else 0.0
    # the opt of the geometric control variate is the same option type
    if use_cv and opt == "put":
        geo = stocha.asian_price(s, k, r, sigma, t, average_type="geometric", method="analytical", q=q,
                                 option_type="put")
    want = oracle.asian_estimate(a, g, use_cv, geo, math.exp(-r * t))
    assert abs(got - want) <= ASIAN_RTOL * abs(want), (got, want)


def test_asian_seasoned_mc_matches_oracle(stocha, oracle):
    # fixed strike: the seasoned option is a scaled fresh one with strike K*
    kw = dict(s=100.0, k=100.0, r=0.05, sigma=0.2, t=1.0, n_steps=252, n_paths=20_000, seed=1)
    got = stocha.asian_price(**kw, method="mc", running_avg=98.0, time_elapsed=0.5)
    kstar, rem = (1.0 * 100.0 - 0.5 * 98.0) / 0.5, 0.5
    fresh = stocha.asian_price(100.0, kstar, 0.05, 0.2, rem, n_steps=252, n_paths=20_000, seed=1, method="mc")
    assert got == 0.5 * fresh and got > 0
    # floating strike: remaining period simulated with the spent average blended in
    for avg in ("arithmetic", "geometric"):
        got = stocha.asian_price(**kw, method="mc", strike_type="floating", average_type=avg, running_avg=95.0,
                                 time_elapsed=0.3)
        want = oracle.asian_floating_seasoned(100.0, 0.05, 0.2, 1.0, 252, avg, "call", 95.0, 0.3, n_paths=20_000,
                                              seed=1)
        assert abs(got - want) <= ASIAN_RTOL * abs(want), (avg, got, want)


def test_asian_mc_reference_expectations(stocha):
    arith = stocha.asian_price(100, 100, 0.05, 0.2, 1.0, method="mc", n_paths=200_000, seed=42)
    geo = stocha.asian_price(100, 100, 0.05, 0.2, 1.0, average_type="geometric", method="analytical")
    assert arith >= geo * 0.90
    assert stocha.asian_price(100, 105, 0.05, 0.2, 1.0, option_type="put") > 0
    assert stocha.asian_price(100, 100, 0.05, 0.2, 1.0, strike_type="floating") > 0
    p1 = stocha.asian_price(100, 100, 0.05, 0.2, 1.0, method="mc", seed=123)
    assert p1 == stocha.asian_price(100, 100, 0.05, 0.2, 1.0, method="mc", seed=123)


@pytest.mark.parametrize("strike,opt", [("floating", "call"), ("floating", "put"), ("fixed", "call"),
                                        ("fixed", "put")])
@pytest.mark.parametrize("season", [False, True])
def test_lookback_mc_matches_oracle(stocha, oracle, strike, opt, season):
    extra = dict(running_max=112.0, running_min=91.0) if season else {}
    kw = dict(s=100.0, r=0.05, sigma=0.3, t=0.75, n_steps=120, strike_type=strike, option_type=opt, k=100.0, q=0.02,
              n_paths=20_000, seed=8, **extra)
    got = stocha.lookback_price(**kw, method="mc")
    want = oracle.lookback_mc(**kw)
    assert abs(got - want) <= MC_RTOL * abs(want), (got, want)


def test_lookback_mc_reference_expectations(stocha):
    analytical = stocha.lookback_price(100, 0.05, 0.2, 1.0, method="analytical")
    mc = stocha.lookback_price(100, 0.05, 0.2, 1.0, method="mc", n_paths=200_000)
    assert mc < analytical * 1.05
    assert stocha.lookback_price(100, 0.05, 0.2, 1.0, method="mc", seed=99) == \
        stocha.lookback_price(100, 0.05, 0.2, 1.0, method="mc", seed=99)
    # a running minimum above spot has no closed form: "auto" falls back to the Monte Carlo
    p = stocha.lookback_price(100, 0.05, 0.2, 1.0, running_min=110.0, n_paths=50_000)
    assert math.isfinite(p) and p > 0


# FP32 form (a GB300 addition): the same draws, log-space FP32 paths.  Lookback
# and Asian prices are continuous in the path values, so they stay within
# rounding of the FP64 form; a barrier decision flips only for a path within
# ~1e-7 of the barrier in log price at a monitoring date, which moves the
# price by a small fraction of its Monte Carlo standard error.
FP32_RTOL = 2e-5
FP32_BARRIER_RTOL = 3e-3


@pytest.mark.parametrize("btype,h", [("up-and-out", 120.0), ("down-and-in", 90.0)])
def test_barrier_fp32_close_to_fp64(stocha, btype, h):
    kw = dict(s=100, k=100, r=.05, sigma=.2, t=1., barrier=h, barrier_type=btype, method="mc", n_paths=400_000,
              n_steps=252, rebate=2.0)
    p64 = stocha.barrier_price(**kw)
    p32 = stocha.barrier_price(**kw, precision="fp32")
    assert abs(p32 - p64) <= FP32_BARRIER_RTOL * abs(p64), (p32, p64)


@pytest.mark.parametrize("avg,strike", [("arithmetic", "fixed"), ("geometric", "floating"),
                                        ("arithmetic", "floating")])
def test_asian_fp32_close_to_fp64(stocha, avg, strike):
    kw = dict(s=100, k=100, r=.05, sigma=.2, t=1., n_steps=252, average_type=avg, strike_type=strike,
              method="mc", n_paths=200_000)
    p64 = stocha.asian_price(**kw)
    p32 = stocha.asian_price(**kw, precision="fp32")
    assert abs(p32 - p64) <= FP32_RTOL * abs(p64), (p32, p64)
    # seasoned floating strike (the block-sum kind)
    kw.update(strike_type="floating", running_avg=103.0, time_elapsed=0.3)
    assert abs(stocha.asian_price(**kw, precision="fp32") - stocha.asian_price(**kw)) <= \
        FP32_RTOL * abs(stocha.asian_price(**kw))


@pytest.mark.parametrize("strike,opt", [("floating", "call"), ("fixed", "put")])
def test_lookback_fp32_close_to_fp64(stocha, strike, opt):
    kw = dict(s=100.0, r=0.05, sigma=0.3, t=0.75, n_steps=120, strike_type=strike, option_type=opt, k=100.0,
              q=0.02, n_paths=200_000, seed=8, running_max=112.0, running_min=91.0, method="mc")
    p64 = stocha.lookback_price(**kw)
    p32 = stocha.lookback_price(**kw, precision="fp32")
    assert abs(p32 - p64) <= FP32_RTOL * abs(p64), (p32, p64)
