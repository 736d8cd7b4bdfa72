"""Exotic options, closed forms and argument checks (no GPU involved).

barrier_price / asian_price / lookback_price with method "analytical" (and
"auto" where the closed form applies) run on the host.  The expectations are
the reference's own (tests/test_exotics.py, src/finance/lookback.rs tests):
Haug's rebate values, the Goldman-Sosin-Gatto lookback values, in/out parity,
knocked-already cases, the Broadie-Glasserman-Kou correction's direction,
Kemna-Vorst seasoning cases and the ValueError messages.
"""
import math

import pytest

BASE = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, barrier=120, barrier_type="up-and-out", option_type="call")


def test_barrier_rebates_match_haug(stocha):
    p_no = stocha.barrier_price(**BASE)
    assert stocha.barrier_price(**BASE, rebate=0.0) == p_no
    assert abs((stocha.barrier_price(**BASE, rebate=5, rebate_at_hit=True) - p_no) - 2.0133) < 1e-3
    assert abs((stocha.barrier_price(**BASE, rebate=5, rebate_at_hit=False) - p_no) - 1.9629) < 1e-3
    # already breached: knock-out pays the rebate at once (at hit) or at expiry
    b = dict(BASE, barrier=90)
    assert abs(stocha.barrier_price(**b, rebate=5, rebate_at_hit=True) - 5.0) < 1e-10
    assert abs(stocha.barrier_price(**b, rebate=5, rebate_at_hit=False) - 5.0 * math.exp(-0.05)) < 1e-10


@pytest.mark.parametrize("direction,h", [("up", 110.0), ("down", 90.0)])
@pytest.mark.parametrize("opt", ["call", "put"])
def test_barrier_in_out_parity(stocha, direction, h, opt):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, barrier=h, option_type=opt)
    out = stocha.barrier_price(**kw, barrier_type=f"{direction}-and-out", method="analytical")
    inn = stocha.barrier_price(**kw, barrier_type=f"{direction}-and-in", method="analytical")
    # in + out = vanilla; the closed forms use the reference's A&S normal CDF
    # (|error| < 1.5e-7), so against an exact CDF they agree to ~1e-5
    d1 = (math.log(100 / 100) + (0.05 + 0.02) * 1.0) / 0.2
    van_call = 100 * _ncdf(d1) - 100 * math.exp(-0.05) * _ncdf(d1 - 0.2)
    van = van_call if opt == "call" else van_call - 100 + 100 * math.exp(-0.05)
    assert abs(out + inn - van) < 5e-5


def _ncdf(x):
    return 0.5 * (1 + math.erf(x / math.sqrt(2)))


def test_barrier_knocked_already(stocha):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, method="analytical")
    assert stocha.barrier_price(**kw, barrier=95, barrier_type="up-and-out") == 0.0
    assert stocha.barrier_price(**kw, barrier=105, barrier_type="down-and-out", option_type="put") == 0.0
    ui = stocha.barrier_price(**kw, barrier=95, barrier_type="up-and-in")
    di = stocha.barrier_price(**kw, barrier=105, barrier_type="down-and-in")
    assert ui == di > 10.0  # the vanilla call


def test_barrier_discrete_monitoring_correction(stocha):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, method="analytical")
    cont = stocha.barrier_price(**kw, barrier=120, barrier_type="uo")
    assert stocha.barrier_price(**kw, barrier=120, barrier_type="uo", n_monitoring=None) == cont
    assert stocha.barrier_price(**kw, barrier=120, barrier_type="uo", n_monitoring=12) > cont
    put = dict(kw, option_type="put")
    cont_p = stocha.barrier_price(**put, barrier=80, barrier_type="do")
    assert stocha.barrier_price(**put, barrier=80, barrier_type="do", n_monitoring=12) > cont_p
    assert abs(stocha.barrier_price(**kw, barrier=120, barrier_type="uo", n_monitoring=100_000) - cont) < 1e-2
    assert stocha.barrier_price(**kw, barrier=120, barrier_type="uo", n_monitoring=0) == cont


def test_barrier_short_names_and_dividend(stocha):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, barrier=120)
    assert abs(stocha.barrier_price(**kw, barrier_type="uo") - stocha.barrier_price(**kw)) < 1e-10
    assert stocha.barrier_price(**kw, q=0.02) != stocha.barrier_price(**kw)


def test_barrier_validation(stocha):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, barrier=120)
    with pytest.raises(ValueError, match="Unknown barrier_type"):
        stocha.barrier_price(**kw, barrier_type="sideways")
    with pytest.raises(ValueError, match="Unknown option_type"):
        stocha.barrier_price(**kw, option_type="straddle")
    with pytest.raises(ValueError, match="Unknown method"):
        stocha.barrier_price(**kw, method="pde")
    for key, msg in [("s", "s must be positive"), ("k", "k must be positive"), ("sigma", "sigma must be positive"),
                     ("t", "t must be positive"), ("barrier", "barrier must be positive")]:
        with pytest.raises(ValueError, match=msg):
            stocha.barrier_price(**dict(kw, **{key: 0.0}))


def test_lookback_closed_forms(stocha):
    assert abs(stocha.lookback_price(100, 0.05, 0.2, 1.0) - 17.2169) < 1e-3
    assert abs(stocha.lookback_price(100, 0.05, 0.2, 1.0, option_type="put") - 12.3398) < 1e-3
    # ATM with K = M = S: the fixed call equals the floating call (reflection)
    fixed = stocha.lookback_price(100, 0.05, 0.2, 1.0, strike_type="fixed", k=100)
    assert abs(fixed - 17.2169) < 1e-3
    assert stocha.lookback_price(100, 0.05, 0.2, 1.0, q=0.03) != stocha.lookback_price(100, 0.05, 0.2, 1.0)
    with pytest.raises(ValueError, match="k must be positive for fixed strike lookback"):
        stocha.lookback_price(100, 0.05, 0.2, 1.0, strike_type="fixed")
    with pytest.raises(ValueError, match="Unknown strike_type"):
        stocha.lookback_price(100, 0.05, 0.2, 1.0, strike_type="average")
    # a running minimum above spot has no closed form
    with pytest.raises(ValueError, match="Analytical solution not available"):
        stocha.lookback_price(100, 0.05, 0.2, 1.0, method="analytical", running_min=110)


def test_asian_geometric_closed_form_and_seasoning(stocha):
    kw = dict(s=100, k=100, r=0.05, sigma=0.2, t=1.0, average_type="geometric", method="analytical")
    p = stocha.asian_price(**kw)
    assert 0 < p < 15.0
    assert stocha.asian_price(**kw, running_avg=None, time_elapsed=None) == p
    assert stocha.asian_price(**kw, running_avg=98, time_elapsed=0.5) > 0
    deep = dict(kw, running_avg=200, time_elapsed=0.9)
    assert abs(stocha.asian_price(**dict(deep, sigma=0.1)) - stocha.asian_price(**dict(deep, sigma=0.5))) < 0.5
    assert stocha.asian_price(**deep, option_type="put") == 0.0
    assert abs(stocha.asian_price(**dict(kw, running_avg=120, time_elapsed=1.0)) - 20.0) < 1e-10
    assert abs(stocha.asian_price(**dict(kw, running_avg=80, time_elapsed=1.0), option_type="put") - 20.0) < 1e-10
    lo = stocha.asian_price(**dict(kw, running_avg=95, time_elapsed=0.5))
    hi = stocha.asian_price(**dict(kw, running_avg=105, time_elapsed=0.5))
    assert hi > lo
    with pytest.raises(ValueError, match="Unknown average_type"):
        stocha.asian_price(100, 100, 0.05, 0.2, 1.0, average_type="harmonic")
    with pytest.raises(ValueError, match="only available for geometric average with fixed strike"):
        stocha.asian_price(100, 100, 0.05, 0.2, 1.0, method="analytical")


def test_exotic_precision_validation(stocha):
    """precision is checked before any CUDA call; the closed forms ignore it."""
    with pytest.raises(ValueError, match="precision must be 'fp64' or 'fp32'"):
        stocha.barrier_price(100, 100, .05, .2, 1., 120, method="mc", precision="fp16")
    with pytest.raises(ValueError, match="precision must be 'fp64' or 'fp32'"):
        stocha.asian_price(100, 100, .05, .2, 1., method="mc", precision="bf16")
    with pytest.raises(ValueError, match="precision must be 'fp64' or 'fp32'"):
        stocha.lookback_price(100, .05, .2, 1., method="mc", precision="half")
    a = stocha.barrier_price(100, 100, .05, .2, 1., 120, method="analytical")
    assert stocha.barrier_price(100, 100, .05, .2, 1., 120, method="analytical", precision="fp32") == a
