"""var_cvar (src/risk/var_cvar.rs) on the device against the oracle (sort by
total_cmp).  VaR is the selected element itself: bit-exact.  CVaR is the tail
mean: equal up to summation order (CVAR_RTOL)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CVAR_RTOL = 1e-12


@pytest.mark.parametrize("n", [1, 2, 10, 1001, 1_000_000])
@pytest.mark.parametrize("conf", [0.01, 0.5, 0.9, 0.95, 0.999])
def test_var_cvar_matches_oracle(stocha, oracle, n, conf):
    r = np.random.default_rng(n).standard_normal(n) * 0.02
    v, c = stocha.var_cvar(r, conf)
    wv, wc = oracle.var_cvar(r, conf)
    assert np.float64(v).tobytes() == np.float64(wv).tobytes()
    assert abs(c - wc) <= CVAR_RTOL * abs(wc) + 1e-300


def test_var_cvar_ties_signed_zeros_and_large(stocha, oracle):
    rng = np.random.default_rng(3)
    ties = rng.integers(-5, 6, 200_003).astype(np.float64) * 0.01  # heavy ties around the VaR value
    zeros = np.array([0.0, -0.0, 0.0, -0.0, 0.01, -0.01] * 1000)
    big = rng.standard_normal(20_000_000)
    for r in (ties, zeros, big):
        for conf in (0.5, 0.95):
            v, c = stocha.var_cvar(r, conf)
            wv, wc = oracle.var_cvar(r, conf)
            assert np.float64(v).tobytes() == np.float64(wv).tobytes()
            assert abs(c - wc) <= CVAR_RTOL * max(abs(wc), 1e-12)


def test_var_cvar_reference_expectations(stocha):
    v, c = stocha.var_cvar(np.array([-(i * 0.01) for i in range(1, 11)]), 0.9)
    assert abs(v - 0.10) < 1e-10 and abs(c - 0.10) < 1e-10
    v, c = stocha.var_cvar(np.array([i * 0.01 for i in range(1, 21)]), 0.95)
    assert v < 0 and c <= v + 1e-10
    with pytest.raises(ValueError, match="returns must not contain NaN or Inf"):
        stocha.var_cvar(np.array([0.01, np.nan, 0.02]), 0.95)
    with pytest.raises(ValueError, match="returns must not contain NaN or Inf"):
        stocha.var_cvar(np.array([0.01, -np.inf]), 0.95)
    # one non-finite value at the end of a large array (the check runs inside
    # the first radix pass, spread over the whole grid)
    big = np.random.default_rng(1).standard_normal(3_000_001) * 0.02
    for bad in (np.nan, np.inf, -np.inf):
        big[-1] = bad
        with pytest.raises(ValueError, match="returns must not contain NaN or Inf"):
            stocha.var_cvar(big, 0.99)
