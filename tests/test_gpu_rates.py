"""Hull-White short-rate paths (src/finance/hull_white.rs) on the device.

The exact transition r <- r e + m + v z has no transcendental per step, so the
device paths equal the oracle's bit for bit (normals exact, same operation
order, no FMA contraction)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,steps", [(1, 1), (1000, 12), (30_000, 252)])
def test_hull_white_bit_exact(stocha, oracle, n, steps):
    got = stocha.hull_white(0.05, 0.1, 0.005, 0.01, 1.0, steps, n, seed=42)
    want = oracle.hull_white(0.05, 0.1, 0.005, 0.01, 1.0, steps, n, seed=42)
    assert got.shape == (n, steps + 1) and np.array_equal(got, want)


def test_hull_white_reference_expectations(stocha):
    p = stocha.hull_white(0.05, 0.1, 0.05, 0.01, 1.0, 12, 100, seed=42)
    assert p.shape == (100, 13) and np.all(p[:, 0] == 0.05)
    # a = 1, theta = 0.05, r0 = 0.10: mean reverts towards theta / a = 0.05
    p = stocha.hull_white(0.10, 1.0, 0.05, 0.01, 5.0, 500, 2000, seed=1)
    assert abs(p[:, -1].mean() - 0.05) < 0.005
    assert np.array_equal(p, stocha.hull_white(0.10, 1.0, 0.05, 0.01, 5.0, 500, 2000, seed=1))


@pytest.mark.parametrize("dim,n", [(1, 1), (2, 1000), (3, 200_001), (7, 5000)])
def test_gaussian_copula_matches_oracle(stocha, oracle, dim, n):
    """One sequential stream: the device's normals (parallel parse) are the
    reference's bit for bit; the uniforms differ by the exp in the normal CDF
    at most (1e-15)."""
    rng = np.random.default_rng(dim)
    a = rng.standard_normal((dim, dim + 2))
    cov = a @ a.T
    d = np.sqrt(np.diag(cov))
    corr = cov / np.outer(d, d)
    corr = (corr + corr.T) / 2
    np.fill_diagonal(corr, 1.0)
    got = stocha.gaussian_copula(corr, n, seed=5)
    want = oracle.gaussian_copula(corr, n, seed=5)
    assert got.shape == (n, dim)
    assert np.max(np.abs(got - want)) <= 1e-15
    assert np.all((got > 0) & (got < 1))


def test_gaussian_copula_reference_expectations(stocha):
    corr = np.array([[1.0, 0.8], [0.8, 1.0]])
    u = stocha.gaussian_copula(corr, 50_000, seed=42)
    assert u.shape == (50_000, 2) and np.all((u > 0) & (u < 1))
    # uniform marginals, positive dependence
    assert abs(u.mean() - 0.5) < 0.01 and np.corrcoef(u.T)[0, 1] > 0.7
    assert np.array_equal(u, stocha.gaussian_copula(corr, 50_000, seed=42))
    assert stocha.gaussian_copula(corr, 0).shape == (0, 2)


def _corr(dim, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((dim, dim + 2))
    cov = a @ a.T
    d = np.sqrt(np.diag(cov))
    corr = cov / np.outer(d, d)
    corr = (corr + corr.T) / 2
    np.fill_diagonal(corr, 1.0)
    return corr


@pytest.mark.parametrize("dim,nu,n", [(1, 3.0, 1), (2, 5.0, 1000), (3, 4.5, 100_001), (8, 30.0, 5000),
                                      (40, 2.5, 2000),
                                      # shape ~1: frequent gamma rejections, so long samples that
                                      # straddle a chunk start beyond the dim + 8 candidate entries
                                      (1, 2.05, 2_000_000)])
def test_student_t_copula_matches_oracle(stocha, oracle, dim, nu, n):
    """One sequential stream with a variable draw count per sample (Marsaglia-
    Tsang rejection), parsed speculatively on the device: every accept/reject
    decision must match the reference's, or every later sample shifts.  The
    uniforms then differ only through libm (log, exp, sin) and the continued
    fraction's stopping test at 3e-7: at most 1e-6, and within 1e-12 for
    all but a few in a thousand."""
    corr = _corr(dim, dim + 11)
    got = stocha.student_t_copula(corr, nu, n, seed=9)
    want = oracle.student_t_copula(corr, nu, n, seed=9)
    assert got.shape == (n, dim)
    err = np.abs(got - want)
    assert np.max(err) <= 1e-6
    assert np.mean(err > 1e-12) <= 3e-3
    assert np.all((got > 0) & (got < 1))


def test_student_t_copula_reference_expectations(stocha):
    corr = np.array([[1.0, 0.5], [0.5, 1.0]])
    u = stocha.student_t_copula(corr, 5.0, 500, seed=42)
    assert u.shape == (500, 2) and np.all((u > 0) & (u < 1))
    u = stocha.student_t_copula(np.array([[1.0, 0.8], [0.8, 1.0]]), 4.0, 100_000, seed=3)
    assert abs(u.mean() - 0.5) < 0.01 and np.corrcoef(u.T)[0, 1] > 0.7
    # tail dependence: joint exceedances of the 0.99 quantile well above independence (1e-4)
    assert np.mean((u[:, 0] > 0.99) & (u[:, 1] > 0.99)) > 1e-3
    assert np.array_equal(u, stocha.student_t_copula(np.array([[1.0, 0.8], [0.8, 1.0]]), 4.0, 100_000, seed=3))
    assert stocha.student_t_copula(corr, 5.0, 0).shape == (0, 2)

