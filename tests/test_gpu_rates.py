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
