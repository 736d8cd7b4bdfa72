"""The FP32 samplers on the device against each other and against the oracle.

The fused FP32 pricing kernels and the Greeks batch draw their normals with the
warp-uniform feed (ZigFeed: every lane steps its generator each iteration, the
fast test runs for every draw and only wedge tests and tail draws diverge); the
path, LSMC and exotic kernels call the per-path loop sampler (normal_f32).  Both
must consume exactly the reference's draws (src/dist/normal.rs:18-67: one per
attempt, one more for a wedge test, two per tail iteration) and form the same
FP32 value from them, so on the same streams their normals and the generator
states after the last consumed draw agree bit for bit (but for the sign of an
exact zero).  Against the oracle's
FP64 normals of the same streams the states are equal and the values agree to
FP32 rounding: the value keeps the top 23 of the draw's 53 fraction bits
(|error| <= 2^-23 X[L], 4.4e-7 at most) plus two roundings; a tail draw's value
uses the hardware logarithm.
"""
import numpy as np
import pytest

from oracle import oracle as O
from stocha_gb300 import _lib

N_PATHS = (1 << 16) + 13  # a ragged last warp
N = 256  # normals per stream: ~2.4e5 wedge tests and ~3.7e3 tail attempts in all
R = 3.654152885361009  # the ziggurat's tail start X[0]


def _draws(form: int, seed: int, n_paths: int, n: int):
    out = np.empty((n_paths, n), np.float32)
    state = np.empty((n_paths, 2), np.uint64)
    lib = _lib.load()
    _lib.check(lib.stocha_debug_zigfeed(None, form, seed, n_paths, n, out.ctypes.data, state.ctypes.data))
    return out, state


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [42, 2**64 - 1])
def test_zigfeed_equals_loop_sampler(stocha, seed):
    loop_v, loop_s = _draws(0, seed, N_PATHS, N)
    feed_v, feed_s = _draws(1, seed, N_PATHS, N)
    assert np.array_equal(loop_s, feed_s)
    assert np.array_equal(loop_v, feed_v)
    # bit for bit, except the sign of an exact zero: a draw whose top 23
    # fraction bits are zero has the FP32 value 0 (the reference's is below
    # 2^-23 X[L] in magnitude); the loop sampler applies the draw's sign bit to
    # it, the feed's signed table gives +0 (about one draw in 1.7e7)
    diff = loop_v.view(np.uint32) != feed_v.view(np.uint32)
    assert np.all(feed_v[diff] == 0.0) and int(diff.sum()) <= 8
    # the slow paths were exercised: tail values lie beyond R
    assert int((np.abs(feed_v) > R).sum()) > 100


@pytest.mark.gpu
def test_fp32_samplers_against_oracle(stocha):
    seed = 42
    v, s = _draws(1, seed, N_PATHS, N)
    base, inc = O.pcg_seed(seed)
    block = (N + 1024) * 2
    worst, worst_tail, tails = 0.0, 0.0, 0
    for i in range(0, N_PATHS, 97):
        st = O.pcg_advance(base, inc, i * block)
        z64, _, end = O.stream_fill(st, inc, "standard_normal", N)
        assert int(s[i, 0]) | (int(s[i, 1]) << 64) == end, f"stream {i}: different draws consumed"
        d = np.abs(v[i].astype(np.float64) - z64)
        tail = np.abs(z64) > R
        tails += int(tail.sum())
        worst = max(worst, float(d[~tail].max()))
        if tail.any():
            worst_tail = max(worst_tail, float((d[tail] / np.abs(z64[tail])).max()))
    assert worst <= 9e-7
    assert tails > 0 and worst_tail <= 2e-6
