#!/usr/bin/env python3
"""Generate the N=256 ziggurat tables for the standard normal (f(x)=exp(-x^2/2)).

The sampler in stocha (src/dist/normal.rs:18-67) reads three constants:
R (the tail boundary), X[0..256] (right edges of the 256 equal-area layers)
and Y[i] = f(X[i]).  Their values are fixed by the construction in stocha's
scripts/gen_ziggurat_table.py:1-126, which this script restates from the
Marsaglia & Tsang (2000) equal-area recurrence:

  * V(r) = r f(r) + int_r^inf f  (the common layer area),
  * x[0] = r,  x[i] = f^-1( f(x[i-1]) + V / x[i-1] )  for i = 1..N-1,
  * r is the bisection point (200 halvings of [2, 5], 50 significant digits)
    at which x[N-1] first drops to 1e-20; a trial r whose recurrence overshoots
    f(0) = 1 is too small.
  * x[N] = 0 and Y = f(X).

The bisection rule (its bracket, iteration count, working precision and the
1e-20 cut-off) has to be the same as stocha's: X[255] = 1.0000000018e-20 is a
by-product of where the bisection stops, and the device sampler must see the
same doubles.  Output is a C include file of hex-float literals (exact).

Run:  python stocha_gb300/gen_ziggurat.py > stocha_gb300/csrc/ziggurat_table.inc
Needs mpmath (present in the development container, not on the GPU host: the
generated file is committed).
"""
from __future__ import annotations

import sys

N_LAYERS = 256
DIGITS = 50
BISECTIONS = 200
TOP_EDGE = "1e-20"


def _layers(mp, r, n):
    """Equal-area layer edges for tail boundary r; None if f overshoots 1."""
    half = mp.mpf(1) / 2
    f = lambda x: mp.exp(-x * x * half)
    area = r * f(r) + mp.sqrt(2 * mp.pi) / 2 * mp.erfc(r / mp.sqrt(2))
    edges = [r]
    for _ in range(1, n):
        level = f(edges[-1]) + area / edges[-1]
        if level > 1:
            return None, area
        edges.append(mp.sqrt(-2 * mp.log(level)))
    return edges, area


def build(n: int = N_LAYERS):
    import mpmath as mp

    mp.mp.dps = DIGITS
    lo, hi = mp.mpf(2), mp.mpf(5)
    cut = mp.mpf(TOP_EDGE)
    for _ in range(BISECTIONS):
        mid = (lo + hi) / 2
        edges, _ = _layers(mp, mid, n)
        if edges is None:
            lo = mid
        elif edges[n - 1] > cut:
            hi = mid
        else:
            lo = mid
    r = (lo + hi) / 2
    edges, area = _layers(mp, r, n)
    assert edges is not None
    xs = edges + [mp.mpf(0)]
    ys = [mp.exp(-x * x / 2) for x in xs]
    return float(r), float(area), [float(x) for x in xs], [float(y) for y in ys]


def emit(out=sys.stdout):
    r, area, xs, ys = build()
    w = out.write
    w("/* Ziggurat tables, N=256 layers, for f(x)=exp(-x*x/2).\n")
    w("   Generated by stocha_gb300/gen_ziggurat.py (mpmath, 50 digits); do not edit.\n")
    w(f"   r = {r!r}, layer area V = {area!r}. */\n")
    w(f"#define STOCHA_ZIG_R_HEX {r.hex()}\n")
    w("#define STOCHA_ZIG_X_INIT { \\\n")
    for i, x in enumerate(xs):
        w(f"  {x.hex()}{',' if i < len(xs) - 1 else ''} /* X[{i}] */ \\\n")
    w("}\n")
    w("#define STOCHA_ZIG_Y_INIT { \\\n")
    for i, y in enumerate(ys):
        w(f"  {y.hex()}{',' if i < len(ys) - 1 else ''} /* Y[{i}] */ \\\n")
    w("}\n")


if __name__ == "__main__":
    emit()
