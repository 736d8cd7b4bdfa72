#!/usr/bin/env python3
"""Constants of the table-driven FP64 exponential of the path kernels.

Tang, "Table-driven implementation of the exponential function in IEEE
floating-point arithmetic", ACM TOMS 15(2), 1989:
    exp(t) = 2^(k/N) * exp(r),  k = round(t * N / ln 2),  r = t - k ln2/N,
with N = 256, |r| <= ln2/512.  This script writes
  * 2^(j/256), j = 0..255, each rounded once to the nearest double;
  * N/ln2 (rounded);
  * ln2/N split for an exact Cody-Waite reduction: HI keeps 35 significant
    bits (k * HI is exact for |k| < 2^18, i.e. |t| < 700), LO = ln2/N - HI.

Run:  python stocha_gb300/gen_exp_table.py > stocha_gb300/csrc/exp_table.inc
(needs mpmath; the generated file is committed).
"""
import sys


def main(out=sys.stdout):
    import mpmath as mp

    mp.mp.dps = 60
    n = 256
    w = out.write
    w("/* 2^(j/256) and reduction constants of the table-driven FP64 exponential.\n")
    w("   Generated by stocha_gb300/gen_exp_table.py (mpmath, 60 digits); do not edit. */\n")
    w("#define STOCHA_EXP2_TAB_INIT { \\\n")
    for j in range(n):
        v = float(mp.power(2, mp.mpf(j) / n))
        w(f"  {v.hex()}{',' if j < n - 1 else ''} \\\n")
    w("}\n")
    inv = float(n / mp.log(2))
    c = mp.log(2) / n
    c_d = float(c)
    # keep 35 significant bits: clear the low 18 of the 53
    import struct

    bits = struct.unpack("<Q", struct.pack("<d", c_d))[0] & ~((1 << 18) - 1)
    hi = struct.unpack("<d", struct.pack("<Q", bits))[0]
    lo = float(c - mp.mpf(hi))
    w(f"#define STOCHA_EXP_INV_LN2_N {inv.hex()}\n")
    w(f"#define STOCHA_EXP_LN2_N_HI {hi.hex()}\n")
    w(f"#define STOCHA_EXP_LN2_N_LO {lo.hex()}\n")


if __name__ == "__main__":
    main()
