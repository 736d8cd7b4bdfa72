#!/usr/bin/env python3
"""Constants of the FP64 kernels' exponential, evaluated on the integer pipes.

Tang's table-driven reduction (ACM TOMS 15(2), 1989) in fixed point:
    exp(t) = 2^(k/256) * exp(r),   k = floor(t * 256/ln2),   r = t - k ln2/256,
so 0 <= r < ln2/256, and exp(r) - 1 by its degree-6 Taylor polynomial with
non-negative terms (unsigned arithmetic throughout).  This script writes, each
rounded once to the nearest integer:
  * 2^(j/256) * 2^63, j = 0..255               (Q63 table)
  * 256/ln2 * 2^54                             (Q54)
  * ln2/256 * 2^72                             (Q72)
  * 2^32/120, 2^32/720, 2^36/24, 2^64/6        (polynomial coefficients)

Run:  python stocha_gb300/gen_exp_table.py > stocha_gb300/csrc/exp_table.inc
(needs mpmath; the generated file is committed).
"""
import sys


def main(out=sys.stdout):
    import mpmath as mp

    mp.mp.dps = 60
    w = out.write

    def q(x, bits):
        v = int(mp.nint(x * mp.mpf(2) ** bits))
        assert 0 < v < 2**64
        return v

    w("/* Q63 table of 2^(j/256) and fixed-point constants of the integer-pipe\n")
    w("   FP64 exponential.  Generated by stocha_gb300/gen_exp_table.py (mpmath,\n")
    w("   60 digits); do not edit. */\n")
    w("#define STOCHA_EXP2_Q63_INIT { \\\n")
    for j in range(256):
        w(f"  0x{q(mp.power(2, mp.mpf(j) / 256), 63):016x}ull{',' if j < 255 else ''} \\\n")
    w("}\n")
    ln2 = mp.log(2)
    w(f"#define STOCHA_IEXP_C54 0x{q(256 / ln2, 54):016x}ull  /* 256/ln2, Q54 */\n")
    w(f"#define STOCHA_IEXP_L72 0x{q(ln2 / 256, 72):016x}ull  /* ln2/256, Q72 */\n")
    w(f"#define STOCHA_IEXP_C120 0x{q(mp.mpf(1) / 120, 32):08x}u  /* 1/120, Q32 */\n")
    w(f"#define STOCHA_IEXP_C720 0x{q(mp.mpf(1) / 720, 32):08x}u  /* 1/720, Q32 */\n")
    w(f"#define STOCHA_IEXP_C24 0x{q(mp.mpf(1) / 24, 36):08x}u  /* 1/24, Q36 */\n")
    w(f"#define STOCHA_IEXP_C6 0x{q(mp.mpf(1) / 6, 64):016x}ull  /* 1/6, Q64 */\n")


if __name__ == "__main__":
    main()
