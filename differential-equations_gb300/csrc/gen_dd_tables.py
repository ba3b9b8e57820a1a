"""Generates dd_tables.inc: the double-double constants of the correctly rounded device math
(dd_math.cuh).  Needs mpmath (shipped with sympy) only when regenerating; the generated file is
committed.

Contents
  PIO2_1, PIO2_2   pi/2 split into two 33-bit pieces (k * piece is exact for |k| < 2^20)
  PIO2_3, PIO2_4   the next two 53-bit pieces
  SIN_TAB/COS_TAB  sin(j/64), cos(j/64) for j = 0..52 as (hi, lo) pairs
  INV6, INV120, INV24, INV720   1/6, 1/120, 1/24, 1/720 as (hi, lo) pairs
"""
import os

import mpmath as mp

mp.mp.prec = 400


def split_dd(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi, lo


def round_bits(v, bits):
    """v rounded to a double with at most `bits` significant bits."""
    e = int(mp.floor(mp.log(abs(v), 2)))
    scale = mp.mpf(2) ** (bits - 1 - e)
    return float(mp.nint(v * scale) / scale)


def main():
    out = []
    pio2 = mp.pi / 2
    p1 = round_bits(pio2, 33)
    rem = pio2 - mp.mpf(p1)
    p2 = round_bits(rem, 33)
    rem -= mp.mpf(p2)
    p3 = float(rem)
    rem -= mp.mpf(p3)
    p4 = float(rem)
    out.append("// Generated by gen_dd_tables.py — do not edit.")
    out.append(f"#define DD_PIO2_1 {p1!r}")
    out.append(f"#define DD_PIO2_2 {p2!r}")
    out.append(f"#define DD_PIO2_3 {p3!r}")
    out.append(f"#define DD_PIO2_4 {p4!r}")
    out.append(f"#define DD_TWO_OVER_PI {float(2 / mp.pi)!r}")
    for name, v in (("INV6", mp.mpf(1) / 6), ("INV120", mp.mpf(1) / 120), ("INV24", mp.mpf(1) / 24),
                    ("INV720", mp.mpf(1) / 720)):
        hi, lo = split_dd(v)
        out.append(f"#define DD_{name}_HI {hi!r}")
        out.append(f"#define DD_{name}_LO {lo!r}")
    n = 53
    out.append(f"#define DD_TAB_N {n}")
    rows = []
    for j in range(n):
        x = mp.mpf(j) / 64
        sh, sl = split_dd(mp.sin(x))
        ch, cl = split_dd(mp.cos(x))
        rows.append(f"    {{{sh!r}, {sl!r}, {ch!r}, {cl!r}}},")
    out.append("// {sin hi, sin lo, cos hi, cos lo} of j/64")
    out.append("#define DD_SINCOS_ROWS \\")
    out.extend([r + " \\" for r in rows])
    out.append("")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dd_tables.inc")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
