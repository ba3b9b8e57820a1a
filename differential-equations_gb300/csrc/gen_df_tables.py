"""Generates df_tables.inc: the tables of the FP32-pair sin and cos (df_math.cuh).  Needs mpmath
(shipped with sympy) only when regenerating; the generated file is committed.

Contents
  DF_PIO64_1..3   pi/64 as three FP32 parts (pi/64 = C1 + C2 + C3 to about 2^-72)
  DF_64_OVER_PI   64/pi rounded to FP32 (picks the table point; its rounding only moves the
                  remainder by a fraction of an ulp of it)
  DF_TRIG_TAB     sin(j pi/64), cos(j pi/64) for j = 0..127 as (hi, lo) FP32 pairs, one
                  16-byte row per j: sin hi, sin lo, cos hi, cos lo
and for the plain FP64 sin and cos (f64_tab_math.cuh):
  F64_PIO64_1, _2 pi/64 as two doubles
  F64_64_OVER_PI  64/pi rounded to a double
  F64_TRIG_TAB    sin(j pi/64), cos(j pi/64) for j = 0..127 as double-double values, one
                  32-byte row per j: sin hi, cos hi, sin lo, cos lo
"""
import os

import mpmath as mp

mp.mp.prec = 300


def f32_exact(v):
    """Nearest FP32 number to the mpf v (rounded once, from the exact value)."""
    if abs(v) < mp.mpf(2) ** -126:  # the table's exact zeros (sin pi, cos pi/2, ...) and below
        return 0.0
    e = int(mp.floor(mp.log(abs(v), 2)))
    scale = mp.mpf(2) ** (23 - e)
    return float(mp.nint(v * scale) / scale)


def pair(v):
    hi = f32_exact(v)
    lo = f32_exact(v - mp.mpf(hi))
    return hi, lo


def _hexf(x):
    """An FP32 number as a C hexadecimal float literal."""
    if x == 0.0:
        return "0.0f"
    m, e = mp.frexp(mp.mpf(x))  # x = m 2^e, 0.5 <= |m| < 1
    sign = "-" if x < 0 else ""
    m = abs(m) * 2
    e -= 1
    frac = int(mp.nint((m - 1) * 2 ** 23))
    return f"{sign}0x1.{frac << 1:06x}p{e:+d}f"


def main(out_dir):
    pio64 = mp.pi / 64
    c1 = f32_exact(pio64)
    c2 = f32_exact(pio64 - c1)
    c3 = f32_exact(pio64 - c1 - c2)
    lines = ["// Generated by gen_df_tables.py — do not edit.", "#pragma once",
             f"#define DF_PIO64_1 {_hexf(c1)}",
             f"#define DF_PIO64_2 {_hexf(c2)}",
             f"#define DF_PIO64_3 {_hexf(c3)}",
             f"#define DF_64_OVER_PI {_hexf(f32_exact(64 / mp.pi))}",
             "#define DF_TRIG_TAB_ROWS \\"]
    rows = []
    for j in range(128):
        sh, sl = pair(mp.sin(j * pio64))
        ch, cl = pair(mp.cos(j * pio64))
        rows.append("    {" + ", ".join(_hexf(v) for v in (sh, sl, ch, cl)) + "}")
    lines.append(", \\\n".join(rows))
    d1 = float(pio64)
    d2 = float(pio64 - mp.mpf(d1))
    lines += [f"#define F64_PIO64_1 {float.hex(d1)}", f"#define F64_PIO64_2 {float.hex(d2)}",
              f"#define F64_64_OVER_PI {float.hex(float(64 / mp.pi))}", "#define F64_TRIG_TAB_ROWS \\"]
    rows = []
    for j in range(128):
        vals = []
        for v in (mp.sin(j * pio64), mp.cos(j * pio64)):
            hi = float(v) if abs(v) >= mp.mpf(2) ** -1000 else 0.0
            lo = float(v - mp.mpf(hi)) if hi != 0.0 else 0.0
            vals += [hi, lo]
        rows.append("    {" + ", ".join(float.hex(x) for x in (vals[0], vals[2], vals[1], vals[3])) + "}")
    lines.append(", \\\n".join(rows))
    with open(os.path.join(out_dir, "df_tables.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main(os.path.dirname(os.path.abspath(__file__)))
