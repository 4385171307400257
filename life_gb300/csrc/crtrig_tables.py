#!/usr/bin/env python3
"""Writes crtrig_tables.h: the double-double tables and series coefficients of
the correctly rounded trigonometry in crtrig.h, computed in 400-bit arithmetic
(mpmath) from their definitions.

* atan(k/256), k = 0..256
* sin(j/128) and cos(j/128), j = 0..101 (covers |r| <= pi/4 + 1/256)
* the Taylor coefficients (-1)^n / (2n+1)!, (-1)^n / (2n)!, (-1)^n / (2n+1)
* pi/2 split for the Cody-Waite reduction, pi/2 and pi as double-doubles

Run by hand when the tables change:  python life_gb300/csrc/crtrig_tables.py
"""
import os

import mpmath

mpmath.mp.prec = 400


def dd(v):
    """(hi, lo) with hi = RN(v), lo = RN(v - hi)."""
    h = float(v)
    return h, float(v - mpmath.mpf(h))


def hx(x: float) -> str:
    return "0.0" if x == 0.0 else float.hex(x)


def table(name: str, values) -> str:
    rows = [f"    {hx(h)}, {hx(l)}," for h, l in (dd(v) for v in values)]
    return f"#define {name} \\\n" + " \\\n".join(r for r in rows) + "\n"


def main():
    out = ["/* Generated by crtrig_tables.py (400-bit mpmath); do not edit. */",
           "#ifndef LIFE_CRTRIG_TABLES_H", "#define LIFE_CRTRIG_TABLES_H", ""]
    out.append("/* atan(k/256), k = 0..256: hi, lo pairs */")
    out.append(table("LIFE_CR_ATAN256", [mpmath.atan(mpmath.mpf(k) / 256) for k in range(257)]))
    out.append("/* sin(j/128), cos(j/128), j = 0..101: sin hi, sin lo, cos hi, cos lo */")
    rows = []
    for j in range(102):
        a = mpmath.mpf(j) / 128
        sh, sl = dd(mpmath.sin(a))
        ch, cl = dd(mpmath.cos(a))
        rows.append(f"    {hx(sh)}, {hx(sl)}, {hx(ch)}, {hx(cl)},")
    out.append("#define LIFE_CR_SINCOS128 \\\n" + " \\\n".join(rows) + "\n")
    coef = []
    for n in range(1, 6):
        h, l = dd(mpmath.mpf(-1) ** n / mpmath.factorial(2 * n + 1))
        coef.append(f"#define LIFE_CR_S{n}H {hx(h)}\n#define LIFE_CR_S{n}L {hx(l)}")
        h, l = dd(mpmath.mpf(-1) ** n / mpmath.factorial(2 * n))
        coef.append(f"#define LIFE_CR_C{n}H {hx(h)}\n#define LIFE_CR_C{n}L {hx(l)}")
        h, l = dd(mpmath.mpf(-1) ** n / (2 * n + 1))
        coef.append(f"#define LIFE_CR_A{n}H {hx(h)}\n#define LIFE_CR_A{n}L {hx(l)}")
    out.append("/* series coefficients: S_n = (-1)^n/(2n+1)!, C_n = (-1)^n/(2n)!, A_n = (-1)^n/(2n+1) */")
    out += coef
    pio2 = mpmath.pi / 2
    # Cody-Waite: three 33-bit pieces and a 53-bit tail of pi/2
    pieces, rest = [], pio2
    for _ in range(3):
        p = mpmath.mpf(float(rest))
        m, e = mpmath.frexp(p)
        p = mpmath.ldexp(mpmath.floor(m * 2 ** 33) / 2 ** 33, e)
        pieces.append(float(p))
        rest -= p
    out.append("/* pi/2 = P1 + P2 + P3 + P4 (P1..P3 have 33 significant bits) */")
    for n, p in enumerate(pieces + [float(rest)], 1):
        out.append(f"#define LIFE_CR_PIO2_{n} {hx(p)}")
    out.append(f"#define LIFE_CR_TWO_OVER_PI {hx(float(2 / mpmath.pi))}")
    for name, v in (("PIO2", pio2), ("PI", mpmath.pi), ("PIO4", mpmath.pi / 4), ("TPIO4", 3 * mpmath.pi / 4)):
        h, l = dd(v)
        out.append(f"#define LIFE_CR_{name}_H {hx(h)}\n#define LIFE_CR_{name}_L {hx(l)}")
    out += ["", "#endif"]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "crtrig_tables.h")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
