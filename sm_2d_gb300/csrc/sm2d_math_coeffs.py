#!/usr/bin/env python
"""Constants of sm2d_math.h, derived here from exact values.

Run ``python sm2d_math_coeffs.py`` to print them as C float literals (and
the accuracy of each function, evaluated in float32 arithmetic, against
double-precision libm).  Nothing here is read at build or run time; the
header carries the printed literals.

* ln 2 and pi/2 are split for Cody-Waite reduction (Cody and Waite, Software
  Manual for the Elementary Functions, 1980): a leading part with few
  significant bits, so that k * part is exact, plus the rounded remainder
  (pi/2 in three parts).
* exp, sin, cos: Taylor coefficients 1/n!.
* log: series of 2 atanh(s), coefficients 1/(2k+1).
* erf: Chebyshev least-squares fits (numpy) of erf(x)/x - 1 in t = x^2 on
  [0, 1], and of erf(x) in u = x - mid on [1, 2] and [2, 4], converted to
  monomial coefficients and rounded to float.
"""
import decimal
import math

import numpy as np
from numpy.polynomial import chebyshev as Ch
from numpy.polynomial import Polynomial

decimal.getcontext().prec = 60
PI_2 = decimal.Decimal("1.570796326794896619231321691639751442098584699687552910487")
LN2 = decimal.Decimal("0.6931471805599453094172321214581765680755001343602552541206")
F = np.float32


def lit(x):
    """Shortest decimal literal that reads back as the same float."""
    s = repr(float(np.float32(x)))
    return s + "f"


def lead(d, bits):
    m, e = math.frexp(float(d))
    return math.ldexp(round(m * (1 << bits)) / (1 << bits), e)


def splits():
    l1 = lead(LN2, 16)
    l2 = float(np.float32(float(LN2 - decimal.Decimal(l1))))
    p1 = lead(PI_2, 12)
    r = PI_2 - decimal.Decimal(p1)
    p2 = lead(r, 12)
    p3 = float(np.float32(float(r - decimal.Decimal(p2))))
    return l1, l2, p1, p2, p3


def erf_fits():
    erf = np.vectorize(math.erf)
    x = np.linspace(1e-4, 1.0, 20001)
    c = Ch.chebfit(2 * x * x - 1, erf(x) / x - 1.0, 6)
    near = Polynomial(Ch.cheb2poly(c))(Polynomial([-1, 2])).coef
    out = [("ERF0", near, None)]
    for name, lo, hi, deg in (("ERF1", 1.0, 2.0, 10), ("ERF2", 2.0, 4.0, 12)):
        xs = np.linspace(lo, hi, 40001)
        mid, half = (lo + hi) / 2, (hi - lo) / 2
        c = Ch.chebfit((xs - mid) / half, erf(xs), deg)
        out.append((name, Polynomial(Ch.cheb2poly(c))(Polynomial([0, 1 / half])).coef, mid))
    return out


def main():
    l1, l2, p1, p2, p3 = splits()
    print("ln2 split:", lit(l1), lit(l2))
    print("pi/2 split:", lit(p1), lit(p2), lit(p3))
    print("1/ln2:", lit(1 / math.log(2)), " 2/pi:", lit(2 / math.pi), " sqrt2:", lit(math.sqrt(2)))
    print("exp taylor:", ", ".join(lit(1 / math.factorial(n)) for n in range(8)))
    print("log atanh:", ", ".join(lit(1 / (2 * k + 1)) for k in range(1, 7)))
    print("sin:", ", ".join(lit((-1) ** k / math.factorial(2 * k + 1)) for k in range(1, 6)))
    print("cos:", ", ".join(lit((-1) ** k / math.factorial(2 * k)) for k in range(1, 7)))
    for name, coef, mid in erf_fits():
        print(f"{name} (mid {mid}):", ", ".join(lit(c) for c in coef))


if __name__ == "__main__":
    main()
