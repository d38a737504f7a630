"""The table-driven logarithm of the Wertheim f' (csrc/common.cuh, tab_log),
restated in Python and checked against exact logarithms.

The method follows P. T. P. Tang, ACM TOMS 16 (1990):
  - x = 2^k y with y in [1, 2), and c_j = 1 + (j + 1/2)/128 for the top seven mantissa bits j of y;
  - ln x = k ln 2 + ln c_j + ln(1 + r), with r = (y - c_j) * (1/c_j) rounded;
  - ln(1 + r) is its Taylor polynomial to r^7, in Horner form with FMAs;
  - ln 2 is split in a high part with eleven trailing zero bits and a low part.
The restatement mirrors each FP64 operation; the fused ones are rounded once
through exact rationals.
The device's table is built the same way, rounded from long double.  The test
pins the error below 2 ulp of the result (of 1.0 where |ln x| < 1) on the
arguments f' meets: rho X^4 and X with rho from 1e-13 to 1, so x from about
1e-30 to 1.  The device code is checked against
the oracle by the GPU tests.
"""
import math
import struct
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np
import pytest

getcontext().prec = 50
N = 128


def fma(a: float, b: float, c: float) -> float:
    """a * b + c rounded once (math.fma where the interpreter has it)."""
    if hasattr(math, "fma"):
        return fma(a, b, c)
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _double(u: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", u))[0]


def _table():
    tab = []
    for j in range(N):
        c = 1.0 + (j + 0.5) / N                                    # exact
        tab.append((1.0 / c, float(Decimal(c).ln())))            # correctly rounded, as from long double
    ln2 = Decimal(2).ln()
    hi = _double(_bits(float(ln2)) & ~0x7FF)
    lo = float(ln2 - Decimal(hi))
    return tab, (hi, lo)


TAB, LN2 = _table()


def tab_log(x: float) -> float:
    u = _bits(x)
    se = u >> 52
    assert 1 <= se <= 2046
    j = (u >> 45) & (N - 1)
    y = _double((u & ((1 << 52) - 1)) | 0x3FF0000000000000)
    c = _double(0x3FF0000000000000 | (j << 45) | (1 << 44))
    inv_c, ln_c = TAB[j]
    r = (y - c) * inv_c
    q = fma(r, 1.0 / 7.0, -1.0 / 6.0)
    q = fma(q, r, 1.0 / 5.0)
    q = fma(q, r, -0.25)
    q = fma(q, r, 1.0 / 3.0)
    q = fma(q, r, -0.5)
    p = fma(r * r, q, r)
    k = float(se - 1023)
    return fma(k, LN2[0], ln_c) + fma(k, LN2[1], p)


def _ulps(got: float, x: float) -> float:
    """Error in ulps of the result, or of 1.0 where |ln x| < 1: the f' terms
    the logarithm feeds are of order 10, so its absolute error is what counts
    near x = 1, where any fixed-table method cancels k ln 2 against ln c_j."""
    exact = Decimal(x).ln()
    err = abs(Decimal(got) - exact)
    m, e = math.frexp(max(abs(float(exact)), 1.0))
    return float(err / Decimal(2) ** (e - 53))


def test_error_below_two_ulp_on_f_prime_arguments():
    rng = np.random.default_rng(1)
    worst = 0.0
    for x in 10.0 ** rng.uniform(-30, 0, 3000):
        x = float(x)
        worst = max(worst, _ulps(tab_log(x), x))
    assert worst < 2.0, worst


def test_every_table_interval_and_exact_powers_of_two():
    for j in range(N):
        for frac in (0.0, 0.25, 0.5, 0.75, 0.999):
            x = (1.0 + (j + frac) / N) * 2.0 ** -17
            assert _ulps(tab_log(x), x) < 2.0
    for k in (-1000, -40, -1, 1, 40, 1000):
        assert _ulps(tab_log(2.0 ** k), 2.0 ** k) < 1.0


def test_table_split_of_ln2():
    hi, lo = LN2
    assert _bits(hi) & 0x7FF == 0
    for k in range(-1074, 1024, 37):
        assert float(k) * hi == float(Decimal(k) * Decimal(hi))   # k * hi exact
    assert abs(Decimal(hi) + Decimal(lo) - Decimal(2).ln()) < Decimal(2) ** -98   # lo rounded: ~2^-100
