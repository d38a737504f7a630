"""CPU model of two FP64 shortcuts of csrc/common.cuh used by the gel mobility
update (csrc/fields.cu), restated with exactly rounded Python arithmetic (an
FMA is one rounding of the exact rational result) and checked against
200-bit references:

* tab_exp, the table-driven exponential after Tang (ACM TOMS 15, 1989): within
  0.51 ulp of e^x over the gel's range and the whole fast range |x| <= 700,
  exact at 0, the table's constants as the library builds them (L1 with 37
  significant bits, so that n L1 is exact);
* div_known, division by a divisor known in advance with one FMA correction:
  the correctly rounded quotient for the gel's divisors (1 - phi_c, c0) and a
  spread of others, over dividends of many magnitudes.
"""
import math
import random
from fractions import Fraction

import pytest

mpmath = pytest.importorskip("mpmath")

N = 64                        # EXPTAB_N
SHIFT = 6755399441055744.0    # 1.5 2^52


def exact(v):
    """The exact rational value of an mpmath number."""
    m, e = mpmath.mpf(v).man_exp
    return Fraction(m) * Fraction(2) ** e if e >= 0 else Fraction(m, 2 ** (-e))


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


@pytest.fixture(scope="module")
def table():
    mpmath.mp.prec = 200
    t = []
    for j in range(N):
        v = exact(mpmath.mpf(2) ** (mpmath.mpf(j) / N))
        lead = float(v)
        t.append((lead, float(v - Fraction(lead))))
    L = exact(mpmath.log(2) / N)
    L1 = Fraction(math.floor(L * 2 ** 43), 2 ** 43)
    t.append((float(L1), float(L - L1)))
    t.append((float(exact(N / mpmath.log(2))), 0.0))
    return t


def tab_exp(x, t):
    L1, L2 = t[N]
    K = t[N + 1][0]
    tt = fma(x, K, SHIFT)
    nd = tt - SHIFT                   # exact
    n = int(nd)
    r = fma(-nd, L2, fma(-nd, L1, x))
    q = fma(r, 1 / 720, 1 / 120)
    q = fma(q, r, 1 / 24)
    q = fma(q, r, 1 / 6)
    q = fma(q, r, 0.5)
    p = fma(r * r, q, r)
    lead, trail = t[n & (N - 1)]
    v = lead + fma(lead, p, trail)
    return math.ldexp(v, n >> 6)      # the exponent-field add: exact for |x| <= 700


def ulps(x, y):
    e = exact(mpmath.exp(mpmath.mpf(x)))
    return float(abs(Fraction(y) - e) / Fraction(math.ulp(float(e))))


def test_table_constants(table):
    L1, L2 = table[N]
    assert Fraction(L1).denominator <= 2 ** 43 and L1 * 2 ** 43 < 2 ** 37   # 37 significant bits
    # n L1 is exact for every n of the fast range (|n| <= 700 * 64 / ln 2 < 2^16)
    n = 64637
    assert Fraction(n * L1) == n * Fraction(L1)
    assert table[0] == (1.0, 0.0)


def test_exp_within_half_ulp(table):
    mpmath.mp.prec = 200
    rng = random.Random(7)
    xs = ([rng.uniform(-12.0, 0.0) for _ in range(1500)]           # the gel's -c / c0
          + [rng.uniform(-700.0, 700.0) for _ in range(500)]
          + [rng.uniform(-1e-3, 1e-3) for _ in range(200)]
          + [0.0, -0.0, 1e-300, -1e-300, 700.0, -700.0, math.log(2) / 128, -math.log(2) / 128, 1.0, -1.0])
    worst = max(ulps(x, tab_exp(x, table)) for x in xs)
    assert worst <= 0.51, worst
    assert tab_exp(0.0, table) == 1.0 and tab_exp(-0.0, table) == 1.0


def div_known(x, d, y):
    q0 = x * y
    r = fma(-q0, d, x)
    return fma(r, y, q0)


@pytest.mark.parametrize("d", [0.7, 0.1, 0.9, 0.05, 3.0, 0.123456789, 1e-7])
def test_division_by_known_divisor_is_correctly_rounded(d):
    rng = random.Random(int(d * 1e9))
    y = 1.0 / d
    for _ in range(4000):
        x = rng.uniform(-10.0, 10.0) * 10.0 ** rng.randint(-8, 8)
        assert div_known(x, d, y) == x / d, (x, d)
    assert div_known(0.0, d, y) == 0.0
