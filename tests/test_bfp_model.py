"""CPU model of the block-floating-point FFT arithmetic (csrc/bfp.cuh and the
fixed-point Stockham passes of csrc/spectral.cu), restated with Python
integers and checked against exact rational arithmetic:

* the twiddle product from 31-bit limbs: each component within 1/2 + 2^-29 of
  the exact round(X W / 2^61), every 64-bit intermediate in range, for
  magnitudes up to the 2^61 bound and the extreme twiddles (+-1, +-i);
* the conversions: double -> fixed rounds to nearest (ties away from zero),
  fixed -> double is the correctly rounded nearest double;
* the headroom: a line scaled with G = log2 L + 1 (columns) or log2 M + 3
  (real rows, with the pre/post-processing) never reaches 2^61 in magnitude,
  even for the worst-case input (all values at the maximum, aligned phases);
* a whole fixed-point transform against an exact DFT: the error stays within
  a few units of 2^-(61 - G) times the line's largest component.
"""
import math
import random
from fractions import Fraction

import numpy as np
import pytest

TOP = 61
I64 = 1 << 63


def chk(v):
    assert -I64 <= v < I64, "64-bit overflow"
    return v


def limbs(W):
    return W >> 31, W & 0x7FFFFFFF


def twiddle(c, s):
    """{hx, lx, hy, ly} of w = c + i s (floats), rounded from the value x 2^61."""
    wx = round(Fraction(c) * 2 ** 61)
    wy = round(Fraction(s) * 2 ** 61)
    return limbs(wx) + limbs(wy), (wx, wy)


def lohi(xl, wl):
    return ((xl << 1) * wl) >> 32          # __umulhi(2 xl, wl)


def wide(a, b):
    return chk(a * b)


def cmul(a, w, conj):
    """fx_cmul: a = (X, Y) ints, w = (hx, lx, hy, ly)."""
    X, Y = a
    hx, lx, hy, ly = w
    xh, xl = X >> 31, X & 0x7FFFFFFF
    yh, yl = Y >> 31, Y & 0x7FFFFFFF
    for h in (xh, yh):
        assert -(1 << 31) <= h < (1 << 31)
    r1 = 1 << 29
    a_xx, m_xx = wide(xh, hx), chk(wide(xh, lx) + wide(xl, hx) + lohi(xl, lx))
    a_yy, m_yy = wide(yh, hy), chk(wide(yh, ly) + wide(yl, hy) + lohi(yl, ly))
    a_xy, m_xy = wide(xh, hy), chk(wide(xh, ly) + wide(xl, hy) + lohi(xl, ly))
    a_yx, m_yx = wide(yh, hx), chk(wide(yh, lx) + wide(yl, hx) + lohi(yl, lx))
    if not conj:
        re = chk(2 * chk(a_xx - a_yy)) + (chk(m_xx - m_yy + r1) >> 30)
        im = chk(2 * chk(a_xy + a_yx)) + (chk(m_xy + m_yx + r1) >> 30)
    else:
        re = chk(2 * chk(a_xx + a_yy)) + (chk(m_xx + m_yy + r1) >> 30)
        im = chk(2 * chk(a_yx - a_xy)) + (chk(m_yx - m_xy + r1) >> 30)
    return chk(re), chk(im)


def exact_cmul(a, W, conj):
    X, Y = a
    wx, wy = W
    if conj:
        wy = -wy
    return Fraction(X * wx - Y * wy, 2 ** 61), Fraction(X * wy + Y * wx, 2 ** 61)


@pytest.mark.parametrize("conj", [False, True])
def test_twiddle_product_rounds_once_per_component(conj):
    rng = random.Random(3)
    angles = [0.0, math.pi / 2, math.pi, -math.pi / 2, math.pi / 4] + [rng.uniform(-math.pi, math.pi) for _ in range(60)]
    worst = 0.0
    for ang in angles:
        c, s = math.cos(ang), math.sin(ang)
        if ang in (0.0, math.pi, math.pi / 2, -math.pi / 2):
            c, s = round(c), round(s)      # the table's exact values
        w, W = twiddle(c, s)
        for _ in range(40):
            r = rng.choice([1.0 - 2 ** -40, rng.random(), rng.random() * 2 ** -20, 0.0])
            phi = rng.uniform(-math.pi, math.pi)
            mag = r * (2 ** TOP - 2 ** 12)            # complex magnitude below 2^61
            a = (int(mag * math.cos(phi)), int(mag * math.sin(phi)))
            got = cmul(a, w, conj)
            want = exact_cmul(a, W, conj)
            for g, e in zip(got, want):
                worst = max(worst, abs(Fraction(g) - e))
                assert abs(Fraction(g) - e) <= Fraction(1, 2) + Fraction(1, 2 ** 29)
            assert math.hypot(*got) < 2 ** TOP + 4
    assert worst > Fraction(1, 4)          # the bound is attained, not vacuous


def test_unit_twiddle_is_exact():
    w, _ = twiddle(1.0, 0.0)
    rng = random.Random(5)
    for _ in range(200):
        a = (rng.randrange(-(2 ** 60), 2 ** 60), rng.randrange(-(2 ** 60), 2 ** 60))
        assert cmul(a, w, False) == a and cmul(a, w, True) == a


# ---------------------------------------------------------------- conversions
def expo(v):
    return (np.float64(v).view(np.int64) >> 52) & 0x7FF


def from_double(v, sh):
    b = int(np.float64(v).view(np.int64))
    e = (b >> 52) & 0x7FF
    m = b & ((1 << 52) - 1)
    if e:
        m |= 1 << 52
    else:
        e = 1
    s = e - 1075 + sh
    if s >= 0:
        r = m << s
    else:
        t = -s
        r = 0 if t > 62 else ((m >> (t - 1)) + 1) >> 1
    return -r if b < 0 else r


def to_double(X, sh):
    return float(Fraction(X, 2 ** sh)) if sh >= 0 else float(X * 2 ** (-sh))


def to_double_int(X, sh):
    """fx_to_double of bfp.cuh restated: the nearest double by integer operations."""
    if X == 0:
        return 0.0
    a = abs(X)
    d = a.bit_length() - 53
    E = d - sh + 1075
    sub = E <= 0
    if sub:
        d += 1 - E
    if d > 62:
        q = 0
    elif d > 0:
        q, rem, half = a >> d, a & ((1 << d) - 1), 1 << (d - 1)
        if rem > half or (rem == half and q & 1):
            q += 1
    else:
        q = a << (-d)
    if sub:
        bits = q
    else:
        if q >> 53:
            q >>= 1
            E += 1
        bits = (0x7FF << 52) if E >= 2047 else ((E << 52) | (q & ((1 << 52) - 1)))
    if X < 0:
        bits |= 1 << 63
    return float(np.array(bits, dtype=np.uint64).view(np.float64))


def test_integer_conversion_to_double_is_correctly_rounded():
    """Normal, subnormal and overflowing results of the integer-only path
    against Python's correctly rounded Fraction -> float."""
    rng = random.Random(11)
    Xs = [1, -1, 3, 2 ** 53 + 1, 2 ** 53 + 3, 2 ** 60 - 1, -(2 ** 61 - 3)] + [rng.randrange(-(2 ** 61), 2 ** 61)
                                                                           for _ in range(300)]
    for X in Xs:
        for sh in (0, 17, 51, 60, 1000, 1070, 1074, 1080, 1100, 1130, 1140, -900, -960, -1000):
            f = Fraction(X, 2 ** sh) if sh >= 0 else Fraction(X * 2 ** (-sh))
            try:
                want = float(f)
            except OverflowError:
                want = math.copysign(math.inf, X)
            got = to_double_int(X, sh)
            assert got == want or (got == 0.0 and want == 0.0), (X, sh, got, want)


def scale(emax, G):
    return TOP - G + 1022 - max(emax, 1)


def test_conversions_round_to_nearest():
    rng = np.random.default_rng(7)
    vals = np.concatenate([rng.standard_normal(300), rng.standard_normal(100) * 1e-9, [0.0, -0.0, 1.0, -1.0]])
    emax = int(max(expo(v) for v in vals))
    sh = scale(emax, 11)
    for v in vals:
        X = from_double(v, sh)
        exact = Fraction(float(v)) * (2 ** sh if sh >= 0 else Fraction(1, 2 ** -sh))
        assert abs(X - exact) <= Fraction(1, 2)
        if abs(X - exact) == Fraction(1, 2):
            assert abs(X) > abs(exact)                 # ties away from zero
        assert abs(X) < 2 ** (TOP - 11)
    # fixed -> double: the nearest double (Python's Fraction -> float rounds to nearest even)
    for X in [1, -1, 2 ** 53 + 1, 2 ** 53 + 3, -(2 ** 60 - 1), 12345678901234567, 2 ** 61 - 1]:
        for s in (0, 5, 60, 1000):
            want = float(Fraction(X, 2 ** s))
            assert to_double(X, s) == want


# ------------------------------------------------------------------ transforms
def make_table(N):
    tab = []
    for q in range(N):
        ang = 2 * math.pi * q / N
        c, s = math.cos(ang), -math.sin(ang)
        if 4 * q % N == 0:
            c, s = round(c), round(s)
        tab.append(twiddle(c, s)[0])
    return tab


def fx_fft(line, tab, wstep, inverse):
    """The fixed-point Stockham FFT of spectral.cu (radix 2 first when log2 L is
    odd, then radix 4), on a list of (X, Y) integer pairs."""
    L = len(line)
    src = list(line)
    Ns = 1
    peak = 0
    if int(math.log2(L)) & 1:
        dst = [None] * L
        for j in range(L // 2):
            v0, v1 = src[j], src[j + L // 2]
            dst[2 * j] = (v0[0] + v1[0], v0[1] + v1[1])
            dst[2 * j + 1] = (v0[0] - v1[0], v0[1] - v1[1])
        src, Ns = dst, 2
    while Ns < L:
        dst = [None] * L
        Q = L // 4
        tstride = (Q // Ns) * wstep
        for j in range(Q):
            k = j & (Ns - 1)
            v0, v1, v2, v3 = src[j], src[j + Q], src[j + 2 * Q], src[j + 3 * Q]
            if Ns > 1:
                m = k * tstride
                t2 = cmul(v2, tab[2 * m], inverse)
                t1 = cmul(v1, tab[m], inverse)
                t3 = cmul(v3, tab[3 * m], inverse)
            else:
                t1, t2, t3 = v1, v2, v3
            s0 = (v0[0] + t2[0], v0[1] + t2[1])
            d0 = (v0[0] - t2[0], v0[1] - t2[1])
            s1 = (t1[0] + t3[0], t1[1] + t3[1])
            d1 = (t1[0] - t3[0], t1[1] - t3[1])
            mi = (d1[1], -d1[0])
            o = (j - k) * 4 + k
            dst[o] = (s0[0] + s1[0], s0[1] + s1[1])
            dst[o + 2 * Ns] = (s0[0] - s1[0], s0[1] - s1[1])
            a = (d0[0] + mi[0], d0[1] + mi[1])
            b = (d0[0] - mi[0], d0[1] - mi[1])
            dst[o + Ns], dst[o + 3 * Ns] = (b, a) if inverse else (a, b)
        src = dst
        Ns *= 4
        peak = max(peak, max(math.hypot(*v) for v in src))
    return src, peak


@pytest.mark.parametrize("L", [4, 8, 32, 64, 128])
@pytest.mark.parametrize("inverse", [False, True])
def test_fixed_point_transform_against_exact_dft(L, inverse):
    rng = np.random.default_rng(L + inverse)
    z = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    z[0] += 3.0                                   # a dominant mode, as a field's mean gives
    G = int(math.log2(L)) + 1
    emax = int(max(max(expo(v.real), expo(v.imag)) for v in z))
    sh = scale(emax, G)
    line = [(from_double(v.real, sh), from_double(v.imag, sh)) for v in z]
    out, peak = fx_fft(line, make_table(L), 1, inverse)
    assert peak < 2 ** TOP
    sign = 1 if inverse else -1
    cmax = max(np.abs(z.real).max(), np.abs(z.imag).max())
    for k in range(L):
        want = sum(complex(v) * np.exp(sign * 2j * math.pi * ((j * k) % L) / L) for j, v in enumerate(z))
        got = complex(to_double(out[k][0], sh), to_double(out[k][1], sh))
        # a few units of 2^-(61 - G) of the largest input component per output, plus
        # the reference sum's own FP64 rounding
        assert abs(got - want) <= 8 * 2.0 ** -(TOP - G) * cmax + 4 * L * 2.0 ** -53 * cmax


@pytest.mark.parametrize("L", [8, 64, 256])
def test_headroom_holds_for_the_worst_case_input(L):
    """Every component at the largest value the scale allows, phases aligned so
    that the DC output takes the full sum: no magnitude reaches 2^61."""
    G = int(math.log2(L)) + 1
    c = 2 ** (TOP - G) - 1
    line = [(c, c)] * L
    out, peak = fx_fft(line, make_table(L), 1, False)
    assert peak < 2 ** TOP
    assert out[0] == (L * c, L * c)
