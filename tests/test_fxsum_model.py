"""The fixed-point neighbour sum of the explicit steps (csrc/fxsum.cuh),
restated with Python integers and checked against exact rational sums.

The CUDA code forms a sum of K doubles as follows:
  - each term becomes T = +-mantissa * 2^5 with the exponent ek = max(e, 1);
  - the terms are aligned to the largest ek by arithmetic right shifts (floor);
  - they are added exactly;
  - the total is rounded once to nearest-even.
Sums whose largest biased exponent lies outside [64, 2000] take the sequential
FP64 sum instead.  These tests pin the algorithm's stated error bound on
random and adversarial inputs: one rounding of the exact sum plus less than
K/32 ulp of the largest term.  They also pin its independence of the order of
the terms.  The device code is checked against the oracle by the GPU parity
tests.
"""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

GUARD = 5


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def fx_sum(xs) -> float:
    T, E = [], []
    for x in xs:
        u = _bits(x)
        e = (u >> 52) & 0x7FF
        mag = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
        T.append((-mag if u >> 63 else mag) << GUARD)
        E.append(e if e else 1)
    emax = max(E)
    if emax < 64 or emax > 2000:
        s = xs[0] + xs[1]
        for x in xs[2:]:
            s += x
        return s
    acc = sum(t >> min(emax - e, 63) for t, e in zip(T, E))   # Python >> floors, as the device's arithmetic shift
    if acc == 0:
        return 0.0
    # acc * 2^(emax - 1075 - GUARD), rounded once to nearest-even
    return float(Fraction(acc) * Fraction(2) ** (emax - 1075 - GUARD))


def fx_lap(xs, v: float) -> float:
    """sum(xs) - K v with the centre as -K times its fixed-point form (fx_lap)."""
    K = len(xs)
    T, E = [], []
    for x in list(xs) + [v]:
        u = _bits(x)
        e = (u >> 52) & 0x7FF
        mag = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
        T.append((-mag if u >> 63 else mag) << GUARD)
        E.append(e if e else 1)
    T[-1] *= -K
    emax = max(E)
    if emax < 64 or emax > 2000:
        s = xs[0] + xs[1]
        for x in xs[2:]:
            s += x
        return float(Fraction(-K) * Fraction(v) + Fraction(s))   # fma(-K, v, s)
    acc = sum(t >> min(emax - e, 63) for t, e in zip(T, E))
    assert abs(acc) < 2 ** 62
    return 0.0 if acc == 0 else float(Fraction(acc) * Fraction(2) ** (emax - 1075 - GUARD))


@pytest.mark.parametrize("k", [4, 6])
def test_laplacian_numerator_error_bound(k):
    rng = np.random.default_rng(20 + k)
    for _ in range(4000):
        c = rng.uniform(-1.0, 1.0) * 2.0 ** rng.integers(-30, 30)
        xs = [float(c * (1 + d)) for d in rng.normal(0, 1e-6, k)]
        got = fx_lap(xs, c)
        exact = sum(Fraction(x) for x in xs) - k * Fraction(c)
        biggest = max(max(abs(x) for x in xs), k * abs(c))
        bound = Fraction(1, 2) * _ulp(float(exact)) + Fraction(k + 1, 32) * _ulp(biggest)
        assert abs(Fraction(got) - exact) <= bound


def _ulp(x: float) -> Fraction:
    m, e = math.frexp(abs(x)) if x != 0 else (0.5, -1074)
    return Fraction(2) ** (e - 53)


def _check(xs):
    got = fx_sum(xs)
    exact = sum(Fraction(x) for x in xs)
    biggest = max(abs(x) for x in xs)
    err = abs(Fraction(got) - exact)
    bound = Fraction(1, 2) * _ulp(float(exact)) + Fraction(len(xs), 32) * _ulp(biggest) if exact != 0 else \
        Fraction(len(xs), 32) * _ulp(biggest)
    assert err <= bound, (xs, got, float(exact))
    return got


@pytest.mark.parametrize("k", [4, 6])
def test_error_bound_on_random_stencils(k):
    rng = np.random.default_rng(k)
    for _ in range(4000):
        scale = rng.integers(-40, 40)
        xs = [float(v) for v in rng.uniform(-1, 1, k) * 2.0 ** (scale + rng.integers(-3, 4, k))]
        _check(xs)


@pytest.mark.parametrize("k", [4, 6])
def test_error_bound_under_cancellation(k):
    """Laplacian-like stencils: terms close to one value, so that the sum cancels."""
    rng = np.random.default_rng(10 + k)
    for _ in range(4000):
        c = rng.uniform(0.1, 1.0) * (-1) ** rng.integers(0, 2)
        xs = [float(c + d) for d in rng.normal(0, 1e-9, k - 1)]
        xs.append(float(-sum(Fraction(x) for x in xs[:-1]) + Fraction(rng.normal(0, 1e-14))))
        _check(xs)


def test_wide_exponent_spread_and_signed_zeros():
    cases = [
        [1.0, -1.0, 1e-300, -0.0],
        [1e200, 1.0, -1e200, 2.0 ** -40],
        [2.0 ** 900, 2.0 ** 850, -(2.0 ** 900), 3.0],
        [0.0, -0.0, 0.0, -0.0],                      # all zero: the sequential fallback, +0
        [1e-310, -3e-309, 2e-308, 5e-324],           # subnormal only: the fallback
        [0.1, 0.2, 0.3, -0.6, 1e-17, -1e-17],
    ]
    for xs in cases:
        got = _check(xs) if any(xs) else fx_sum(xs)
        assert not math.isnan(got)
    assert math.copysign(1.0, fx_sum([0.0, -0.0, 0.0, -0.0])) == 1.0


def test_order_independent():
    rng = np.random.default_rng(3)
    for _ in range(500):
        xs = [float(v) for v in rng.normal(0, 1, 6) * 2.0 ** rng.integers(-60, 60, 6)]
        ref = fx_sum(xs)
        for _ in range(5):
            rng.shuffle(xs)
            assert fx_sum(xs) == ref
