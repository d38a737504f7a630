"""The block-fixed-point split step of Landau `euler` (kernel_variant 5,
csrc/euler.cu: mu_bfp_kernel / update_bfp_kernel), restated with Python
integers and checked on the CPU.

One exponent serves the whole field for a step:
  - emax is the largest biased exponent of |psi|; each value becomes
    X = floor(psi 2^(1080 - emax)), |X| < 2^58;
  - mu = psi (psi^2 + lshift) - c2 sum(X) is formed in integers in units of
    2^lmu, lmu = max(3 s, elin + s) + 2 - 58 with s = emax - 1022 and
    |lshift| + 2 D c2 < 2^elin: psi (psi^2 + lshift) in FP64, truncated to the
    unit, minus floor(sum * (c2's mantissa << 10) / 2^64) shifted to the unit;
  - psi' = fma(c1, double(L) 2^lmu, psi) with L = sum(M_nb) - 2 D M, exact.

These tests pin the integer ranges the device code relies on (no int64
overflow), the per-step error against the exact rational step, and
agreement with the oracle's FP64 run over many steps.  The device kernels are
checked against the oracle by the GPU parity tests.
"""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

import oracle
from chgb import config

GUARD = 5


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _fma(a: float, b: float, c: float) -> float:
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _term(x: float):
    u = _bits(x)
    e = (u >> 52) & 0x7FF
    mag = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
    return (-mag if u >> 63 else mag) << GUARD, (e if e else 1)


def _fixed(x: float, u: int) -> int:
    """floor(x 2^(1080 - u)) for a biased exponent of x at most u (bfp_fixed)."""
    T, ek = _term(x)
    assert u >= ek
    return T >> (u - ek)            # Python's >> floors, as the device's arithmetic shift


def _rolls(a, dims):
    out = 0
    for ax in range(dims):
        out = out + np.roll(a, 1, axis=ax) + np.roll(a, -1, axis=ax)
    return out


def consts(p):
    dx2 = p.dx * p.dx
    c2 = 2.0 * p.k[0] / dx2
    c1 = p.dt * p.M / dx2
    ls = 2.0 * p.dims * c2 - p.model.epsilon
    u = _bits(c2)
    e = (u >> 52) & 0x7FF
    mag = (u & ((1 << 52) - 1)) | ((1 << 52) if e else 0)
    mc = (-mag if u >> 63 else mag) * 1024
    ec = e if e else 1
    lin = abs(ls) + 2.0 * p.dims * abs(c2)
    elin = math.frexp(lin)[1] if lin > 0 else -4000      # lin < 2^elin (ilogb + 1)
    return c1, c2, ls, mc, ec, elin


def bfp_step(psi, dims, p, record=None):
    """One step of the device algorithm on a field of shape (N,)*dims."""
    c1, c2, ls, mc, ec, elin = consts(p)
    emax = max(((_bits(float(v)) >> 52) & 0x7FF) for v in psi.flat)
    s = emax - 1022
    emu = max(3 * s, elin + s) + 2
    lmu = emu - 58
    assert 1 <= emax <= 2046 and -1000 <= lmu <= 900, "the model covers mode 1 only"
    X = np.vectorize(lambda v: _fixed(float(v), emax), otypes=[object])(psi)
    sm = _rolls(X, dims)
    umu = lmu + 1080
    rc = umu + 1021 - emax - ec
    assert rc >= 2
    F = np.vectorize(lambda r: _fixed(float(r) * _fma(float(r), float(r), ls), umu), otypes=[object])(psi)
    C = np.vectorize(lambda sv: ((sv * mc) >> 64) >> rc, otypes=[object])(sm)
    M = F - C
    L = _rolls(M, dims) - 2 * dims * M
    out = np.empty_like(psi)
    for idx in np.ndindex(psi.shape):
        l = int(L[idx])
        ld = math.ldexp(float(l), lmu) if l else 0.0    # float(int) rounds to nearest-even, as __ll2double_rn
        out[idx] = _fma(c1, ld, float(psi[idx]))
    if record is not None:
        record.update(X=max(abs(int(v)) for v in X.flat), M=max(abs(int(v)) for v in M.flat),
                      L=max(abs(int(v)) for v in L.flat), emax=emax, lmu=lmu)
    return out


def exact_step(psi, dims, p):
    """The same step in exact rational arithmetic (the folded Landau form)."""
    c1, c2, ls, *_ = consts(p)
    q = np.vectorize(Fraction, otypes=[object])(psi)
    mu = q * (q * q + Fraction(ls)) - Fraction(c2) * _rolls(q, dims)
    L = _rolls(mu, dims) - 2 * dims * mu
    return q + Fraction(c1) * L


def _params(dims, N, dt=None, k=1.0, eps=0.9):
    return config.params(dims, N, "euler", "landau", dt=dt or (0.01 if dims == 2 else 0.005), k=k, epsilon=eps)


@pytest.mark.parametrize("dims,N", [(2, 16), (3, 8)])
@pytest.mark.parametrize("scale", [0.01, 1.0, 3e5, 1e-30])
def test_step_error_and_integer_ranges(dims, N, scale):
    """One step from fields of several magnitudes: X, M and L stay inside the
    int64 ranges the kernels rely on (|X| < 2^58, |M| < 2^58, |L| < 2^62), and
    the result is within the stated truncation error of the exact step."""
    p = _params(dims, N, dt=1e-12 if scale > 1 else None)
    rng = np.random.default_rng(5)
    psi = rng.uniform(-1.0, 1.0, (N,) * dims) * scale
    psi.flat[0] = scale * (1.0 - 2.0 ** -52)                 # a value at the top of its binade
    rec = {}
    got = bfp_step(psi, dims, p, rec)
    assert rec["X"] < 2 ** 58 and rec["M"] < 2 ** 58 and rec["L"] < 2 ** 62
    want = exact_step(psi, dims, p)
    c1, c2, ls, *_ = consts(p)
    # per mu: two truncations of 2^lmu, the sum's 2D truncations of 2^(emax - 1080)
    # times c2, two roundings of psi (psi^2 + lshift); L gathers 4D mu errors
    unit = Fraction(2) ** rec["lmu"]
    xunit = Fraction(2) ** (rec["emax"] - 1080)
    fmax = max(abs(Fraction(float(r)) * (Fraction(float(r)) ** 2 + Fraction(ls))) for r in psi.flat)
    dmu = 2 * unit + 2 * dims * Fraction(c2) * xunit + fmax * Fraction(2) ** -51
    for idx in np.ndindex(psi.shape):
        w = want[idx]
        bound = Fraction(c1) * (4 * dims * dmu) + abs(w - Fraction(float(psi[idx]))) * Fraction(2) ** -52 \
            + abs(w) * Fraction(2) ** -52
        assert abs(Fraction(float(got[idx])) - w) <= bound, idx


def test_values_at_the_bound():
    """A field whose values sit at +-(2^s - ulp) everywhere in a checkerboard,
    where |sum| and |mu| reach their bounds: no overflow, same bound."""
    dims, N = 3, 8
    p = _params(dims, N, dt=1e-12, k=4.0, eps=-3.0)
    top = 1.0 - 2.0 ** -53
    idx = np.indices((N,) * dims).sum(axis=0)
    psi = np.where(idx % 2 == 0, top, -top)
    rec = {}
    bfp_step(psi, dims, p, rec)
    assert rec["M"] < 2 ** 58 and rec["L"] < 2 ** 62


@pytest.mark.parametrize("dims,N,steps", [(2, 16, 40), (3, 8, 20)])
def test_many_steps_agree_with_the_oracle(dims, N, steps):
    """Stepping the model from the reference's seeded initial field stays
    within 1e-14 (relative max-norm) of the oracle's FP64 run."""
    p = _params(dims, N)
    rho0 = config.init_density(dims, N, [0.0], initial_A=0.5, seed=7)
    psi = rho0.reshape((N,) * dims)
    for _ in range(steps):
        psi = bfp_step(psi, dims, p)
    ref = oracle.OracleSim(p, rho0)
    ref.step(steps)
    want = ref.rho().reshape((N,) * dims)
    assert np.max(np.abs(psi - want)) / np.max(np.abs(want)) <= 1e-14
    # the integer Laplacian sums to zero over the box: mass moves by roundings only
    assert abs(psi.mean() - rho0.mean()) <= 1e-16


def to_double_int(L: int, lmu: int) -> float:
    """The device's bfp_to_double_int, restated: L 2^lmu rounded to the nearest
    double, ties to even, from the leading bit, a shift and the remainder."""
    a = abs(L)
    top = a.bit_length() - 1
    E = top
    if top > 52:
        r = top - 52
        rem, half = a & ((1 << r) - 1), 1 << (r - 1)
        M = a >> r
        if rem > half or (rem == half and (M & 1)):
            M += 1
            if M >> 53:
                M >>= 1
                E += 1
    else:
        M = a << (52 - top)
    bits = ((1 if L < 0 else 0) << 63) | ((E + 1023 + lmu) << 52) | (M & ((1 << 52) - 1))
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def test_integer_rounding_to_double_is_the_conversion():
    """Half of the update's warps convert the exact integer Laplacian L with
    bfp_to_double_int instead of the FP64-pipe conversion; both must give
    float(L) 2^lmu exactly (round to nearest, ties to even): random L of every
    bit length, the ties just below, at and above a power of two, and the
    carry into the next binade."""
    rng = np.random.default_rng(17)
    cases = []
    for bits in range(1, 62):
        for _ in range(40):
            v = int(rng.integers(1 << (bits - 1), 1 << bits, dtype=np.int64)) if bits < 63 else 1
            cases += [v, -v]
    for top in range(53, 62):
        r = top - 52
        base = 1 << top
        for M in (base >> r, (base >> r) + 1, (1 << 53) - 1):
            for rem in (0, 1, (1 << (r - 1)) - 1 if r > 1 else 0, 1 << (r - 1), (1 << (r - 1)) + 1, (1 << r) - 1):
                v = (M << r) + rem
                if 0 < v < (1 << 62):
                    cases += [v, -v]
    for lmu in (-60, -1, 0, 5, 300):
        for L in cases:
            assert to_double_int(L, lmu) == math.ldexp(float(L), lmu), (L, lmu)
