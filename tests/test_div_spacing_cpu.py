"""The correctly rounded division by a grid spacing used by the orthorhombic stress update
(div_spacing in elanfmt_gb300/csrc/ewfd_kernels.cuh), restated with exact rational arithmetic and
exact round-to-nearest-even: in FP32, Markstein's correction of the reciprocal product gives the
IEEE quotient on samples of every binade class the kernel sends through it (the device checks the
same over whole binades per spacing before it uses the path, fdiv_verified); in FP64, where each
corrected quotient is checked against its exact residual before it is used, every accepted
quotient is the IEEE one and almost every quotient is accepted."""
from fractions import Fraction

import numpy as np


def rn32(v: Fraction) -> Fraction:
    """v rounded to the nearest float32 (ties to even), subnormals included, as a Fraction."""
    if v == 0:
        return Fraction(0)
    s = -1 if v < 0 else 1
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    q = max(e - 23, -149)                      # weight of the last significand bit
    scaled = a / Fraction(2) ** q
    n = scaled.numerator // scaled.denominator
    rem = scaled - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return s * Fraction(n) * Fraction(2) ** q


def f32(x: float) -> Fraction:
    return Fraction(float(np.float32(x)))


def markstein(x: Fraction, d: Fraction) -> Fraction:
    r = rn32(1 / d)
    q = rn32(x * r)
    e = rn32(x - q * d)
    assert e == x - q * d, "the residual must be exact"
    return q if e == 0 else rn32(q + e * r)


def test_rn32_matches_numpy_rounding():
    rng = np.random.default_rng(0)
    for v in rng.normal(size=200) * 10.0 ** rng.integers(-30, 30, 200):
        assert rn32(Fraction(float(v))) == Fraction(float(np.float32(v)))


def test_markstein_quotient_is_ieee_quotient():
    rng = np.random.default_rng(1)
    spacings = [40.0, 10.0, 12.5, 3.0, 0.1, 7.3, 120.0, 33.33, 1e-3, 5e8]
    for dv in spacings:
        d = f32(dv)
        for scale in (2.0 ** -90, 1.0, 2.0 ** 99):
            sig = 1.0 + rng.integers(0, 1 << 23, 400) / float(1 << 23)
            for s in sig:
                x = Fraction(float(np.float32(s * scale)))
                for xs in (x, -x):
                    assert markstein(xs, d) == rn32(xs / d), (dv, float(xs))
        # significands with an exactly representable quotient (residual 0)
        for k in range(1, 50):
            x = rn32(d * k)
            assert markstein(x, d) == rn32(x / d)


# ---- FP64: the correction step with a per-result check (div_spacing(double)) ----

def rn64(v: Fraction) -> Fraction:
    """v rounded to the nearest float64 (ties to even), normal range, as a Fraction."""
    if v == 0:
        return Fraction(0)
    s = -1 if v < 0 else 1
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    q = e - 52
    scaled = a / Fraction(2) ** q
    n = scaled.numerator // scaled.denominator
    rem = scaled - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return s * Fraction(n) * Fraction(2) ** q


def checked_quotient(x: Fraction, d: Fraction):
    """The kernel's FP64 path: the corrected quotient and whether its check accepts it."""
    r = rn64(1 / d)
    q0 = rn64(x * r)
    e0 = rn64(x - q0 * d)
    q1 = rn64(q0 + e0 * r)
    e1 = rn64(x - q1 * d)
    a = abs(q1)
    ex = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** ex > a:
        ex -= 1
    pow2 = a == Fraction(2) ** ex
    T = Fraction(2) ** (ex - 53 - (1 if pow2 else 0)) * abs(d)
    return q1, abs(e1) < T


def test_fp64_checked_quotient_is_ieee_quotient():
    """Whenever the check accepts, the quotient is the IEEE one; and it accepts almost always."""
    rng = np.random.default_rng(2)
    accepted = total = 0
    for dv in (40.0, 10.0, 12.5, 3.0, 0.1, 7.3, 120.0, 33.33, 1e-3, 5e8, 2.0 ** 40 + 1.0):
        d = Fraction(dv)
        for scale in (2.0 ** -790, 2.0 ** -20, 1.0, 2.0 ** 37, 2.0 ** 790):
            sig = 1.0 + rng.integers(0, 1 << 52, 120, dtype=np.int64) / float(1 << 52)
            xs = [Fraction(float(s * scale)) for s in sig] + [rn64(d * k * Fraction(scale)) for k in range(1, 20)]
            for x in xs:
                for xx in (x, -x):
                    q, ok = checked_quotient(xx, d)
                    total += 1
                    if ok:
                        accepted += 1
                        assert q == rn64(xx / d), (dv, float(xx))
    assert accepted > 0.99 * total, (accepted, total)
