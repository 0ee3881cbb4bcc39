"""The correctly rounded division by a grid spacing used by the orthorhombic stress update
(div_spacing in elanfmt_gb300/csrc/ewfd_kernels.cuh), restated with exact rational arithmetic and
exact round-to-nearest-even to float32: Markstein's correction of the reciprocal product gives
the IEEE quotient on samples of every binade class the kernel sends through it.  The device
checks the same over whole binades per spacing before it uses the path (fdiv_verified)."""
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
