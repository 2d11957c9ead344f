"""The minimum-image distance of the plain form's fixed-point pair kernels
(k_delta64, k_total64_fix), restated in exact integer and rational
arithmetic on the CPU: positions become u = round(frac(x / L) 2^64) (x / L
rounded in FP64, as on the device), the difference of two is one 64-bit
integer subtraction (its wraparound is the minimum image), and its
conversion to FP64 is the one rounding of each component. Each fraction
carries the rounding of x / L, about one ulp of the coordinate, the same
order as the FP64 coordinate's own representation; so against the exact
minimum-image distance of the FP64 positions (rationals) the distance is off
by at most ~1e-13 sigma, as is the reference's x_j - x_i in FP64 (which is
exact for close pairs, where the fixed-point form keeps the coordinates'
ulp). Far below the parity bar of the energy changes (1e-10 relative)."""
import math
from fractions import Fraction

import numpy as np


def fix64(x, L):
    f = x * (1.0 / L)
    f -= math.floor(f)
    if f >= 1.0:
        f = 0.0
    return round(f * 2.0 ** 64) % 2 ** 64  # round half even, as __double2ull_rn


def fixed_r(a, b, L):
    s = Fraction(L) / 2 ** 64
    r2 = Fraction(0)
    for xa, xb in zip(a, b):
        d = (fix64(xb, L) - fix64(xa, L)) % 2 ** 64
        if d >= 2 ** 63:
            d -= 2 ** 64
        r2 += Fraction(float(d)) ** 2  # the one rounding: int64 -> FP64
    return math.sqrt(float(r2 * s * s))


def exact_r(a, b, L):
    r2 = Fraction(0)
    for xa, xb in zip(a, b):
        d = Fraction(xb) - Fraction(xa)
        d -= Fraction(L) * round(d / Fraction(L))
        r2 += d * d
    return math.sqrt(float(r2)), r2


def reference_r(a, b, L):
    r2 = 0.0
    for xa, xb in zip(a, b):
        d = xb - xa
        d -= L * round(d / L)
        r2 += d * d
    return math.sqrt(r2)


def test_fixed_point_distance_accuracy():
    rng = np.random.default_rng(5)
    L = 80.0
    worst_fix = worst_ref = 0.0
    for k in range(3000):
        a = rng.uniform(-L, 2 * L, 3)  # some outside the box: the fraction wraps them
        if k % 3 == 0:  # close pairs, some far from the origin
            b = a + rng.normal(size=3) * 10.0 ** rng.uniform(-6, 0)
        else:
            b = rng.uniform(0, L, 3)
        r, r2 = exact_r(a, b, L)
        if r2 == 0 or r2 >= Fraction(L * L / 4):
            continue
        tol = 1e-13 + 4e-16 * r
        worst_fix = max(worst_fix, abs(fixed_r(a, b, L) - r) / tol)
        worst_ref = max(worst_ref, abs(reference_r(a, b, L) - r) / tol)
    assert worst_fix < 1.0, worst_fix
    assert worst_ref < 1.0, worst_ref
