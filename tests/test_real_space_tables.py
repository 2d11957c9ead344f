"""The tables of h(u) = erfc(sqrt u)/sqrt u behind the real-space Ewald term
(erfc(sqrt(alpha) r)/r = sqrt(alpha) h(alpha r^2)).

FP32 (the precision form's pair kernels), (erfc(sqrt(alpha) r)/r = sqrt(alpha) h(alpha r^2)),
evaluated in float32 exactly as the kernel does (bin from the exponent and top
five mantissa bits of u, v = 1 + the bin-local fraction, cubic by FMA-free
Horner) against scipy's erfc in double precision. Bar: 3e-7 relative for
u < 4 (the FP32 erfc fit it replaces is good to 1.2e-7, and FP32 rounding of
the result is 6e-8); for 4 <= u < 32, where h is below 1/400 of its value at
u = 0.25 (h(0.25) = 0.96, a close pair), an absolute error under 1e-9: below
the FP32 rounding of a close pair's term.

FP64 (every form's FP64 kernels: the plain form's moves, the from-scratch
energies, the FP64 trial energies), evaluated with the kernel's bin
arithmetic against mpmath at 40 digits: 4e-16 relative below u = 8 (two
roundings of the Horner sum; the FP64 erfc it replaces is good to a few
ulps); above, where h < 3e-5, an absolute error under 1e-17."""
import numpy as np
import pytest


def _eval(tab, u):
    u = np.asarray(u, np.float32)
    bits = u.view(np.int32)
    idx = np.clip((bits >> 18) - ((127 - 14) << 5), 0, len(tab) - 1)
    c = tab[idx]
    y = (((bits << 5) & 0x7FFFFF) | 0x3F800000).view(np.float32)  # v = 1 + f
    h = c[:, 3]
    for q in (2, 1, 0):
        h = (h * y + c[:, q]).astype(np.float32)
    return h


def test_h32_table_accuracy():
    special = pytest.importorskip("scipy.special")
    import plum_gb300 as pg
    tab = pg.h32_table()
    assert tab.shape == (19 * 32, 4)
    rng = np.random.default_rng(0)
    u = np.float32(2.0) ** rng.uniform(-14, 5, 400000).astype(np.float32)
    got = _eval(tab, u).astype(np.float64)
    ud = u.astype(np.float64)
    want = special.erfc(np.sqrt(ud)) / np.sqrt(ud)
    low = ud < 4
    rel = np.abs(got[low] - want[low]) / want[low]
    assert rel.max() < 3e-7, rel.max()
    assert np.abs(got[~low] - want[~low]).max() < 1e-9


def test_h64_table_accuracy():
    mp = pytest.importorskip("mpmath")
    import plum_gb300 as pg
    mp.mp.dps = 40
    tab = pg.h64_table()
    assert tab.shape == (17 * 32, 10)
    rng = np.random.default_rng(1)
    for u in 2.0 ** rng.uniform(-12, 5, 3000):
        bits = np.array([u]).view(np.int64)[0]
        idx = int(bits >> 47) - ((1023 - 12) << 5)
        y = np.array([((bits << 5) & 0xFFFFFFFFFFFFF) | 0x3FF0000000000000],
                     np.int64).view(np.float64)[0] - 1.5
        c = tab[idx]
        h = c[8]
        for q in range(7, -1, -1):
            h = h * y + c[q]
        want = float(mp.erfc(mp.sqrt(mp.mpf(u))) / mp.sqrt(mp.mpf(u)))
        if u < 8:
            assert abs(h - want) <= 4e-16 * want, (u, h, want)
        else:
            assert abs(h - want) < 1e-17, (u, h, want)
