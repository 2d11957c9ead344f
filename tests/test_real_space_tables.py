"""The tables of h(u) = erfc(sqrt u)/sqrt u behind the real-space Ewald term
(erfc(sqrt(alpha) r)/r = sqrt(alpha) h(alpha r^2)).

FP32 (the precision form's pair kernels), evaluated in float32 as the kernel
does (bin from the exponent and top five mantissa bits of u, w = f/32 from the
18 bits below them, cubic by FMA-free Horner) against scipy's erfc in double
precision. Bar: 3e-7 relative for u < 4 (the FP32 erfc fit it replaces is
good to 1.2e-7, and FP32 rounding of the result is 6e-8); for 4 <= u < 32,
where h is below 1/400 of its value at u = 0.25 (h(0.25) = 0.96, a close
pair), an absolute error under 1e-9: below the FP32 rounding of a close
pair's term. The batch's cut table (variable u' = s u, s = 16 / (alpha
r_c^2)) meets the same bars in u below the cut-off and is exactly zero from
u' = 16 on, past the table's end too.

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
    idx = np.minimum(((bits >> 18) - ((127 - 14) << 5)).astype(np.uint32), len(tab) - 1)
    c = tab[idx]
    w = ((bits & 0x3FFFF) | 0x3F800000).view(np.float32) - np.float32(1.0)  # f / 32, exact
    h = c[:, 3]
    for q in (2, 1, 0):
        h = (h * w + c[:, q]).astype(np.float32)
    return h


def _check_h(got, u):
    special = pytest.importorskip("scipy.special")
    ud = np.asarray(u, np.float64)
    want = special.erfc(np.sqrt(ud)) / np.sqrt(ud)
    low = ud < 4
    rel = np.abs(got[low] - want[low]) / want[low]
    assert rel.max() < 3e-7, rel.max()
    if (~low).any():
        assert np.abs(got[~low] - want[~low]).max() < 1e-9


def test_h32_table_accuracy():
    pytest.importorskip("scipy.special")
    import plum_gb300 as pg
    tab = pg.h32_table()
    assert tab.shape == (19 * 32, 4)
    rng = np.random.default_rng(0)
    u = np.float32(2.0) ** rng.uniform(-14, 5, 400000).astype(np.float32)
    _check_h(_eval(tab, u).astype(np.float64), u)


@pytest.mark.parametrize("arc2", [7.84, 0.3, 25.0])
def test_h32_cut_table(arc2):
    """alpha r_c^2 = 7.84: the 20,000-particle workload (r_c = L/2,
    alpha = (5.6/L)^2); 0.3 and 25 put the cut-off near the ends."""
    pytest.importorskip("scipy.special")
    import plum_gb300 as pg
    s = float(np.float32(16.0 / arc2))  # the batch passes the scale as a float
    tab = pg.h32_table(s, 16.0)
    assert tab.shape == (19 * 32, 4)
    assert not tab[(4 + 14) * 32:].any()  # bins from u' = 16 on
    rng = np.random.default_rng(2)
    up = np.float32(2.0) ** rng.uniform(-14, 4, 400000).astype(np.float32)
    got = _eval(tab, up).astype(np.float64)
    _check_h(got, up.astype(np.float64) / s)
    beyond = np.float32(2.0) ** rng.uniform(4, 9, 1000).astype(np.float32)
    assert not _eval(tab, beyond).any()


def test_h32_table_rejects_bad_scale():
    import plum_gb300 as pg
    with pytest.raises(pg.PlumError):
        pg.h32_table(0.0, 16.0)
    with pytest.raises(pg.PlumError):
        pg.h32_table(1.0, -1.0)


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
