"""Precision form (FP32 pair and k-space arithmetic, FP64 S(k) and running
totals) on the GPU against the reference's golden fixtures.

Tolerances: dE within 2e-5 of the scale max(1, |dE_pair|, |dE_ewald|) of
the reference's FP64 value; energies from the FP64 recompute within 1e-10."""
import numpy as np
import pytest

from _cases import CASES, de_moves, load, rel

pytestmark = pytest.mark.gpu
TOL32 = 2e-5


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.parametrize("case", CASES)
def test_fp32_energy_difference(pg, case):
    d, g = load(case)
    s = pg.System(d, form=pg.FORM_FP32)
    np.testing.assert_allclose(s.energies(), g["energies"], rtol=1e-10, atol=1e-10)
    worst = 0.0
    for m, trial, moved, exp in de_moves(g):
        got = s.energy_difference(m, trial, moved)
        s.finalize(False)
        if exp[0] >= 1e8:
            assert got[0] >= 1e8
            continue
        scale = max(1.0, abs(exp[1]), abs(exp[2]))
        worst = max(worst, rel(got[0], exp[0], scale))
    assert worst < TOL32, worst


@pytest.mark.parametrize("case", CASES)
def test_fp32_replay_agrees_until_a_near_tie(pg, case, built):
    """On the recorded stream the FP32 chain takes the reference's decisions;
    a decision may only differ where u is within FP32 error of exp(-dE), after
    which the chains legitimately diverge. Require at least 150 agreeing steps."""
    d, g = load(case)
    s = pg.System(d, form=pg.FORM_FP32)
    n = len(g["run_type"])
    used, mt, ac, et = s.run_moves(built.mt19937(int(g["run_seed"]), 400000), n)
    same = (mt == g["run_type"]) & (ac == g["run_accept"])
    first = n if same.all() else int(np.argmin(same))
    assert first >= 150, first
    k = min(first, n) - 1
    assert rel(et[k], g["run_etot"][k], max(1.0, abs(g["run_etot"][k]))) < 1e-4


def test_fp32_drift_is_reset_by_recompute(pg):
    d, _ = load("bulk_medium")
    s = pg.System(d, form=pg.FORM_FP32)
    s.set_recompute(512)
    s.seed(5)
    s.run(2048)
    dr = s.drift()
    e = s.energies()
    assert abs(dr[4]) < 1e-3 * max(1.0, abs(e.sum()))
    fresh = s.total_energy()[:4]
    np.testing.assert_allclose(s.energies(), fresh, rtol=1e-10, atol=1e-9)


def test_fp32_and_fp64_agree_statistically_short(pg):
    """Same stream, same start: over 3000 moves both forms visit configurations
    with the same mean energy to well within the fluctuation."""
    d, _ = load("bulk_small")
    a = pg.System(d, form=pg.FORM_FP32)
    b = pg.System(d, form=pg.FORM_FP64)
    a.seed(11)
    b.seed(11)
    ea, eb = [], []
    for _ in range(30):
        a.run(100)
        b.run(100)
        ea.append(a.energies().sum())
        eb.append(b.energies().sum())
    ea, eb = np.array(ea[10:]), np.array(eb[10:])
    sd = np.sqrt(ea.var() + eb.var()) + 1e-9
    assert abs(ea.mean() - eb.mean()) < 4 * sd
