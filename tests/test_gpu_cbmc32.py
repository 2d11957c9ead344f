"""Configurational-bias trial energies in the precision form: all trial sites
of a growth step in one launch with FP32 pair and k-space arithmetic and
FP64 sums across blocks (kern_cbmc32.cu), against the reference's own
BeadsEnergy values (tests/golden/muvt_*/cbmc.npz) and, at the size of the
grand-canonical workload (L = 50, 40 chains of 30, 2,000 salt pairs,
32 trials), against the CPU oracle's FP64 restatement and the plain form.

Tolerance: |u32 - u64| <= 1e-4 + 1e-5 |u64| (k_BT). Each FP32 term carries a
relative error of a few 1e-7 (the squared distance raised to the sixth power
in LJ, the fast reciprocal), so a sum dominated by one close contact is off
by up to ~1e-6 of itself; where u is small enough for its Rosenbluth weight
exp(-u) to matter (u < 10) the bound is 2e-4, a relative weight change far
below the statistical noise of any exchange run. Overlaps (u >= 1e8) must
agree exactly."""
import os

import numpy as np
import pytest

from test_cbmc import rows

pytestmark = pytest.mark.gpu


def close32(a, b):
    if b >= 1e8:
        return a >= 1e8
    return a < 1e8 and abs(a - b) <= 1e-4 + 1e-5 * abs(b)


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.parametrize("case", ["muvt_neutral", "muvt_charged"])
def test_fp32_trial_energies_match_reference(pg, case):
    s = None
    worst = 0.0
    for d, charged, did, b1, b2, chain, ci, u in rows(case):
        s = s or pg.System(d, form=1)
        got = s.cbmc_trials(b1[None], b2[None] if charged else None,
                            chain if len(chain) else None, ci if (charged and len(chain)) else None,
                            did)
        assert close32(got[0], u), (case, did, len(chain), got[0], u)
        if u < 1e8:
            worst = max(worst, abs(got[0] - u))
    print(case, "max |u32 - u_ref|", worst)


def _workload(tmp, charged):
    from plum_gb300 import systems
    d = str(tmp / ("muvt50_%d" % charged))
    spec = systems.MuVTSpec(bead_charge=-1.0 if charged else 0.0, salt_first=True)
    systems.write_muvt(d, spec, seed=31 + charged)
    return d


def _trial_sites(s, rng, T, cl, charged):
    """T trial sites one bond from the end of a grown chain of cl beads
    placed in the box (trial counterions uniform in the box)."""
    box = 50.0
    start = rng.uniform(0, box, 3)
    steps = rng.normal(size=(max(cl, 1), 3))
    steps /= np.linalg.norm(steps, axis=1)[:, None]
    chain = start + np.cumsum(steps, axis=0)[:cl]
    tip = chain[-1] if cl else start
    d = rng.normal(size=(T, 3))
    b1 = tip + d / np.linalg.norm(d, axis=1)[:, None]
    b2 = rng.uniform(0, box, (T, 3)) if charged else None
    ci = rng.uniform(0, box, (cl, 3)) if (charged and cl) else None
    return b1, b2, (chain if cl else None), ci


@pytest.mark.parametrize("charged", [0, 1])
def test_fp32_trials_at_workload_size(pg, built, tmp_path, charged):
    """32 trial sites of growth steps (first bead, mid-chain, deletion of a
    chain) on the 5,200-particle grand-canonical box: the one-launch FP32
    kernel against the plain form's FP64 kernels and, for a few sites, the
    CPU oracle."""
    d = _workload(tmp_path, charged)
    s64 = pg.System(d, form=0)
    s32 = pg.System(d, form=1)
    o = built.Oracle(d)
    rng = np.random.default_rng(5 + charged)
    n_mol = len(s64.topology()[0]) - 1
    worst = worst_small = 0.0
    for cl, did in ((0, -1), (1, -1), (15, -1), (29, -1), (10, n_mol - (31 if charged else 1))):
        b1, b2, chain, ci = _trial_sites(s64, rng, 32, cl, charged)
        u64 = s64.cbmc_trials(b1, b2, chain, ci, did)
        u32 = s32.cbmc_trials(b1, b2, chain, ci, did)
        for t in range(32):
            assert close32(u32[t], u64[t]), (cl, did, t, u32[t], u64[t])
            if u64[t] < 1e8:
                worst = max(worst, abs(u32[t] - u64[t]) / max(1.0, abs(u64[t])))
            if abs(u64[t]) < 50:
                worst_small = max(worst_small, abs(u32[t] - u64[t]))
        for t in (0, 17):
            ref = o.beads_energy(b1[t], None if b2 is None else b2[t], chain, ci, did)
            assert abs(u64[t] - ref) <= 1e-10 * max(1.0, abs(ref)) or (ref >= 1e8 and u64[t] >= 1e8)
            assert close32(u32[t], ref), (cl, did, t, u32[t], ref)
    print("charged", charged, "max |u32 - u64| / max(1, |u64|)", worst,
          "max |u32 - u64| where |u64| < 50", worst_small)


def test_fp32_trials_one_launch_and_deterministic(pg, tmp_path):
    d = _workload(tmp_path, 0)
    s = pg.System(d, form=1)
    rng = np.random.default_rng(9)
    b1, b2, chain, ci = _trial_sites(s, rng, 32, 12, 0)
    a = s.cbmc_trials(b1, b2, chain, ci, -1)
    b = s.cbmc_trials(b1, b2, chain, ci, -1)
    np.testing.assert_array_equal(a, b)
    ms, launches = s.cbmc_time(b1, b2, chain, ci, -1, reps=20)
    assert launches == 1 and ms > 0
    one = s.cbmc_trials(b1[5:6], None, chain, ci, -1)
    assert close32(one[0], a[5])
