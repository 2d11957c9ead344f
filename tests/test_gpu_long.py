"""1e5-step runs against the reference's own (tests/golden/<case>/long.npz,
made by running the reference's step loop: tests/golden/make_golden.py long).

* Replay: the plain FP64 form fed the same recorded mt19937 stream repeats
  the reference's move-type, accept and draw-count sequence for all 1e5
  steps, with the same running energy, Rg and end-to-end distance at every
  100th step and the same final coordinates and rho(z).
* Statistics (tests/golden/stat_*/stats.npz: 8 independently seeded 6e4-step
  runs of the reference on small charged bulk and slab systems): 8
  independently seeded GPU runs from the same start sample the total
  energy, the chain-averaged Rg^2 and rho(z) in 1-sigma bins the same way;
  the means over runs agree with the reference's within 2 combined standard
  errors (from the spread of the per-run means), for the plain FP64 and the
  precision FP32 forms. Same algorithm, same start and same protocol give
  the same expected per-run means whether or not the runs have reached
  equilibrium (these still relax slowly), so the comparison needs none."""
import os

import numpy as np
import pytest

from _cases import load

pytestmark = pytest.mark.gpu

LONG = ["bulk_small", "slab_wca"]


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


def long_fixture(case):
    d, _ = load(case)
    return d, dict(np.load(os.path.join(d, "long.npz")))


def coarse(rz, width=50):
    n = (len(rz) // width) * width
    return rz[:n].reshape(-1, width, 3).mean(axis=1)


@pytest.mark.parametrize("case", LONG)
def test_replay_1e5_steps(pg, built, case):
    d, g = long_fixture(case)
    s = pg.System(d)
    every = int(g["every"])
    n = len(g["run_type"])
    total = int(g["run_draws"].astype(np.int64).sum())
    stream = built.mt19937(int(g["run_seed"]), total + 100000)
    pos = 0
    mts, acs, ets, obs = [], [], [], []
    for _ in range(n // every):
        used, mt, ac, et = s.run_moves(stream[pos:pos + 400 * every], every)
        pos += used
        mts.append(mt)
        acs.append(ac)
        ets.append(et[-1])
        obs.append(s.observables())
    np.testing.assert_array_equal(np.concatenate(mts), g["run_type"])
    np.testing.assert_array_equal(np.concatenate(acs), g["run_accept"])
    assert pos == total
    np.testing.assert_allclose(ets, g["run_etot_sampled"], rtol=1e-7, atol=1e-6)
    np.testing.assert_allclose(np.array(obs)[:, [0, 4]], g["run_obs_sampled"][:, [0, 4]],
                               rtol=1e-8)
    np.testing.assert_allclose(s.positions(), g["run_coords"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(s.rhoz(), g["run_rhoz"], rtol=0, atol=1e-9)


STAT = ["stat_bulk", "stat_slab"]


def stat_fixture(case):
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", case)
    return d, dict(np.load(os.path.join(d, "stats.npz")))


def run_means(samples_e, samples_g, rhoz, burn_samples):
    """Per-run means after the burn-in: energy, Rg^2, rho(z) bins."""
    e = np.array([x[burn_samples:].mean() for x in samples_e])
    g = np.array([x[burn_samples:].mean() for x in samples_g])
    return e, g, np.array(rhoz)


def compare_runs(mine, ref, what):
    """Means of independent runs agree within 2 combined standard errors."""
    for name, a, b in zip(("energy", "Rg2"), mine[:2], ref[:2]):
        sa = a.std(ddof=1) / np.sqrt(len(a))
        sb = b.std(ddof=1) / np.sqrt(len(b))
        assert abs(a.mean() - b.mean()) <= 2.0 * np.hypot(sa, sb), \
            (what, name, a.mean(), b.mean(), sa, sb)
    za, zb = mine[2], ref[2]
    se = np.hypot(za.std(axis=0, ddof=1) / np.sqrt(len(za)), zb.std(axis=0, ddof=1) / np.sqrt(len(zb)))
    live = se > 0
    z = np.abs(za.mean(axis=0) - zb.mean(axis=0))[live] / se[live]
    assert (z <= 2.0).mean() >= 0.85 and z.max() <= 4.0, (what, np.sort(z)[-5:], live.sum())


def ref_means(g):
    burn = int(g["burn"]) // int(g["every"])
    return run_means(g["energy"], g["rg2"], g["rhoz"], burn)


@pytest.mark.parametrize("case", STAT)
@pytest.mark.parametrize("form", [0, 1])
def test_equilibrium_statistics_match_reference(pg, case, form):
    """8 independently seeded runs of the plain (FP64) or precision (FP32)
    form against the reference's 8: mean energy, Rg^2, and the monomer and
    ion z-profiles."""
    d, g = stat_fixture(case)
    steps, every, burn = int(g["steps"]), int(g["every"]), int(g["burn"])
    E, G, Z = [], [], []
    for k in range(len(g["seeds"])):
        s = pg.System(d, form=form)
        s.seed(7000 + k)
        e, gg, z = [], [], []
        for t in range(steps // every):
            s.run(every)
            e.append(s.energies().sum())
            gg.append(s.observables()[0])
            if (t + 1) * every > burn:
                z.append(coarse(s.rhoz()))
        E.append(np.array(e))
        G.append(np.array(gg))
        Z.append(np.mean(z, axis=0))
        s.close()
    compare_runs(run_means(E, G, Z, burn // every), ref_means(g), (case, form))
