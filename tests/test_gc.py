"""Grand-canonical exchange (Simulation::GCMove with configurational-bias
chain insertion and deletion, simulation.cc:357-404, cbmc.cc:5-442) against
the reference's own runs (tests/golden/gcx_*/gc.npz, make_golden.py gc).

The layouts put the salt first, declared as the run's coion molecules, so
that the exchanged chains stay the last molecules (the reference's deletion
indexes them after phantom + coion + grafted + grafted_counterion); the
charged case uses rigid bonds (see make_golden.py).

* CPU: the oracle's restatement replays the recorded stream with the same
  move types, accept flags and draws, and the same final coordinates.
* GPU: the reference-named host classes (Simulation::Step, GCMove, the
  CBMC insertion and deletion of ForceField) with every growth step's trial
  energies on the device reproduce the same sequence from the same seed.
  Device append/erase of molecules keeps the energies equal to a fresh
  total."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GC = ["gcx_neutral", "gcx_charged"]


def fixture(case):
    d = os.path.join(HERE, "golden", case)
    return d, dict(np.load(os.path.join(d, "gc.npz")))


@pytest.mark.parametrize("case", GC)
def test_oracle_exchange_replays_reference(built, case):
    d, g = fixture(case)
    o = built.Oracle(d)
    n = len(g["run_type"])
    stream = built.mt19937(int(g["run_seed"]), int(g["run_draws"].sum()) + 100000)
    used, mt, ac, et = o.run_stream(n, stream)
    assert (mt >= 5).sum() > 50 and ac[mt >= 5].sum() > 10
    np.testing.assert_array_equal(mt, g["run_type"])
    np.testing.assert_array_equal(ac, g["run_accept"])
    assert used == int(g["run_draws"].sum())
    np.testing.assert_allclose(et, g["run_etot"], rtol=1e-9, atol=1e-9)
    np.testing.assert_array_equal(o.coords(), g["run_coords"])


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("case", GC)
def test_gpu_exchange_replays_reference(case, form):
    """form 0: plain FP64. form 1: the precision form, whose trial energies
    come from the one-launch FP32 kernel (kern_cbmc32.cu) and whose moves use
    the FP32 energy change; a near tie could turn one decision, but on these
    fixtures' 400 steps (over 200 exchange attempts) none does, so the
    sequence and coordinates are the reference's, and the running total
    agrees to the FP32 bound."""
    import plum_gb300 as pg
    d, g = fixture(case)
    sim = pg.HostSimulation(d, seed=int(g["run_seed"]), form=form)
    mt, ac = sim.steps(len(g["run_type"]))
    np.testing.assert_array_equal(mt, g["run_type"])
    np.testing.assert_array_equal(ac, g["run_accept"])
    np.testing.assert_allclose(sim.positions(), g["run_coords"], rtol=0, atol=1e-9)
    tol = 1e-8 if form == 0 else 1e-6
    assert abs(sim.energies().sum() - g["run_etot"][-1]) <= tol * max(1.0, abs(g["run_etot"][-1]))


@pytest.mark.gpu
def test_gpu_append_and_erase_keep_energies_exact():
    import plum_gb300 as pg
    d, _ = fixture("gcx_neutral")
    s = pg.System(d)
    n0 = s.n_bead
    ms, q, ty = s.topology()
    pos = s.positions()
    first = int(np.nonzero(np.diff(ms) > 1)[0][0])  # first chain
    L = int(ms[first + 1] - ms[first])
    chain = pos[ms[first]:ms[first + 1]] + np.array([3.1, 0.7, -2.2])
    s.append_molecules([L], chain, q[ms[first]:ms[first + 1]], ty[ms[first]:ms[first + 1]])
    assert s.n_bead == n0 + L
    np.testing.assert_allclose(s.energies(), s.total_energy()[:4], rtol=1e-12, atol=1e-9)
    s.erase_molecules(s.n_mol - 1, 1)
    assert s.n_bead == n0
    np.testing.assert_array_equal(s.positions(), pos)
    fresh = pg.System(d)
    np.testing.assert_allclose(s.energies(), fresh.energies(), rtol=1e-12, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GC + ["muvt_neutral", "muvt_charged"])
def test_gpu_widom_chemical_potential_matches_oracle(built, case):
    """ForceField::CalcChemicalPotentialF of the host classes (trial energies
    on the device) against the CPU restatement, which
    tests/test_oracle_widom.py pins to the reference: three successive
    averages from the same seed (so the same draws were consumed)."""
    import plum_gb300 as pg
    d = os.path.join(HERE, "golden", case)
    sim = pg.HostSimulation(d, seed=9)
    o = built.Oracle(d, seed=9)
    for _ in range(3):
        a, b = sim.chem_pot(), o.chem_pot()
        assert abs(a - b) <= 1e-6 * abs(b), (case, a, b)
    sim.close()
    o.close()
