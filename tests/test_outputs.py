"""The reference's output files (Simulation::PrintStat, PrintTraj,
PrintLastCrd, PrintLastTop, PrintLastRhoZ; simulation.cc:685-1064) written by
the host Simulation over the device state, against the files the reference
itself wrote for the same run (tests/golden/outputs_bulk_small, made by
tests/golden/make_golden.py outputs: bulk_small, seed 77, 3000 steps, 1000
equilibration steps, sampling every 10, stat every 500, trajectory every
1000).

Every line and every non-numeric token must match. A numeric token may
differ from the reference's by one unit in its last printed digit (the
running totals and observables agree with the reference's to about 1e-10,
so only a value within that of a rounding boundary could print differently);
coordinates printed with 18 digits agree within 1e-7 (the replay bound).
"nan" and "-nan" are the same (the sign of 0/0 differs between x86 and Arm).
"""
import math
import os
import shutil

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "outputs_bulk_small")
SRC = os.path.join(HERE, "golden", "bulk_small")
FILES = ("out_stat.dat", "out_traj_p.xyz", "out_traj_c.xyz", "out_traj_a.xyz",
         "out_traj_n.xyz", "out_lastcrd.dat", "out_lastcrd.dat2", "out_lasttop.dat",
         "out_lastrhoZ.dat", "out_lastrhoZ.dat2")


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return None


def _last_digit(tok):
    """Size of one unit in the last printed digit of a numeric token."""
    mant, _, exp = tok.lower().partition("e")
    decimals = len(mant.split(".")[1]) if "." in mant else 0
    return 10.0 ** ((int(exp) if exp else 0) - decimals)


def compare_files(got_path, want_path, coord_tol=None):
    got = open(got_path).read().splitlines()
    want = open(want_path).read().splitlines()
    assert len(got) == len(want), (got_path, len(got), len(want))
    for n, (g, w) in enumerate(zip(got, want)):
        gt, wt = g.split(), w.split()
        assert len(gt) == len(wt), (got_path, n, g, w)
        for k, (a, b) in enumerate(zip(gt, wt)):
            x, y = _num(a), _num(b)
            if y is None or x is None:
                assert a == b, (got_path, n, a, b)
            elif math.isnan(y) or math.isnan(x):
                assert math.isnan(x) and math.isnan(y), (got_path, n, a, b)
            else:
                tol = coord_tol if (coord_tol is not None and 2 <= k <= 4) else \
                    _last_digit(b) * 1.0000001
                assert abs(x - y) <= tol, (got_path, n, k, a, b)


def test_fixture_files_present_and_comparable():
    """The committed reference files parse, and each compares equal to
    itself under the test's rules (the rules themselves)."""
    for f in FILES:
        p = os.path.join(CASE, f)
        assert os.path.exists(p), f
        compare_files(p, p, coord_tol=1e-7 if "lastcrd" in f else None)
    stat = open(os.path.join(CASE, "out_stat.dat")).read().splitlines()
    assert stat[0].startswith("#Step") and len(stat) == 7
    assert _last_digit("3.233") == pytest.approx(1e-3)
    assert _last_digit("-4.20698") == pytest.approx(1e-5)
    assert _last_digit("1.5e-05") == pytest.approx(1e-6)


@pytest.mark.gpu
def test_output_files_match_reference(tmp_path):
    import plum_gb300 as pg
    for f in ("input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(SRC, f), tmp_path / f)
    shutil.copy(os.path.join(CASE, "run.in"), tmp_path / "run.in")
    sim = pg.HostSimulation(str(tmp_path), seed=77)
    sim.enable_output(str(tmp_path))
    sim.run()
    sim.finish()
    sim.close()
    for f in FILES:
        compare_files(tmp_path / f, os.path.join(CASE, f),
                      coord_tol=1e-7 if "lastcrd" in f else None)


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_checkpoint_restart_is_exact(tmp_path, form):
    """300 steps, a checkpoint, 300 more steps; a second Simulation from the
    same inputs (another seed) reads the checkpoint and runs the same 300
    steps: bit-identical positions and energies."""
    import numpy as np
    import plum_gb300 as pg
    a = pg.HostSimulation(SRC, seed=11, form=form)
    a.run_steps(300)
    ck = tmp_path / "state.ckpt"
    a.write_checkpoint(ck)
    a.run_steps(300)
    b = pg.HostSimulation(SRC, seed=99, form=form)
    b.read_checkpoint(ck)
    b.run_steps(300)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.energies(), b.energies())
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["gcx_neutral", "gcx_charged"])
def test_checkpoint_restart_is_exact_with_exchange(tmp_path, case):
    """Runs with grand-canonical exchange: 300 steps (insertions and
    deletions change the molecule list), a checkpoint, 300 more steps. A
    second Simulation from the same inputs (another seed) reads the
    checkpoint, which first gives its context the checkpoint's molecules, and
    runs the same 300 steps: the same molecules, bit-identical positions and
    energies."""
    import numpy as np
    import plum_gb300 as pg
    d = os.path.join(HERE, "golden", case)
    a = pg.HostSimulation(d, seed=11)
    n0 = a.n_bead()
    a.steps(300)
    ck = tmp_path / "gc.ckpt"
    a.write_checkpoint(ck)
    n_ck = a.n_bead()
    a.steps(300)
    b = pg.HostSimulation(d, seed=99)
    b.read_checkpoint(ck)
    assert b.n_bead() == n_ck
    b.steps(300)
    assert a.n_bead() == b.n_bead()
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.energies(), b.energies())
    assert n0 > 0
    a.close()
    b.close()


@pytest.mark.parametrize("case,lines", [("outputs_slab_charged_sites", 5),
                                        ("outputs_gcx_charged", 4)])
def test_wall_and_exchange_fixtures_are_comparable(case, lines):
    """The reference's files of a slab run (charged surface sites) and of an
    exchange run parse under the comparison's rules. In the slab run the
    reference's three LJ pressure columns hold values near 1e8 once sampling
    has started (its PairForce reads an uninitialised local,
    potential_truncated_lj.cc:95-100) while the three Ewald columns are
    ordinary numbers; the exchange run prints its molecule count."""
    d = os.path.join(HERE, "golden", case)
    for f in FILES:
        p = os.path.join(d, f)
        assert os.path.exists(p), f
        compare_files(p, p, coord_tol=1e-7 if "lastcrd" in f else None)
    stat = open(os.path.join(d, "out_stat.dat")).read().splitlines()
    assert len(stat) == lines
    head = stat[0].split()
    last = stat[-1].split()
    assert len(head) == len(last)
    if case == "outputs_slab_charged_sites":
        lj = [float(last[head.index(c)]) for c in ("<Pzz_LJ_ion>", "<Pzz_LJ_pol>")]
        el = [float(last[head.index(c)]) for c in ("<Pzz_EL_ion>", "<Pzz_EL_pol>")]
        assert min(abs(v) for v in lj) > 1e6
        assert max(abs(v) for v in el) < 1.0 and min(abs(v) for v in el) > 0
    else:
        assert int(last[head.index("NoOfMol")]) > 0
