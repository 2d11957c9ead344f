"""The wall-force pressure of slit systems (ForceField::CalcPressureForceLJELSlit,
pressure.cc:404-488) on the device against the CPU restatement, and the
restatement's Ewald columns against the reference's own p_tensor
(tests/golden/slab_charged_sites: wall sites of charge +-0.5, so that the
Ewald columns are not zero; made by tests/golden/make_golden.py pressure).

* CPU: the device's per-item arithmetic (plum_gb300/csrc/slit_pressure.h,
  compiled for the host by tests/slit_pressure_harness.cc) over the oracle's
  configurations, against the oracle's evaluation, to 1e-12 of each column's
  sum of |terms|. The reciprocal part is summed as group structure factors
  there instead of over (site, bead) pairs, so this also checks that
  rewriting.
* CPU: the oracle's Ewald columns (p_tensor 3-5, 9-11) against the
  reference's at three configurations. The reference's LJ columns are not
  compared: its PairForce reads an uninitialised local
  (potential_truncated_lj.cc:95-100).
* GPU: plum_pressure_slit at the fixture's configurations against the oracle,
  both forms; the host ForceField's accumulation and the stat file's columns.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
CASE = os.path.join(GOLDEN, "slab_charged_sites")
SLABS = ["slab_charged_sites", "slab_wca", "slab_lj", "slab_hardwall", "slab_wellwall",
         "stat_slab"]
EWALD = [3, 4, 5, 9, 10, 11]


def fixture():
    return dict(np.load(os.path.join(CASE, "pressure.npz")))


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("slit") / "slit_pressure_harness")
    lib = os.path.join(ROOT, "oracle", "_ref")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "slit_pressure_harness.cc"), "-L" + lib, "-loracle",
                        "-Wl,-rpath," + lib, "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("case", SLABS)
def test_device_arithmetic_matches_oracle(harness, case):
    out = subprocess.run([harness, os.path.join(GOLDEN, case), "61", "0", "300"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rows = [np.array([float(x) for x in ln.split()]) for ln in out.stdout.splitlines()]
    assert len(rows) == 2
    first_oracle = rows[0][12:]
    for n, v in enumerate(rows):
        mine, scale, orc = v[:6], v[6:12], v[12:].copy()
        if n:  # the oracle adds the wall-wall terms on its first evaluation only
            orc[[2, 5]] = first_oracle[[2, 5]]
        tol = 1e-12 * np.maximum(scale, 1e-300) + 1e-300
        assert np.all(np.abs(mine - orc) <= tol), (case, n, mine, orc, scale)
    if case == "slab_charged_sites":
        assert np.all(np.abs(rows[0][[3, 4]]) > 1e-3)


def test_oracle_ewald_columns_match_reference(built):
    g = fixture()
    O = built.Oracle(CASE, seed=int(g["run_seed"]))
    for k in range(len(g["coords"])):
        O.set_coords(g["coords"][k])
        p = O.pressure_force_slit()
        want = g["p_tensor"][k]
        for c in EWALD:
            assert abs(p[c] - want[c]) <= 1e-10 * max(1e-3, abs(want[c])), (k, c, p[c], want[c])
    O.close()


def test_fixture_configurations_follow_the_reference_trajectory(built):
    """The fixture's later configurations are where the oracle's own run from
    the same seed arrives (the oracle replays the reference's draws)."""
    g = fixture()
    O = built.Oracle(CASE, seed=int(g["run_seed"]))
    for k in range(1, len(g["coords"])):
        O.run(int(g["steps"]))
        np.testing.assert_allclose(O.coords(), g["coords"][k], rtol=0, atol=1e-9)
    O.close()


def oracle_increments(ob, coords_list, seed):
    """Increments of p_tensor[6..11] of one oracle evaluation per configuration
    (the wall-wall ones from the first evaluation)."""
    O = ob.Oracle(CASE, seed=seed)
    prev = np.zeros(12)
    out = []
    for k, xyz in enumerate(coords_list):
        O.set_coords(xyz)
        p = O.pressure_force_slit()
        inc = (p - prev)[6:12]
        if k:
            inc[[2, 5]] = out[0][[2, 5]]
        out.append(inc)
        prev = p
    O.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_device_pressure_matches_oracle(built, form):
    import plum_gb300 as pg
    g = fixture()
    want = oracle_increments(built, g["coords"], int(g["run_seed"]))
    s = pg.System(CASE, form=form)
    for k, xyz in enumerate(g["coords"]):
        s.set_positions(xyz)
        got = s.pressure_slit()
        np.testing.assert_allclose(got, want[k], rtol=1e-9, atol=1e-11, err_msg=str(k))
    assert np.all(np.abs(want[0][[3, 4]]) > 1e-3)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["slab_lj", "slab_hardwall"])
def test_device_pressure_matches_oracle_other_walls(built, case):
    import plum_gb300 as pg
    d = os.path.join(GOLDEN, case)
    O = built.Oracle(d, seed=3)
    want = O.pressure_force_slit()[6:12]
    O.close()
    s = pg.System(d)
    np.testing.assert_allclose(s.pressure_slit(), want, rtol=1e-9, atol=1e-11)
    s.close()


@pytest.mark.gpu
def test_host_forcefield_accumulates_like_the_reference(built, tmp_path):
    """Two evaluations on the starting configuration through the host
    ForceField: p_tensor[6..11] and the averages 0-5 as pressure.cc:471-487
    forms them; then the stat file of a short run prints GetPressure's six
    columns."""
    import plum_gb300 as pg
    g = fixture()
    want = oracle_increments(built, [g["coords"][0]], int(g["run_seed"]))[0]
    sim = pg.HostSimulation(CASE, seed=5)
    p, n = sim.pressure(evaluate=True)
    assert n == 1
    np.testing.assert_allclose(p[6:12], want, rtol=1e-9, atol=1e-11)
    p2, n = sim.pressure(evaluate=True)
    assert n == 2
    area = 10.0 * 10.0
    np.testing.assert_allclose(p2[[6, 7, 9, 10]], 2 * p[[6, 7, 9, 10]], rtol=1e-12)
    np.testing.assert_allclose(p2[[8, 11]], p[[8, 11]], rtol=0, atol=0)
    np.testing.assert_allclose(p2[[0, 1, 3, 4]], p2[[6, 7, 9, 10]] / (2 * area), rtol=1e-12)
    np.testing.assert_allclose(p2[[2, 5]], p[[8, 11]] / area, rtol=1e-12)
    sim.close()

    for f in ("input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(CASE, f), tmp_path / f)
    lines = open(os.path.join(CASE, "run.in")).read().splitlines()
    item = {ln.split()[0]: i for i, ln in enumerate(lines) if ln.split()}
    for key, v in (("s1_total_simulation_steps", 400), ("s1_equilibrium_steps", 0),
                   ("s1_sampling_frequency", 10), ("s1_sampling_print_frequency", 200)):
        lines[item[key]] = "%s %d" % (key, v)
    prefix = lines[item["s1_prefix_of_output_file_names"]].split()[1]
    (tmp_path / "run.in").write_text("\n".join(lines) + "\n")
    sim = pg.HostSimulation(str(tmp_path), seed=5)
    sim.enable_output(str(tmp_path))
    sim.run()
    p, n = sim.pressure()
    assert n == 4  # steps 100, 200, 300, 400
    sim.finish()
    sim.close()
    stat = [ln for ln in open(tmp_path / (prefix + "_stat.dat")).read().splitlines()
            if ln.strip()]
    assert stat[-1].split()[0] == "400"
    cols = " ".join("%g" % v for v in p[:6])
    assert cols in stat[-1], (cols, stat[-1])
