"""The reference-named C++ host classes (include/plum_host.hpp) on the GPU:
Simulation::TranslationalMove's host control flow against the reference's
golden replay, and the device step loop against the host control flow."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from _cases import CASES, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.parametrize("case", CASES)
def test_host_translational_moves_replay_reference(pg, case):
    d, g = load(case)
    sim = pg.HostSimulation(d, seed=int(g["run_seed"]))
    n = len(g["run_type"])
    mt, ac = sim.translational_moves(n)
    np.testing.assert_array_equal(mt, g["run_type"])
    np.testing.assert_array_equal(ac, g["run_accept"])
    assert abs(sim.energies().sum() - g["run_etot"][-1]) < 1e-9 * max(1, abs(g["run_etot"][-1]))
    np.testing.assert_allclose(sim.positions(len(g["run_coords"])), g["run_coords"], atol=1e-9)


@pytest.mark.parametrize("case", ["bulk_small", "slab_lj"])
def test_device_loop_equals_host_control_flow(pg, case):
    d, g = load(case)
    a = pg.HostSimulation(d, seed=2468)
    b = pg.HostSimulation(d, seed=2468)
    a.translational_moves(400)
    b.run_steps(400)
    nb = len(g["run_coords"])
    np.testing.assert_allclose(a.positions(nb), b.positions(nb), atol=1e-9)
    np.testing.assert_allclose(a.energies(), b.energies(), rtol=1e-10, atol=1e-9)
    # both continue from the same generator state
    a.translational_moves(100)
    b.run_steps(100)
    np.testing.assert_allclose(a.positions(nb), b.positions(nb), atol=1e-9)


def test_command_line_driver(pg, tmp_path):
    d, g = load("bulk_small")
    for f in ("input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    text = open(os.path.join(d, "run.in")).read().splitlines()
    text[3] = "s1_total_simulation_steps 500"
    text[5] = "s1_sampling_frequency 50"
    (tmp_path / "run.in").write_text("\n".join(text) + "\n")
    exe = os.path.join(os.path.dirname(pg.LIB_PATH), "plum_gpu")
    out = subprocess.run([exe, "123"], stdin=open(tmp_path / "run.in"), cwd=tmp_path,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "steps 500" in out.stdout and "<Rg^2>" in out.stdout
