"""The synthetic workloads (plum_gb300/systems.py) that stand in for the
reference's inputs: written in the reference's formats, neutral, with no two
beads closer than the generators' minimum separation (0.8 sigma, periodic
axes by the nearest image), chains of unit bonds, walls' sites on their
planes, and the same files for the same seed."""
import os

import numpy as np
import pytest

from plum_gb300 import systems


def read(d):
    rows = [ln.split() for ln in open(os.path.join(d, "input_crd.dat")).read().splitlines()[2:]
            if ln.strip()]
    mol = np.array([int(r[0]) for r in rows])
    sym = [r[1] for r in rows]
    xyz = np.array([[float(v) for v in r[2:5]] for r in rows])
    q = np.array([float(r[5]) for r in rows])
    top = open(os.path.join(d, "input_top.dat")).read().split()
    box = np.array([float(top[top.index(k) + 1]) for k in
                    ("Box_Length_X:", "Box_Length_Y:", "Box_Length_Z:")])
    return mol, sym, xyz, q, box


def min_pair_distance(xyz, box, periodic):
    best = np.inf
    for i in range(len(xyz) - 1):
        d = xyz[i + 1:] - xyz[i]
        for a in range(3):
            if periodic[a]:
                d[:, a] -= box[a] * np.round(d[:, a] / box[a])
        best = min(best, float(np.sqrt((d * d).sum(axis=1)).min()))
    return best


@pytest.mark.parametrize("kind", ["bulk", "brush", "muvt"])
def test_workload_is_well_formed(tmp_path, kind):
    d = str(tmp_path / kind)
    if kind == "bulk":
        systems.write_bulk(d, systems.CONFIGS["bulk_1000"], seed=20261203)
    elif kind == "brush":
        systems.write_brush(d, systems.brush_ensemble(1, seed=7)[0], seed=7)
    else:
        systems.write_muvt(d, systems.MuVTSpec(), seed=5)
    mol, sym, xyz, q, box = read(d)
    assert os.path.exists(os.path.join(d, "run.in"))
    assert abs(q.sum()) < 1e-9
    assert np.all(np.diff(mol) >= 0)  # beads grouped by molecule
    periodic = (True, True, kind != "brush")
    sites = np.array([s == "S" for s in sym])
    free = ~sites
    assert min_pair_distance(xyz[free], box, periodic) >= 0.8 - 1e-9
    for m in np.unique(mol[free]):
        b = xyz[mol == m]
        if len(b) > 1:
            np.testing.assert_allclose(np.linalg.norm(np.diff(b, axis=0), axis=1), 1.0,
                                       atol=1e-9)
    if kind == "brush":
        z = xyz[sites][:, 2]
        assert np.all((z == 0.0) | (z == box[2]))
        assert np.all((xyz[free][:, 2] > 0) & (xyz[free][:, 2] < box[2]))


def test_same_seed_same_files(tmp_path):
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    for d in (a, b):
        systems.write_bulk(d, systems.CONFIGS["bulk_1000"], seed=11)
    for f in ("run.in", "input_crd.dat", "input_top.dat"):
        assert open(os.path.join(a, f)).read() == open(os.path.join(b, f)).read()


def test_brush_sites_alternate_charge(tmp_path):
    spec = systems.BrushSpec(n_graft=2, chain_len=5, lxy=10.0, height=12.0, n_sites=6,
                             site_charge=0.5)
    d = str(tmp_path / "b")
    systems.write_brush(d, spec, seed=3)
    mol, sym, xyz, q, box = read(d)
    qs = q[np.array([s == "S" for s in sym])]
    np.testing.assert_array_equal(qs, np.tile([0.5, -0.5], 6))


def test_brush_ensemble_follows_the_batching_workload():
    """The 256 confined-brush replicas of the batching form: wall gap H in
    [30, 60], Lx = Ly = 32, 16-64 grafted chains of 20-80 beads, charge
    fraction in [0.1, 1], 64 surface sites per wall; the draws spread over
    the ranges and the sizes are uneven."""
    from plum_gb300 import systems
    specs = systems.brush_ensemble(256, 20261203)
    assert len(specs) == 256
    g = np.array([s.n_graft for s in specs])
    n = np.array([s.chain_len for s in specs])
    h = np.array([s.height for s in specs])
    f = np.array([s.charge_frac for s in specs])
    assert g.min() >= 16 and g.max() <= 64 and n.min() >= 20 and n.max() <= 80
    assert h.min() >= 30.0 and h.max() <= 60.0 and f.min() >= 0.1 and f.max() <= 1.0
    assert all(s.lxy == 32.0 and s.n_sites == 64 for s in specs)
    assert g.max() - g.min() > 40 and n.max() - n.min() > 50 and h.max() - h.min() > 25
    beads = g * n
    assert beads.max() > 5 * beads.min()  # uneven sizes
    assert systems.brush_ensemble(256, 20261203)[17] == specs[17]  # seeded
