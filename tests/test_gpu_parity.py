"""Plain FP64 form on the GPU against the reference's golden fixtures and the
CPU oracle, through the C ABI (plum_gb300/_lib/libplumgpu.so).

Bars: energies and dE within 1e-10 relative (dE relative to the size of its
pair and Ewald parts); the recorded-stream replay must give the identical
move-type, accept and draw-count sequence."""
import numpy as np
import pytest

from _cases import CASES, de_moves, load, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.parametrize("case", CASES)
def test_total_energy(pg, case):
    d, g = load(case)
    s = pg.System(d)
    e = s.total_energy()
    for a, b in zip(e[:4], g["energies"]):
        assert rel(a, b) < 1e-10, (e, g["energies"])
    assert s.info.real_cutoff == g["ewald"][0]
    assert list(s.info.real_cell) == list(g["ewald"][2:5])
    assert list(s.info.k_cell) == list(g["ewald"][5:8])


@pytest.mark.parametrize("case", CASES)
def test_energy_difference(pg, case):
    d, g = load(case)
    s = pg.System(d)
    for m, trial, moved, exp in de_moves(g):
        got = s.energy_difference(m, trial, moved)
        s.finalize(False)
        scale = max(1.0, abs(exp[1]), abs(exp[2]))
        assert rel(got[0], exp[0], scale) < 1e-10, (case, m, got, exp)
        assert rel(got[1], exp[1], scale) < 1e-10
        assert rel(got[2], exp[2], scale) < 1e-10
    # rejected trials leave the running totals untouched
    np.testing.assert_allclose(s.energies(), g["energies"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_replay_recorded_stream(pg, case, built):
    d, g = load(case)
    s = pg.System(d)
    n = len(g["run_type"])
    stream = built.mt19937(int(g["run_seed"]), 400000)
    used, mt, ac, et = s.run_moves(stream, n)
    np.testing.assert_array_equal(mt, g["run_type"])
    np.testing.assert_array_equal(ac, g["run_accept"])
    assert used == int(g["run_draws"].sum())
    np.testing.assert_allclose(et, g["run_etot"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(s.positions(), g["run_coords"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(s.observables()[[0, 4]], g["run_obs"][[0, 4]], rtol=1e-10)
    np.testing.assert_allclose(s.rhoz(), g["run_rhoz"], rtol=1e-12, atol=1e-12)
    fresh = s.total_energy()[:4]
    np.testing.assert_allclose(fresh, g["run_recompute"], rtol=1e-10, atol=1e-9)


def test_accept_commits_and_reject_restores(pg):
    d, g = load("bulk_small")
    s = pg.System(d)
    e0 = s.energies().copy()
    x0 = s.positions().copy()
    m, trial, moved, exp = next(de_moves(g))
    de = s.energy_difference(m, trial, moved)
    s.finalize(True)
    e1 = s.energies()
    assert rel(e1.sum() - e0.sum(), de[0], max(1.0, abs(de[1]), abs(de[2]))) < 1e-10
    x1 = s.positions()
    start = g["de_start"]
    np.testing.assert_array_equal(x1[start[m]:start[m + 1]][moved == 1], trial[moved == 1])
    # a full recompute agrees with the incrementally updated totals
    np.testing.assert_allclose(s.total_energy()[:4], e1, rtol=1e-10, atol=1e-9)
    # and moving back gives -dE
    back = s.energy_difference(m, x0[start[m]:start[m + 1]], moved)
    s.finalize(False)
    assert rel(back[0], -de[0], max(1.0, abs(de[1]), abs(de[2]))) < 1e-10


def test_device_generator_matches_recorded_stream(pg, built):
    d, g = load("bulk_small")
    a = pg.System(d)
    b = pg.System(d)
    a.seed(99)
    a.run(250)
    b.run_moves(built.mt19937(99, 400000), 250, logs=False)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.energies(), b.energies())


def test_medium_system_long_replay_against_oracle(pg, built):
    d, g = load("bulk_medium")
    s = pg.System(d)
    o = built.Oracle(d)
    stream = built.mt19937(555, 2000000)
    n = 1500
    used, mt, ac, et = s.run_moves(stream, n)
    used_o, mt_o, ac_o, et_o = o.run_stream(n, stream)
    assert used == used_o
    np.testing.assert_array_equal(mt, mt_o)
    np.testing.assert_array_equal(ac, ac_o)
    np.testing.assert_allclose(et, et_o, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(s.positions(), o.coords(), rtol=0, atol=1e-8)


@pytest.mark.parametrize("chain_len,use_bond", [(200, True), (300, True), (300, False),
                                                (600, True)])
def test_long_chain_pivots_against_oracle(pg, built, tmp_path, chain_len, use_bond):
    """Pivots of long chains replay the oracle's draw sequence: the block's
    parallel scan of the beads' draws (up to 512 beads, with the bond-length
    draw of the bond potential and without it), its hand-back to thread 0's
    scan when the draws run past the staged window (300 beads with the bond
    draw need ~1,050 stream words), and the sequential pivot of chains over
    512 beads. High temperature (beta = 0.02) so that moves are accepted."""
    from plum_gb300 import systems
    d = str(tmp_path / "long")
    systems.write_bulk(d, systems.BulkSpec(n_chain=2, chain_len=chain_len, n_ion=60, box=30.0,
                                           move_size=0.15,
                                           move_prob=(0.1, 0.05, 0.55, 0.15, 0.15),
                                           use_bond=use_bond), seed=7, beta=0.02)
    s = pg.System(d)
    o = built.Oracle(d)
    stream = built.mt19937(77, 400000)
    n = 120
    used, mt, ac, et = s.run_moves(stream, n)
    used_o, mt_o, ac_o, et_o = o.run_stream(n, stream)
    assert (np.asarray(mt_o) == 2).sum() > 40
    assert used == used_o
    np.testing.assert_array_equal(mt, mt_o)
    np.testing.assert_array_equal(ac, ac_o)
    np.testing.assert_allclose(et, et_o, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(s.positions(), o.coords(), rtol=0, atol=1e-8)


@pytest.mark.parametrize("workload", ["bulk_1000_pinned", "bulk_1000"])
def test_from_scratch_totals_against_oracle(pg, built, tmp_path, workload):
    """The from-scratch FP64 totals of the 1,000-bead bulk system: with
    r_c = L/2 (the fixed-point pair kernel: one image, cubic box) and with the
    reference's automatic r_c = 28 > L/2 (image cells), both forms, against
    the oracle's at 1e-10."""
    from plum_gb300 import systems
    d = str(tmp_path / workload)
    systems.write_bulk(d, systems.CONFIGS[workload], seed=5)
    want = built.Oracle(d).energies()
    for form in (pg.FORM_FP64, pg.FORM_FP32):
        s = pg.System(d, form=form)
        got = s.total_energy()[:4]
        for a, b in zip(got, want):
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (workload, form, got, want)
        s.close()


def test_stream_exhaustion_reported(pg, built):
    d, _ = load("bulk_small")
    s = pg.System(d)
    with pytest.raises(pg.PlumError) as ei:
        s.run_moves(built.mt19937(3, 30), 50)
    assert ei.value.code == 6


def test_bad_input_is_an_error(pg, tmp_path):
    import shutil, os
    d, _ = load("bulk_small")
    for f in ("input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    text = open(os.path.join(d, "run.in")).read()
    (tmp_path / "run.in").write_text(text[:text.index("s3_end_flag")])
    with pytest.raises(pg.PlumError) as ei:
        pg.System(str(tmp_path))
    assert ei.value.code == 1


@pytest.mark.parametrize("case", ["bulk_small", "slab_wca", "bulk_1000"])
def test_chain_observables_match_the_definition(pg, case):
    """Per-chain Rg^2 (simulation.cc:406-434: (1/n^2) sum_{j<k} r_jk^2 on the
    unwrapped coordinates) and end-to-end^2 from the device against numpy on
    the same positions, and their chain average against plum_observables."""
    d, _ = load(case)
    s = pg.System(d)
    s.seed(3)
    s.run(300)
    pos = s.positions()
    ms = s.topology()[0]
    got = s.chain_observables()
    want = []
    for m in range(len(ms) - 1):
        x = pos[ms[m]:ms[m + 1]]
        n = len(x)
        if n < 2:
            continue
        dd = ((x[:, None, :] - x[None, :, :]) ** 2).sum(axis=2)
        want.append((dd[np.triu_indices(n, 1)].sum() / n ** 2, ((x[0] - x[-1]) ** 2).sum()))
    want = np.array(want)
    np.testing.assert_allclose(got[:, 0], want[:, 0], rtol=1e-12)
    np.testing.assert_allclose(got[:, 4], want[:, 1], rtol=1e-12)
    np.testing.assert_allclose(got[:, 0].mean(), s.observables()[0], rtol=1e-12)
