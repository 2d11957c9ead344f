"""The CPU oracle against the reference: golden fixtures produced by the
reference's own code (tests/golden/make_golden.py), and, where the reference
checkout is present, live comparisons on fresh seeded inputs and on the
reference's shipped NVT examples."""
import os
import shutil
import tempfile

import numpy as np
import pytest

from _cases import CASES, de_moves, load, rel


@pytest.mark.parametrize("case", CASES)
def test_total_energy_matches_reference(built, case):
    d, g = load(case)
    o = built.Oracle(d, seed=int(g["run_seed"]))
    for a, b in zip(o.energies(), g["energies"]):
        assert rel(a, b) < 1e-12
    ew_o, ew_r = o.ewald_info(), g["ewald"]
    # real cutoff, k^2 cutoff, real cells, k cells, Ewald box, alpha, lB, volume
    np.testing.assert_array_equal(ew_o[[0, 2, 3, 4, 5, 6, 7]], ew_r[[0, 2, 3, 4, 5, 6, 7]])
    np.testing.assert_allclose(ew_o[8:14], ew_r[8:14], rtol=0, atol=0)
    assert ew_o[1] == ew_r[1]


@pytest.mark.parametrize("case", CASES)
def test_energy_difference_matches_reference(built, case):
    d, g = load(case)
    o = built.Oracle(d)
    for m, trial, moved, exp in de_moves(g):
        got = o.delta_energy(m, trial, moved)
        scale = max(1.0, abs(exp[1]), abs(exp[2]))
        assert rel(got[0], exp[0], scale) < 1e-10, (m, got, exp)
        assert rel(got[1], exp[1], scale) < 1e-10
        assert rel(got[2], exp[2], scale) < 1e-10


@pytest.mark.parametrize("case", CASES)
def test_replay_matches_reference(built, case):
    d, g = load(case)
    o = built.Oracle(d, seed=int(g["run_seed"]))
    n = len(g["run_type"])
    mt, ac, dr, et = o.run(n)
    np.testing.assert_array_equal(mt, g["run_type"])
    np.testing.assert_array_equal(ac, g["run_accept"])
    np.testing.assert_array_equal(dr, g["run_draws"])
    np.testing.assert_allclose(et, g["run_etot"], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(o.coords(), g["run_coords"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(o.observables()[[0, 4]], g["run_obs"][[0, 4]], rtol=1e-12)
    np.testing.assert_allclose(o.rhoz(), g["run_rhoz"], rtol=0, atol=1e-12)
    # running totals agree with a from-scratch recompute
    np.testing.assert_allclose(o.total_energy()[:4], g["run_recompute"], rtol=1e-10, atol=1e-9)


@pytest.mark.parametrize("case", CASES)
def test_mt19937_matches_reference_generator(built, case):
    d, g = load(case)
    np.testing.assert_array_equal(built.mt19937(int(g["run_seed"]), 4000), g["rng_words"])


def test_recorded_stream_equals_internal_generator(built):
    d, g = load("bulk_small")
    o1 = built.Oracle(d, seed=4242)
    o2 = built.Oracle(d)
    n = 300
    mt1, ac1, _, et1 = o1.run(n)
    used, mt2, ac2, et2 = o2.run_stream(n, built.mt19937(4242, 100000))
    assert used > 0
    np.testing.assert_array_equal(mt1, mt2)
    np.testing.assert_array_equal(ac1, ac2)
    np.testing.assert_array_equal(et1, et2)


def test_stream_exhaustion_is_reported(built):
    d, _ = load("bulk_small")
    o = built.Oracle(d)
    used, *_ = o.run_stream(50, built.mt19937(1, 20))
    assert used == -1


def test_malformed_runin_is_an_error_not_a_hang(built, tmp_path):
    d, _ = load("bulk_small")
    for f in ("input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    text = open(os.path.join(d, "run.in")).read()
    # drop the LJ table's "end" token: the reference would read forever at EOF
    cut = text.index("s3_end_flag")
    (tmp_path / "run.in").write_text(text[:cut])
    with pytest.raises(ValueError):
        built.Oracle(str(tmp_path))


def _ref_dir():
    from oracle import bindings as ob
    return ob.REF_DIR


REF_EXAMPLES = os.path.join(_ref_dir(), "examples")


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="reference checkout absent")
@pytest.mark.parametrize("example", ["bulk_nvt", "confined_nvt"])
def test_reference_examples_live(built, example, tmp_path):
    """The reference's shipped NVT examples, reference vs oracle, live."""
    if not built.have_ref():
        pytest.skip("reference harness not built")
    src = os.path.join(REF_EXAMPLES, example)
    for f in ("run.in", "input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    r = built.Ref(str(tmp_path), seed=5)
    o = built.Oracle(str(tmp_path), seed=5)
    np.testing.assert_allclose(o.energies(), r.energies(), rtol=1e-11, atol=1e-11)
    n = 150
    mt1, ac1, dr1, et1 = r.run(n)
    mt2, ac2, dr2, et2 = o.run(n)
    np.testing.assert_array_equal(mt1, mt2)
    np.testing.assert_array_equal(ac1, ac2)
    np.testing.assert_array_equal(dr1, dr2)
    np.testing.assert_allclose(et2, et1, rtol=1e-10, atol=1e-9)


@pytest.mark.skipif(not os.path.isdir(os.path.join(_ref_dir(), "src")),
                    reason="reference checkout absent")
def test_fresh_seeded_system_live(built, tmp_path):
    """A freshly generated system (not a committed fixture), reference vs oracle."""
    if not built.have_ref():
        pytest.skip("reference harness not built")
    from plum_gb300 import systems
    spec = systems.BulkSpec(n_chain=3, chain_len=12, n_ion=36, box=12.0,
                            move_prob=(0.2, 0.2, 0.2, 0.2, 0.2))
    systems.write_bulk(str(tmp_path), spec, seed=2027)
    r = built.Ref(str(tmp_path), seed=31)
    o = built.Oracle(str(tmp_path), seed=31)
    mt1, ac1, dr1, et1 = r.run(400)
    mt2, ac2, dr2, et2 = o.run(400)
    np.testing.assert_array_equal(ac1, ac2)
    np.testing.assert_array_equal(dr1, dr2)
    np.testing.assert_allclose(et2, et1, rtol=1e-10, atol=1e-9)
