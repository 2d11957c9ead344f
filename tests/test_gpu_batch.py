"""Replica batches (precision form): every replica of one launch must behave
as the same system run alone -- on the reference's recorded stream each
replica reproduces its golden trajectory until a near tie."""
import numpy as np
import pytest

from _cases import CASES, load, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.parametrize("tune", [None, (2048, 256, 304, 2), (16384, 64, 1216, 3),
                                  (4096, 128, 608, 4), (4096, 1024, 608, 4)])
def test_uneven_replicas_replay_their_references(pg, tune):
    """Also with other work-item sizes than the defaults (what the autotuner
    may pick): the items only change the order of FP32 partial sums."""
    dirs, gs = [], []
    for c in CASES:
        d, g = load(c)
        dirs.append(d)
        gs.append(g)
    b = pg.Batch(dirs)
    if tune:
        b.set_tune(*tune)
    b.seed(np.array([int(g["run_seed"]) for g in gs], np.uint32))
    n = 150
    b.run(n)
    for r, g in enumerate(gs):
        rep = b.replica(r)
        e = rep.energies().sum()
        ref = g["run_etot"][n - 1]
        assert rel(e, ref, max(1.0, abs(ref))) < 1e-4, (CASES[r], e, ref)
        # the running totals stay consistent with an FP64 recompute (not with
        # the dipole correction on: there the reference's running Ewald total
        # carries the dipole term of the configuration before the last
        # accepted move)
        if not g["ewald"][14]:
            fresh = rep.total_energy()[:4].sum()
            assert rel(e, fresh, max(1.0, abs(fresh))) < 1e-4


@pytest.mark.parametrize("table", [True, False])
def test_real_space_term_table_and_fit_replay(pg, table):
    """Both real-space terms of the batched kernel (the h(u) table and the
    FP32 erfc fit) replay the reference's bulk fixtures to 1e-4 after 150
    steps."""
    cases = [c for c in CASES if not load(c)[1]["ewald"][14]]
    dirs, gs = zip(*[load(c) for c in cases])
    b = pg.Batch(list(dirs))
    b.set_real_term(table)
    assert b.real_term() == int(table)
    b.seed(np.array([int(g["run_seed"]) for g in gs], np.uint32))
    b.run(150)
    for r, g in enumerate(gs):
        e = b.replica(r).energies().sum()
        ref = g["run_etot"][149]
        assert rel(e, ref, max(1.0, abs(ref))) < 1e-4, (cases[r], table, e, ref)


def test_replicas_match_single_system_runs(pg):
    d, g = load("bulk_medium")
    b = pg.Batch([d] * 4)
    b.seed(np.array([11, 12, 13, 14], np.uint32))
    b.run(300)
    for r in range(4):
        s = pg.System(d, form=pg.FORM_FP32)
        s.seed(11 + r)
        s.run(300)
        np.testing.assert_allclose(b.replica(r).energies(), s.energies(), rtol=2e-4, atol=2e-3)


def test_batch_runs_are_repeatable(pg):
    d, _ = load("slab_lj")
    a = pg.Batch([d] * 3)
    c = pg.Batch([d] * 3)
    a.seed(5)
    c.seed(5)
    a.run(200)
    c.run(200)
    for r in range(3):
        np.testing.assert_array_equal(a.replica(r).positions(), c.replica(r).positions())


def test_autotune_picks_a_candidate_and_keeps_running(pg):
    d, _ = load("bulk_medium")
    b = pg.Batch([d] * 8)
    b.seed(3)
    ip, kt, grid, mb = b.autotune(4)
    assert ip in (4096, 8192, 16384, 32768) and kt in (128, 256, 512, 1024) and grid > 0
    assert mb in (2, 3, 4) and b.real_term() in (0, 1)
    assert b.run(100) > 0


def test_two_step_chains_give_the_same_trajectories(pg):
    """Replicas split in two graph branches (plum_batch_set_groups) do the
    same arithmetic: bit-identical positions and energies."""
    d, _ = load("bulk_medium")
    out = []
    for g in (1, 2):
        b = pg.Batch([d] * 6)
        b.seed(np.arange(30, 36, dtype=np.uint32))
        b.set_groups(g)
        b.run(300)
        out.append([(b.replica(r).positions(), b.replica(r).energies()) for r in range(6)])
        b.close()
    for (pa, ea), (pb, eb) in zip(*out):
        np.testing.assert_array_equal(pa, pb)
        np.testing.assert_array_equal(ea, eb)


def test_batch_recompute_resets_drift_past_1e4_steps(pg):
    """The batch's full FP64 recompute (every 10^4 moves per replica, phases
    staggered over the replicas) on a charged case: after 12,000 steps every
    replica has been recomputed at least once, the drift it found is finite,
    non-zero (FP32 energy changes) and small against the total, the
    recomputes ran inside the timed batch runs, and the running totals still
    equal a from-scratch recompute to the precision form's 1e-4."""
    d, _ = load("bulk_medium")
    R = 4
    b = pg.Batch([d] * R)
    b.seed(np.arange(31, 31 + R, dtype=np.uint32))
    n_rc, ms = 0, 0.0
    for _ in range(12):
        b.run(1000)
        dr, n, t = b.drift()
        n_rc += n
        ms += t
    assert n_rc >= R and ms > 0.0, (n_rc, ms)
    assert (dr[:, 5] >= 1).all(), dr[:, 5]
    for r in range(R):
        rep = b.replica(r)
        e = rep.energies().copy()
        assert np.isfinite(dr[r]).all()
        assert 0.0 < dr[r, 4] < 1e-3 * max(1.0, abs(e.sum())), (dr[r], e)
        fresh = rep.total_energy()[:4]
        assert rel(e.sum(), fresh.sum(), max(1.0, abs(fresh.sum()))) < 1e-4
    b.close()


def test_batch_recompute_off_and_cadence(pg):
    """set_recompute(0) switches the recompute off; a cadence of 64 moves
    recomputes every replica about once per 64 steps."""
    d, _ = load("bulk_small")
    b = pg.Batch([d] * 3)
    b.seed(9)
    b.set_recompute(0)
    b.run(640)
    dr, n, _ = b.drift()
    assert n == 0 and (dr[:, 5] == 0).all()
    b.set_recompute(64)
    b.run(640)
    dr, n, _ = b.drift()
    assert 27 <= n <= 33, n
    b.close()
