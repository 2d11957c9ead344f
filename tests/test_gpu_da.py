"""Delayed acceptance with the learned surrogate in the replica batch.

* Exactness: replicas equilibrated with the plain rule and continued with
  and without delayed acceptance sample the same mean energy and Rg^2
  (paired per replica, within 2.5 standard errors).
* The zero network (s = 0) passes every move at stage one, so stage two is
  the plain Metropolis rule: its counters give the plain method's chain
  acceptance on the same replicas.
* Gain: the trained network rejects most chain moves that the exact energy
  change would reject before that change is computed; the test states how
  many exact evaluations one accepted chain move costs with and without it.
"""
import os

import numpy as np
import pytest

from _cases import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.fixture(scope="module")
def trained(pg):
    from plum_gb300 import surrogate as S
    d, _ = load("bulk_small")
    desc, de, _ = S.collect(d, 40000, n_ctx=4, seed=300, moves_per_call=20000)
    sg, st = S.fit(desc, de, epochs=40, batch=1024, lr=1e-3, seed=3)
    return sg, st


def test_surrogate_learns_the_energy_change(trained):
    _, st = trained
    assert st["rmse_vs_fp64"] < 0.8 * st["exact_std"], st


def _lj_fluid(tmp):
    """100 beads (4 LJ chains of 10 + 60 free beads, cut at 2.5 sigma, no
    charges) in a box of 8 sigma: equilibrates within a few thousand steps."""
    from plum_gb300 import systems
    d = str(tmp / "lj_fluid")
    systems.write_bulk(d, systems.BulkSpec(n_chain=4, chain_len=10, n_ion=60, box=8.0,
                                           bead_charge=0.0, use_ewald=False), seed=41)
    return d


def _paired_stationarity(pg, d, sg, R=64, burn=20000, every=100, n=200):
    """Replicas equilibrated with the plain rule continue from the same
    configurations with and without delayed acceptance (independent seeds):
    per replica the mean energy and Rg^2 over the continuation differ by no
    more than 2.5 standard errors of the paired differences. A surrogate that
    broke detailed balance would shift the sampled distribution away from
    the equilibrium both runs start in. Returns the surrogate's counters."""
    a = pg.Batch([d] * R)
    a.seed(np.arange(100, 100 + R, dtype=np.uint32))
    a.run(burn)
    snap = [a.replica(r).positions() for r in range(R)]
    b = pg.Batch([d] * R)
    b.seed(np.arange(5000, 5000 + R, dtype=np.uint32))
    for r in range(R):
        b.replica(r).set_positions(snap[r])
    b.set_surrogate(sg)
    ra = [a.replica(r) for r in range(R)]
    rb = [b.replica(r) for r in range(R)]
    ea, eb, ga, gb = (np.zeros((n, R)) for _ in range(4))
    for k in range(n):
        a.run(every)
        b.run(every)
        for r in range(R):
            ea[k, r] = ra[r].energies().sum()
            eb[k, r] = rb[r].energies().sum()
            ga[k, r] = ra[r].observables()[0]
            gb[k, r] = rb[r].observables()[0]
    moves, passed, acc = b.da_stats()
    assert moves > 0 and 0 < passed < moves and acc > 0
    for name, x, y in (("energy", ea, eb), ("Rg2", ga, gb)):
        diff = y.mean(axis=0) - x.mean(axis=0)
        se = diff.std(ddof=1) / np.sqrt(R)
        assert abs(diff.mean()) <= 2.5 * se, (name, diff.mean(), se, x.mean(), y.mean())
    a.close()
    b.close()
    return moves, passed, acc


def test_delayed_acceptance_keeps_the_stationary_distribution(pg, tmp_path):
    """The paired test on an uncharged LJ fluid with a surrogate trained on it."""
    from plum_gb300 import surrogate as S
    d = _lj_fluid(tmp_path)
    desc, de, _ = S.collect(d, 30000, n_ctx=4, seed=900, moves_per_call=20000)
    sg, st = S.fit(desc, de, epochs=40, batch=1024, lr=1e-3, seed=4)
    _paired_stationarity(pg, d, sg)


def test_delayed_acceptance_keeps_the_stationary_distribution_charged(pg, trained):
    """The paired test on the charged bulk case (Ewald on: every stage-one
    rejection takes the serial step's own S(k) commit path), with the
    surrogate trained on it and no dead zone, so that stage one rejects
    often."""
    sg, _ = trained
    d, _ = load("bulk_small")
    moves, passed, acc = _paired_stationarity(pg, d, sg)
    assert moves - passed > 0.2 * moves, (moves, passed)


def test_delayed_acceptance_bookkeeping_matches_recompute_charged(pg, trained):
    """After 2,500 delayed-acceptance steps of 8 charged replicas, with the
    periodic recompute off so that every running sum spans the whole run,
    each replica's running totals and S(k) equal a from-scratch FP64
    recompute of its final configuration. Moves that stage one rejects skip
    the exact energy change, and the serial step then applies the S(k) change
    of the last accepted move itself (the delta kernel would otherwise do
    it); a missed or doubled commit would move S(k) by a whole bead's
    q e^{ik.r} (order 1) at most k. Tolerances: the totals within 1e-4 of
    their size (FP32 energy changes summed in FP64, as the precision form's
    other recompute checks), S(k) within 1e-3 per vector (FP32 phase
    changes summed in FP64: about 1e-5 after this run)."""
    sg, _ = trained
    d, _ = load("bulk_small")
    R = 8
    b = pg.Batch([d] * R)
    b.seed(np.arange(70, 70 + R, dtype=np.uint32))
    b.set_recompute(0)
    b.set_surrogate(sg)
    b.run(2500)
    moves, passed, acc = b.da_stats()
    assert moves - passed > 0.2 * moves and acc > 0, (moves, passed, acc)
    worst_e, worst_s = 0.0, 0.0
    for r in range(R):
        rep = b.replica(r)
        run = rep.energies().copy()
        sk_run, kn = rep.structure_factor()
        assert len(kn) > 0
        fresh = rep.total_energy()[:4]
        sk_fresh, _ = rep.structure_factor()
        worst_e = max(worst_e, abs(run.sum() - fresh.sum()) / max(1.0, abs(fresh.sum())))
        worst_s = max(worst_s, float(np.abs(sk_run - sk_fresh).max()))
        np.testing.assert_allclose(run, fresh, rtol=1e-4, atol=1e-3)
    assert worst_e < 1e-4, worst_e
    assert worst_s < 1e-3, worst_s
    b.close()


def test_gain_over_the_method_without_the_network(pg, trained):
    sg, st = trained
    d, _ = load("bulk_small")
    zero = pg.Surrogate(seed=1)
    zero.set_params(np.zeros(zero.n_params, np.float32))
    out = {}
    for name, net in (("plain", zero), ("surrogate", sg)):
        b = pg.Batch([d] * 16)
        b.seed(500)
        b.set_surrogate(net)
        b.run(2000)
        moves, passed, acc = b.da_stats()
        out[name] = dict(moves=moves, passed=passed, accepted=acc,
                         exact_per_accept=passed / max(acc, 1), chain_acc=acc / moves)
        b.close()
    p, s = out["plain"], out["surrogate"]
    assert p["passed"] == p["moves"]  # s = 0: stage one never rejects
    gain = p["exact_per_accept"] / s["exact_per_accept"]
    print("delayed acceptance", out, "exact evaluations saved per accepted move x%.2f" % gain,
          "rmse", st["rmse_vs_fp64"])
    assert gain > 1.5
    assert s["chain_acc"] > 0.5 * p["chain_acc"]


@pytest.mark.parametrize("workload,replicas,blocks,cap", [("bulk_1000", 8, 20, 0),
                                                          ("bulk_1000", 4, 12, 6),
                                                          ("bulk_20000_pinned", 2, 8, 0)])
def test_cell_list_descriptors_equal_all_pairs(pg, tmp_path, workload, replicas, blocks, cap):
    """The descriptor cell lists (rebuilt per batch of steps, entries moved on
    every accepted move) give the all-pairs kernel's integers: two batches
    from the same starts and seeds, one with and one without the lists,
    produce the same descriptors after every batch of steps and so the same
    stage-one decisions and trajectories. cap = 6 makes the list of beads
    that changed cell overflow: those replicas take the all-pairs kernel and
    the list grows until nothing overflows."""
    from plum_gb300 import surrogate as S
    from plum_gb300 import systems
    d = str(tmp_path / workload)
    systems.write_bulk(d, systems.CONFIGS[workload], seed=5)
    here = os.path.dirname(os.path.abspath(__file__))
    sg = S.load(os.path.join(here, "..", "plum_gb300", "data",
                             "surrogate_bulk_20000_pinned.npz"))
    out = []
    for on in (True, False):
        b = pg.Batch([d] * replicas)
        b.seed(np.arange(42, 42 + replicas, dtype=np.uint32))
        b.set_surrogate(sg)
        b.set_cells(on)
        if cap:
            b.set_cell_cap(cap)
        desc = []
        for _ in range(blocks):
            b.run(25)
            desc.append(b.descriptors())
        out.append((np.array(desc), [b.replica(r).positions() for r in range(replicas)],
                    b.da_stats()))
        if on and cap:
            # the lists grew past the cap
            with_lists, valid, most, per_cell = b.cell_stats()
            assert per_cell > cap and with_lists == replicas, (per_cell, with_lists)
        b.close()
    (da, pa, sa), (db, pb, sb) = out
    assert sa[0] > 0 and da.any()
    np.testing.assert_array_equal(da, db)
    for x, y in zip(pa, pb):
        np.testing.assert_array_equal(x, y)
    assert tuple(sa) == tuple(sb)
