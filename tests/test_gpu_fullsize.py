"""Parity at the full size of the measured workload, bulk_20000_pinned
(20,000 beads: 100 chains of 100 charged beads and 10,000 counterions in a
periodic box of L = 80, r_c = L/2, |n| <= 12 per axis, 7,812 half-space k
vectors), with tolerances that do not grow with the size:

* the plain FP64 form's total energy (1e-9) and energy changes of trial
  moves of every kind (1e-8 of the larger energy component: a chain move
  sums 2 x 10^6 pair differences, in another order than the restatement's)
  against the FP64 CPU restatement on the same configuration;
* the precision form's energy changes against the plain form's on the same
  trial moves (2e-4 of max(1, |dE|, |dE_pair|, |dE_ewald|); over 10^4 moves
  of this workload the largest error measured was 4e-5 of max(1, |dE|));
* after 2,000 device steps, the plain form's running totals against a
  from-scratch recompute to 1e-9 (the incremental S(k) and pair updates lose
  nothing); the precision form's, which add FP32 energy changes until its
  periodic FP64 recompute, to 1e-4 of the total.
The restatement's total energy at this size takes about half a minute on
one host core.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORKLOAD = "bulk_20000_pinned"
SEED = 20261203  # the first replica of the measured batch


@pytest.fixture(scope="module")
def system_dir(tmp_path_factory):
    from plum_gb300 import systems
    d = str(tmp_path_factory.mktemp("full") / WORKLOAD)
    systems.write_bulk(d, systems.CONFIGS[WORKLOAD], seed=SEED)
    return d


@pytest.fixture(scope="module")
def oracle(built, system_dir):
    o = built.Oracle(system_dir, seed=1)
    yield o
    o.close()


def scale(d):
    return max(1.0, abs(d[1]), abs(d[2]))


def trial_moves(pos, mol_start, per_kind=2, seed=3):
    """Trial moves of each of the reference's five kinds (tests/_moves.py):
    per_kind ion translations and 4 x per_kind chain moves."""
    from _moves import kind_trials
    rng = np.random.default_rng(seed)
    sizes = np.diff(mol_start)
    return [(m, tr, mv) for _, m, tr, mv in kind_trials(pos, mol_start, sizes, rng,
                                                        per_kind=per_kind)]


def test_total_energy_matches_restatement(oracle, system_dir):
    import plum_gb300 as pg
    want = oracle.energies()  # the from-scratch totals of its set-up
    for form in (pg.FORM_FP64, pg.FORM_FP32):
        s = pg.System(system_dir, form=form)
        assert s.n_bead == 20000
        got = s.total_energy()[:4]
        for a, b in zip(got, want):
            assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (form, got, want)
        s.close()


def test_energy_changes_match_restatement(oracle, system_dir):
    import plum_gb300 as pg
    s64 = pg.System(system_dir, form=pg.FORM_FP64)
    s32 = pg.System(system_dir, form=pg.FORM_FP32)
    ms = s64.topology()[0]
    pos = s64.positions()
    np.testing.assert_array_equal(pos, oracle.coords())
    finite = 0
    for m, tr, mv in trial_moves(pos, ms):
        want = oracle.delta_energy(m, tr, mv)
        a = s64.energy_difference(m, tr, mv)
        s64.finalize(False)
        b = s32.energy_difference(m, tr, mv)
        s32.finalize(False)
        if want[0] >= 1e8:
            assert a[0] >= 1e8 and b[0] >= 1e8, (m, want, a, b)
            continue
        finite += 1
        assert abs(a[0] - want[0]) <= 1e-8 * scale(want), (m, a, want)
        assert abs(b[0] - a[0]) <= 2e-4 * max(scale(a), abs(a[0])), (m, b, a)
    assert finite >= 5
    s64.close()
    s32.close()


@pytest.mark.parametrize("form", [0, 1])
def test_running_totals_equal_recompute(system_dir, form):
    import plum_gb300 as pg
    s = pg.System(system_dir, form=form)
    s.seed(7)
    accepted = s.run(2000)
    assert accepted > 0
    run = s.energies().copy()
    fresh = s.total_energy()[:4]
    if form == pg.FORM_FP64:
        for a, b in zip(run, fresh):
            assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (run, fresh)
    else:
        assert abs(run.sum() - fresh.sum()) <= 1e-4 * max(1.0, abs(fresh.sum())), (run, fresh)
    s.close()
