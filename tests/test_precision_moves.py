"""The trial moves the precision comparisons probe the energy surface with
(plum_gb300.precision.propose): shapes of the reference's move kinds
(molecule.cc:103-312) -- an ion step of exactly 3 move_size, a rigid chain
translation of at most move_size / 2 per axis, a crankshaft rotation that
keeps its end beads and every bond length, a reptation that keeps bond
lengths, a pivot that keeps every distance on the rotated side."""
import numpy as np

from plum_gb300.precision import propose


def _chain(n, rng):
    steps = rng.normal(size=(n - 1, 3))
    steps /= np.linalg.norm(steps, axis=1)[:, None]
    return np.vstack([[0, 0, 0], np.cumsum(steps, axis=0)]) + 5.0


def test_move_shapes():
    rng = np.random.default_rng(1)
    chain = _chain(30, rng)
    ions = rng.uniform(0, 10, size=(5, 3))
    pos = np.vstack([chain, ions])
    mol_start = np.array([0, 30, 31, 32, 33, 34, 35])
    seen = set()
    for _ in range(400):
        m, tr, mv = propose(pos, mol_start, rng, move_size=0.5)
        cur = pos[mol_start[m]:mol_start[m + 1]]
        assert tr.shape == cur.shape and mv.shape == (len(cur),) and mv.dtype == np.int32
        if len(cur) == 1:
            assert np.isclose(np.linalg.norm(tr[0] - cur[0]), 1.5)
            seen.add("ion")
            continue
        d = tr - cur
        bonds = np.linalg.norm(np.diff(tr, axis=0), axis=1)
        if np.allclose(d, d[0]) and mv.all():
            if np.linalg.norm(d[0]) < 0.2 and np.allclose(np.abs(d[0]), 0.1):
                continue  # the fallback nudge of a pivot that moved nothing
            assert np.all(np.abs(d[0]) <= 0.25 + 1e-12)
            seen.add("com")
        elif not mv.all():
            # crankshaft or pivot: unmoved beads keep their places, bonds keep length
            np.testing.assert_allclose(tr[mv == 0], cur[mv == 0], atol=1e-12)
            np.testing.assert_allclose(bonds, 1.0, atol=1e-9)
            seen.add("partial")
        else:
            # reptation: bond lengths preserved, one end re-grown at the bond length
            np.testing.assert_allclose(bonds, 1.0, atol=1e-9)
            assert np.allclose(tr[:-1], cur[1:]) or np.allclose(tr[1:], cur[:-1])
            seen.add("reptation")
    assert seen == {"ion", "com", "partial", "reptation"}
