"""The trial moves the energy-change checks probe the energy surface with
(tests/_moves.py kind_trials) have the shapes of the reference's move kinds
(molecule.cc:103-312): an ion step of exactly 3 move_size, a chain
translation of at most move_size / 2 per axis, a pivot whose bonds all come
out within r0 +- 10%, a crankshaft rotation that keeps its end beads and
every bond length, a reptation that keeps the old bonds and adds one of
r0 +- 10%."""
import numpy as np

from _moves import kind_trials


def _chain(n, rng):
    steps = rng.normal(size=(n - 1, 3))
    steps /= np.linalg.norm(steps, axis=1)[:, None]
    return np.vstack([[0, 0, 0], np.cumsum(steps, axis=0)]) + 5.0


def test_move_shapes():
    rng = np.random.default_rng(1)
    chains = [_chain(30, rng) for _ in range(3)]
    ions = rng.uniform(0, 10, size=(5, 3))
    pos = np.vstack(chains + [ions])
    sizes = np.array([30, 30, 30, 1, 1, 1, 1, 1])
    start = np.concatenate([[0], np.cumsum(sizes)])
    seen = set()
    for kind, m, tr, mv in kind_trials(pos, start, sizes, rng, move_size=0.5, per_kind=40):
        cur = pos[start[m]:start[m + 1]]
        seen.add(kind)
        assert tr.shape == cur.shape and mv.shape == (len(cur),) and mv.dtype == np.int32
        bonds = np.linalg.norm(np.diff(tr, axis=0), axis=1)
        if kind == 0:
            assert len(cur) == 1 and np.isclose(np.linalg.norm(tr[0] - cur[0]), 1.5)
        elif kind == 1:
            d = tr - cur
            assert np.allclose(d, d[0]) and (np.abs(d[0]) <= 0.25 + 1e-12).all()
        elif kind == 2:
            assert mv.all() and ((bonds > 0.9 - 1e-9) & (bonds < 1.1 + 1e-9)).all()
        elif kind == 3:
            f, l = np.flatnonzero(mv)[[0, -1]]
            f, l = f - 1, l + 1
            assert np.allclose(tr[:f + 1], cur[:f + 1]) and np.allclose(tr[l:], cur[l:])
            assert np.allclose(bonds, np.linalg.norm(np.diff(cur, axis=0), axis=1))
        else:
            old = np.linalg.norm(np.diff(cur, axis=0), axis=1)
            fwd = np.allclose(tr[:-1], cur[1:])
            assert fwd or np.allclose(tr[1:], cur[:-1])
            kept, new = (bonds[:-1], bonds[-1]) if fwd else (bonds[1:], bonds[0])
            assert np.allclose(kept, old[1:] if fwd else old[:-1])
            assert 0.9 - 1e-9 < new < 1.1 + 1e-9
    assert seen == {0, 1, 2, 3, 4}
