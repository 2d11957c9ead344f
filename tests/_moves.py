"""Trial moves of the reference's five move kinds for the energy-change
checks (test helper): built from current coordinates with numpy draws, in
the shapes and sizes of Molecule::BeadTranslate, COMTranslate, Pivot,
Crankshaft and RandomReptation (molecule.cc:103-312). They are probes of the
energy surface, not a Markov chain; the chain's own proposals are compared
through the recorded-stream replays."""
import numpy as np


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def kind_trials(coords, start, sizes, rng, move_size=1.0, bond=1.0, per_kind=5, first_mol=0):
    """Trial configurations of each of the reference's move kinds
    (molecule.cc:103-312), built from the current coordinates with numpy
    draws: ion translation by exactly 3 move_size, chain COM translation
    (per axis up to 0.5 move_size), pivot (each bead outward of the pivot
    perturbed by up to move_size and re-projected to a bond of r0 +- 10%,
    the rest of that side carried along), crankshaft (beads strictly between
    first and last rotated about the first-last axis) and reptation (shift by
    one bead, new end one bond from the old end). Yields (kind, mol, trial,
    moved) with kind 0..4 in the reference's order [bead, COM, pivot, crank,
    rept]."""
    chains = [m for m in range(first_mol, len(sizes)) if sizes[m] > 1]
    ions = [m for m in range(first_mol, len(sizes)) if sizes[m] == 1]
    for kind in range(5):
        for _ in range(per_kind):
            if kind == 0:
                m = int(ions[rng.integers(len(ions))])
            else:
                m = int(chains[rng.integers(len(chains))])
            cur = coords[start[m]:start[m + 1]].copy()
            n = len(cur)
            moved = np.ones(n, np.int32)
            t = cur.copy()
            if kind == 0:
                t[0] = cur[0] + 3.0 * move_size * _unit(rng)
            elif kind == 1:
                t = cur + 0.5 * move_size * rng.uniform(-1.0, 1.0, size=3)
            elif kind == 2:
                p = int(rng.integers(n))
                size = move_size * rng.uniform()
                for rng_dir in (range(p + 1, n), range(p - 1, -1, -1)):
                    for i in rng_dir:
                        j = i - 1 if rng_dir.step == 1 else i + 1
                        x = t[i] + size * _unit(rng)
                        d = x - t[j]
                        b = bond + (bond / 5.0) * (rng.uniform() - 0.5)
                        c = t[j] + d * (b / np.linalg.norm(d))
                        sl = slice(i, n) if rng_dir.step == 1 else slice(0, i + 1)
                        t[sl] += c - t[i]
            elif kind == 3:
                first = int(rng.integers(0, n - 2))
                last = min(n - 1, first + 2 + int(rng.integers(0, n - first - 2)))
                axis = cur[last] - cur[first]
                axis /= np.linalg.norm(axis)
                ang = move_size * (rng.uniform() * 2 * np.pi - np.pi)
                K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]],
                              [-axis[1], axis[0], 0]])
                Rm = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * (K @ K)
                moved[:] = 0
                moved[first + 1:last] = 1
                t[first + 1:last] = (cur[first + 1:last] - cur[first]) @ Rm.T + cur[first]
            else:
                b = bond + (bond / 5.0) * (rng.uniform() - 0.5)
                if rng.integers(2):
                    t[:-1] = cur[1:]
                    t[-1] = cur[-1] + b * _unit(rng)
                else:
                    t[1:] = cur[:-1]
                    t[0] = cur[0] + b * _unit(rng)
            yield kind, m, t, moved
