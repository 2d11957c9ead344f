"""Accuracy of the precision (FP32) form against the plain FP64 form on
identical trial moves: the energy-change error and the fraction of
Metropolis decisions that would flip.

Trial moves follow the reference's move kinds (Molecule::BeadTranslate,
COMTranslate, Crankshaft, RandomReptation, Pivot; molecule.cc:103-312) in
shape and size, drawn from numpy (they are probes of the energy surface, not
a Markov chain): an ion translated by 3 move_size along a random direction;
a chain translated by up to move_size / 2 per axis; a sub-chain rotated about
the axis through its end beads by move_size (2 pi u - pi); a reptation step
(every bead takes its neighbour's place, the new end one bond away); a
pivot (the beads past a random bead rotated rigidly about it by a random
angle of up to move_size pi).

For uniform u, the Metropolis decisions u < exp(-beta dE32) and
u < exp(-beta dE64) differ with probability
|min(1, exp(-beta dE32)) - min(1, exp(-beta dE64))|; its mean over the trial
moves is the flip fraction.
"""
from __future__ import annotations

import math

import numpy as np


def _rot(axis, ang):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    c, s = math.cos(ang), math.sin(ang)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + s * K + (1 - c) * (K @ K)


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def propose(pos, mol_start, rng, move_size=0.5, bond=1.0):
    """(molecule, trial [n][3], moved [n] int32) for a random molecule."""
    nmol = len(mol_start) - 1
    m = int(rng.integers(nmol))
    b0, b1 = int(mol_start[m]), int(mol_start[m + 1])
    cur = pos[b0:b1].copy()
    n = b1 - b0
    moved = np.ones(n, np.int32)
    if n == 1:
        return m, cur + 3 * move_size * _unit(rng), moved
    kind = int(rng.integers(4))
    if kind == 0:  # COM translation
        v = 0.5 * move_size * rng.random(3) * np.where(rng.random(3) < 0.5, -1, 1)
        return m, cur + v, moved
    if kind == 1 and n >= 3:  # crankshaft
        f = int(rng.integers(0, n - 2))
        l = f + 2 + int(rng.integers(0, n - f - 2))
        R = _rot(cur[l] - cur[f], move_size * (2 * math.pi * rng.random() - math.pi))
        tr = cur.copy()
        tr[f + 1:l] = (cur[f + 1:l] - cur[f]) @ R.T + cur[f]
        moved[:] = 0
        moved[f + 1:l] = 1
        return m, tr, moved
    if kind == 2:  # reptation
        tr = cur.copy()
        if rng.random() < 0.5:
            tr[:-1] = cur[1:]
            tr[-1] = cur[-1] + bond * _unit(rng)
        else:
            tr[1:] = cur[:-1]
            tr[0] = cur[0] + bond * _unit(rng)
        return m, tr, moved
    # pivot
    p = int(rng.integers(n))
    R = _rot(_unit(rng), move_size * math.pi * (2 * rng.random() - 1))
    tr = cur.copy()
    if rng.random() < 0.5:
        tr[p + 1:] = (cur[p + 1:] - cur[p]) @ R.T + cur[p]
        moved[:p + 1] = 0
    else:
        tr[:p] = (cur[:p] - cur[p]) @ R.T + cur[p]
        moved[p:] = 0
    if moved.sum() == 0:
        moved[:] = 1
        tr = cur + 0.1 * _unit(rng)
    return m, tr, moved


def compare(s64, s32, mol_start, n=200, seed=0, beta=1.0, move_size=0.5):
    """FP32 vs FP64 energy changes of n trial moves on s64's configuration
    (s32 is set to it first). Returns a dict of error and flip statistics."""
    pos = s64.positions()
    s32.set_positions(pos)
    rng = np.random.default_rng(seed)
    d64, d32 = [], []
    for _ in range(n):
        m, tr, mv = propose(pos, mol_start, rng, move_size=move_size)
        a = s64.energy_difference(m, tr, mv)
        s64.finalize(False)
        b = s32.energy_difference(m, tr, mv)
        s32.finalize(False)
        d64.append(a[0])
        d32.append(b[0])
    d64, d32 = np.array(d64), np.array(d32)
    live = np.abs(d64) < 1e7  # overlaps (1e8) are rejected by both forms alike
    err = (d32 - d64)[live]
    p64 = np.minimum(1.0, np.exp(-beta * np.clip(d64, -700, 700)))
    p32 = np.minimum(1.0, np.exp(-beta * np.clip(d32, -700, 700)))
    both_big = (d64 >= 1e8) == (d32 >= 1e8)
    return {"n_moves": int(n), "n_finite": int(live.sum()),
            "de_abs_err_rms": float(np.sqrt(np.mean(err ** 2))) if live.any() else None,
            "de_abs_err_max": float(np.abs(err).max()) if live.any() else None,
            "de_rel_err_max": float((np.abs(err) / np.maximum(1.0, np.abs(d64[live]))).max())
            if live.any() else None,
            "overlap_agreement": float(both_big.mean()),
            "flip_fraction": float(np.mean(np.abs(p32 - p64)))}
