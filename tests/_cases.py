"""Shared helpers for the golden-fixture tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(d for d in os.listdir(GOLDEN)
               if os.path.isfile(os.path.join(GOLDEN, d, "ref.npz")))


def load(case):
    return os.path.join(GOLDEN, case), dict(np.load(os.path.join(GOLDEN, case, "ref.npz")))


def de_moves(g):
    """Yields (mol, trial[n,3], moved[n], expected[3]) from a fixture."""
    start = g["de_start"]
    off = 0
    for k, m in enumerate(g["de_mol"]):
        n = start[m + 1] - start[m]
        yield int(m), g["de_trial"][off:off + n], g["de_moved"][off:off + n], g["de_out"][k]
        off += n


def rel(a, b, scale=1.0):
    return abs(a - b) / max(scale, abs(b))
