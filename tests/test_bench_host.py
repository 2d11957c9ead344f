"""Host-side measurement helpers of bench.py: the pooled integrated
autocorrelation time and the per-chain Rg^2 (CPU only)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_pooled_tau_of_ar1_series():
    """AR(1) with coefficient phi has tau_int = (1 + phi) / (2 (1 - phi))."""
    rng = np.random.default_rng(0)
    phi, T, C = 0.9, 3000, 400
    x = np.zeros((T, C))
    e = rng.normal(size=(T, C))
    for t in range(1, T):
        x[t] = phi * x[t - 1] + e[t]
    tau, how = bench.tau_pooled(x[200:])
    want = (1 + phi) / (2 * (1 - phi))
    assert how == "sokal" and abs(tau - want) < 0.1 * want, (tau, want)


def test_chain_rg2_matches_the_reference_definition():
    rng = np.random.default_rng(1)
    pos = rng.normal(size=(35, 3)) * 3
    mol_start = np.array([0, 10, 20, 21, 22, 35])  # chains of 10, 10, 13 and two ions
    got = bench.chain_rg2(pos, mol_start)
    want = []
    for a, b in ((0, 10), (10, 20), (22, 35)):
        x = pos[a:b]
        n = len(x)
        d = ((x[:, None, :] - x[None, :, :]) ** 2).sum(axis=2)
        want.append(d[np.triu_indices(n, 1)].sum() / n ** 2)
    np.testing.assert_allclose(np.sort(got), np.sort(want), rtol=1e-12)
