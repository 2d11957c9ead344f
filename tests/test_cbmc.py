"""Configurational-bias trial-site energies (ForceField::BeadsEnergy,
cbmc.cc:5-151) against the reference's own values: the CPU oracle's
restatement here, the GPU's batched trial kernel under -m gpu."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CBMC = ["muvt_neutral", "muvt_charged"]


def rows(case):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "cbmc.npz")))
    off = 0
    for k in range(len(g["u"])):
        cl = int(g["cl"][k])
        chain = g["chain"][off:off + cl]
        ci = g["chain_ci"][off:off + cl]
        off += cl
        yield d, bool(g["charged"]), int(g["delete_id"][k]), g["b1"][k], g["b2"][k], chain, ci, g["u"][k]


def close(a, b):
    if b >= 1e8:
        return a >= 1e8
    return abs(a - b) <= 1e-10 * max(1.0, abs(b))


@pytest.mark.parametrize("case", CBMC)
def test_oracle_beads_energy_matches_reference(built, case):
    o = None
    for d, charged, did, b1, b2, chain, ci, u in rows(case):
        o = o or built.Oracle(d)
        got = o.beads_energy(b1, b2 if charged else None, chain if len(chain) else None,
                             ci if (charged and len(chain)) else None, did)
        assert close(got, u), (case, did, len(chain), got, u)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CBMC)
def test_gpu_trial_energies_match_reference(case):
    import plum_gb300 as pg
    s = None
    for d, charged, did, b1, b2, chain, ci, u in rows(case):
        s = s or pg.System(d)
        got = s.cbmc_trials(b1[None], b2[None] if charged else None,
                            chain if len(chain) else None, ci if (charged and len(chain)) else None,
                            did)
        assert close(got[0], u), (case, did, len(chain), got[0], u)


@pytest.mark.gpu
def test_gpu_trials_batched_equal_one_by_one():
    import plum_gb300 as pg
    d = os.path.join(GOLDEN, "muvt_charged")
    s = pg.System(d)
    rng = np.random.default_rng(3)
    b1 = rng.uniform(0, 14, size=(32, 3))
    b2 = rng.uniform(0, 14, size=(32, 3))
    chain = np.array([[3.0, 3.0, 3.0], [3.9, 3.2, 3.1]])
    ci = rng.uniform(0, 14, size=(2, 3))
    all_u = s.cbmc_trials(b1, b2, chain, ci, -1)
    for t in range(0, 32, 7):
        one = s.cbmc_trials(b1[t:t + 1], b2[t:t + 1], chain, ci, -1)
        assert all_u[t] == one[0]
