"""Learned surrogate: the CPU checker (oracle/mlp_ref.py) against finite
differences here, and the GPU kernels (descriptor, tcgen05 forward and
backward, Adam, training, data collection) against the checker under -m gpu.

Tolerances: the GPU accumulates in FP32 where the checker uses FP64 with the
same bf16 rounding points, so a few bf16 roundings can land on the other
side; s agrees to 2e-3 of its scale on average and 2e-2 at worst, gradients
to 2% in norm with cosine similarity above 0.999. Descriptors are integer
sums (units of 2^-12); a pair whose FP32 distance lands in the next fine
bin (1/32 sigma) moves a bin by at most 0.08, so they agree to 0.2 per bin."""
import os

import numpy as np
import pytest

from oracle import mlp_ref as M

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def random_case(n, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAM)
    p[M.OFF_W1:M.OFF_B1] = rng.uniform(-0.2, 0.2, M.N_HID * M.N_IN)
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, M.N_HID)
    p[M.OFF_W2:M.OFF_B2] = rng.uniform(-0.15, 0.15, M.N_HID * M.N_HID)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.1, M.N_HID)
    p[M.OFF_W3:M.OFF_B3] = rng.uniform(-0.2, 0.2, M.N_HID)
    p[M.OFF_B3] = 0.3
    x = rng.gamma(2.0, 3.0, size=(n, M.N_IN))
    mu = x.mean(axis=0)
    isd = 1.0 / (x.std(axis=0) + 1e-3)
    t = rng.normal(0, 2.0, n)
    return p.astype(np.float32), mu.astype(np.float32), isd.astype(np.float32), x, t


# --------------------------------------------------------------- CPU checker
def test_checker_gradient_matches_finite_differences():
    p, mu, isd, x, t = random_case(40, 1)
    p = p.astype(np.float64)
    g = M.grad_exact(p, mu, isd, 1.7, x, t)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.integers(M.OFF_W1, M.OFF_B1, 6), rng.integers(M.OFF_B1, M.OFF_W2, 3),
                          rng.integers(M.OFF_W2, M.OFF_B2, 6), rng.integers(M.OFF_B2, M.OFF_W3, 3),
                          rng.integers(M.OFF_W3, M.OFF_B3, 3), [M.OFF_B3]])
    for i in idx:
        h = 1e-6
        a = p.copy()
        b = p.copy()
        a[i] += h
        b[i] -= h
        fd = (M.loss_exact(a, mu, isd, 1.7, x, t) - M.loss_exact(b, mu, isd, 1.7, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_checker_surrogate_is_antisymmetric():
    p, mu, isd, x, _ = random_case(30, 3)
    s = M.predict(p, mu, isd, 2.0, x)
    np.testing.assert_array_equal(M.predict(p, mu, isd, 2.0, M.swap(x)), -s)


def test_checker_rounded_gradient_is_close_to_exact():
    p, mu, isd, x, t = random_case(64, 4)
    g, _ = M.grad(p, mu, isd, 1.0, x, t)
    ge = M.grad_exact(p.astype(np.float64), mu, isd, 1.0, x, t)
    assert np.linalg.norm(g - ge) < 0.05 * np.linalg.norm(ge)


def test_checker_descriptor_swaps_for_the_reverse_move():
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, 10, size=(60, 3))
    aft = pos.copy()
    aft[10:20] += rng.normal(0, 0.5, size=(10, 3))
    types = (np.arange(60) >= 30).astype(int)
    d = M.descriptor(pos, aft, 10, 20, types, [10.0, 10.0, 10.0])
    r = M.descriptor(aft, pos, 10, 20, types, [10.0, 10.0, 10.0])
    np.testing.assert_array_equal(r, M.swap(d[None])[0])


# --------------------------------------------------------------- GPU kernels
def _close_s(a, b):
    scale = max(1.0, float(np.abs(b).max()))
    assert np.mean(np.abs(a - b)) <= 2e-3 * scale, (np.mean(np.abs(a - b)), scale)
    assert np.max(np.abs(a - b)) <= 2e-2 * scale, (np.max(np.abs(a - b)), scale)


@pytest.fixture(scope="module")
def pg():
    import plum_gb300
    plum_gb300.lib()
    return plum_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 64, 200, 1000])
def test_gpu_forward_matches_checker(pg, n):
    p, mu, isd, x, _ = random_case(n, 10 + n)
    sg = pg.Surrogate(seed=1)
    sg.set_params(p)
    sg.set_norm(mu, isd, 2.5)
    got = sg.predict(x)
    _close_s(got, M.predict(p, mu, isd, 2.5, x.astype(np.float32)))
    # exact antisymmetry on the GPU too
    np.testing.assert_array_equal(sg.predict(M.swap(x)), -got)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 200, 4096])
def test_gpu_gradient_matches_checker(pg, n):
    p, mu, isd, x, t = random_case(n, 20 + n)
    sg = pg.Surrogate(seed=1)
    sg.set_params(p)
    sg.set_norm(mu, isd, 1.5)
    g, loss = sg.grad(x, t)
    gc, lc = M.grad(p, mu, isd, 1.5, x.astype(np.float32), t)
    assert abs(loss - lc) <= 1e-3 * max(1.0, lc), (loss, lc)
    for name, lo, hi in (("W1", M.OFF_W1, M.OFF_B1), ("b1", M.OFF_B1, M.OFF_W2),
                         ("W2", M.OFF_W2, M.OFF_B2), ("b2", M.OFF_B2, M.OFF_W3),
                         ("w3", M.OFF_W3, M.OFF_B3)):
        a, b = g[lo:hi].astype(np.float64), gc[lo:hi]
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)
        assert cos > 0.999, (name, cos)
        assert np.linalg.norm(a - b) <= 0.02 * np.linalg.norm(b), name
    assert abs(g[M.OFF_B3]) < 1e-6  # b3 cancels in f(x) - f(swap x)


@pytest.mark.gpu
def test_gpu_adam_step_matches_checker(pg):
    p, mu, isd, x, t = random_case(128, 7)
    sg = pg.Surrogate(seed=1)
    sg.set_params(p)
    g = np.random.default_rng(8).normal(0, 0.01, M.N_PARAM).astype(np.float32)
    sg.adam_step(g, 1e-3)
    sg.adam_step(0.5 * g, 1e-3)
    q, m, v = M.adam(p, np.zeros_like(p), np.zeros_like(p), g, 1, 1e-3)
    q, m, v = M.adam(q, m, v, 0.5 * g, 2, 1e-3)
    np.testing.assert_allclose(sg.params(), q, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_gpu_training_fits_a_known_surrogate(pg):
    """Targets from a hidden network of the same form: Adam on the GPU must
    bring the loss far below the targets' variance."""
    import torch
    p0, mu, isd, x, _ = random_case(16384, 30)
    t = M.predict(p0, mu, isd, 1.0, x.astype(np.float32))
    sg = pg.Surrogate(seed=5)
    sg.set_norm(mu, isd, 1.0)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    losses = sg.train(xd, td, batch=1024, epochs=30, lr=2e-3, seed=1)
    assert losses[-1] < 0.1 * np.var(t), (losses[0], losses[-1], np.var(t))
    assert losses[-1] < losses[0]


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_gpu_descriptor_matches_checker(pg, form):
    d = os.path.join(GOLDEN, "bulk_small")
    s = pg.System(d, form=form)
    pos = s.positions()
    # bead symbols from the coordinate file: chains "P", ions "C"
    sym = [ln.split()[1] for ln in open(os.path.join(d, "input_crd.dat")).read().splitlines()[2:]
           if ln.strip()]
    typ = np.array([0 if c == "P" else 1 for c in sym])
    info = s.info
    rng = np.random.default_rng(40 + form)
    # molecule 0 is a chain of 20 beads (bulk_small: 4 x 20 + 80 ions)
    lo, hi = 0, 20
    for trial in range(4):
        k0 = int(rng.integers(0, 15))
        moved = np.zeros(20, np.int32)
        moved[k0:] = 1
        tr = pos[lo:hi] + moved[:, None] * rng.normal(0, 0.4, size=(20, 3))
        s.energy_difference(0, tr, moved)
        got = s.move_descriptor()
        s.finalize(False)
        after = pos.copy()
        after[lo:hi] = tr
        want = M.descriptor(pos, after, lo + k0, hi, typ, list(info.box), info.npbc)
        assert np.abs(got - want).max() <= 0.2, (np.abs(got - want).max(), form)
        assert np.abs(got - want).mean() <= 0.01
        assert want.sum() > 10


@pytest.mark.gpu
def test_gpu_data_collection_leaves_the_trajectory_unchanged(pg):
    d = os.path.join(GOLDEN, "bulk_small")
    a = pg.System(d)
    b = pg.System(d)
    a.seed(77)
    b.seed(77)
    desc, de = a.collect_surrogate_data(3000, 5000)
    b.run(3000)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.energies(), b.energies())
    n = desc.shape[0]
    # chain moves are 60% of the move mix (pivot, crankshaft, reptation)
    assert 0.5 * 3000 < n < 0.7 * 3000
    dh = desc.cpu().numpy()
    dd = de.cpu().numpy()
    assert (dh >= 0).all() and np.isfinite(dd).all()
    # an empty descriptor only for a crankshaft that moved no bead (dE = 0)
    empty = dh.sum(axis=1) == 0
    assert (dd[empty] == 0).all() and empty.mean() < 0.2
