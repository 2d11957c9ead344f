"""Host-side measurement helpers of bench.py: the pooled integrated
autocorrelation time, the paired 2-SE check and its labels, and the pooled
writer of the brush ensemble (CPU only)."""
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


def test_paired_check():
    """Same mean: the difference of paired means lies within 2 SE; a shift of
    10 SE is flagged."""
    rng = np.random.default_rng(1)
    start = rng.normal(size=64) * 5.0        # what each pair shares
    x = start + rng.normal(size=64)
    y = start + rng.normal(size=64)
    ok = bench.paired_check(x, y)
    assert ok["within_2_se"] and abs(ok["paired_difference"]) < 2 * ok["standard_error"]
    assert ok["standard_error"] < 0.3  # pairing removes the shared spread
    bad = bench.paired_check(x + 10 * ok["standard_error"], y)
    assert not bad["within_2_se"]


def test_paired_check_names_the_other_arm():
    x, y = [1.0, 2.0, 3.0], [1.1, 2.1, 2.9]
    assert "plain_fp64_mean" in bench.paired_check(x, y)
    r = bench.paired_check(x, y, other="plain_dynamics")
    assert "plain_dynamics_mean" in r and "plain_fp64_mean" not in r


def test_brush_ensemble_written_by_the_pool_equals_a_sequential_write(tmp_path, monkeypatch):
    """The process pool writes the same files as a replica written on its own
    (every replica has its own seed)."""
    import filecmp
    monkeypatch.setattr(bench.tempfile, "gettempdir", lambda: str(tmp_path / "pool"))
    os.makedirs(tmp_path / "pool")
    dirs = bench.make_brush_ensemble(3, seed=7)
    monkeypatch.setattr(bench.tempfile, "gettempdir", lambda: str(tmp_path / "one"))
    os.makedirs(tmp_path / "one")
    for i, d in enumerate(dirs):
        (one,) = bench.make_brush_ensemble(3, seed=7, only=i)
        for f in ("run.in", "input_crd.dat", "input_top.dat"):
            assert filecmp.cmp(os.path.join(d, f), os.path.join(one, f), shallow=False), (i, f)
