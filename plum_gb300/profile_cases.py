"""Small, self-contained cases of the surrogate kernels for a profiler.

    python -m plum_gb300.profile_cases da [workload] [replicas]
        trains a small surrogate on 6,000 collected moves of the workload
        (default bulk_20000_pinned), then runs a replica batch (default 16)
        with delayed acceptance; the third batch of 32 steps runs inside the
        NVTX range "da" (descriptor, smearing and tcgen05 inference launches),
        then the same without the surrogate inside "plain".
    python -m plum_gb300.profile_cases chosen [replicas]
        the measured form of the 20,000-particle workload: replicas
        (default 64) with the shipped surrogate weights (dead zone 12 k_BT),
        autotuned work items, two step chains; after 256 warm-up steps one
        batch of 32 steps runs inside the NVTX range "chosen".
    python -m plum_gb300.profile_cases train
        one epoch of surrogate training on 65,536 random descriptors in
        batches of 4,096 inside the NVTX range "train" (k_mlp<true>, the
        gradient reduction and Adam), then one inference pass inside "infer".

    python -m plum_gb300.profile_cases pressure [evaluations]
        the wall-force pressure of one confined brush replica of the batched
        workload with charged surface sites (64 per wall, +-0.5): after two
        warm-up evaluations, the given number (default 3) run inside the
        NVTX range "pressure" (k_slit_pairs, k_slit_recip, k_slit_sum), with
        their mean wall time printed.

All keep the device footprint under 1 GB so a full-set capture of one to
three launches ends within a minute or two.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np


def _workload(name, seed):
    from . import systems
    d = os.path.join(tempfile.gettempdir(), "plum_prof_%s_%d" % (name, seed))
    if not os.path.exists(os.path.join(d, "run.in")):
        systems.write_bulk(d, systems.CONFIGS[name], seed=seed)
    return d


def delayed_acceptance(name="bulk_20000_pinned", replicas=16):
    import torch
    import plum_gb300 as pg
    from . import surrogate as S
    d = _workload(name, 20261203)
    desc, de, _ = S.collect(d, 6000, n_ctx=1, moves_per_call=10000)
    sg, _ = S.fit(desc, de, epochs=5, batch=1024)
    b = pg.Batch([_workload(name, 20261203 + i) for i in range(replicas)])
    b.seed(77)
    for label, net in (("da", sg), ("plain", None)):
        b.set_surrogate(net)
        for i in range(3):
            if i == 2:
                torch.cuda.nvtx.range_push(label)
            b.run(32)
            if i == 2:
                torch.cuda.nvtx.range_pop()
        ms, k = b.last_timing()
        print(label, "ms", ms, "steps", k, "da_stats", b.da_stats() if net else None, flush=True)
    b.close()


def chosen(replicas=64):
    import torch
    import plum_gb300 as pg
    from . import surrogate as S
    here = os.path.dirname(os.path.abspath(__file__))
    sg = S.load(os.path.join(here, "data", "surrogate_bulk_20000_pinned.npz"))
    sg.set_margin(12.0)
    b = pg.Batch([_workload("bulk_20000_pinned", 20261203 + r) for r in range(replicas)])
    b.seed(77)
    b.set_surrogate(sg)
    tune = b.autotune(16)
    b.set_groups(2)
    b.run(256)
    torch.cuda.nvtx.range_push("chosen")
    b.run(32)
    torch.cuda.nvtx.range_pop()
    ms, k = b.last_timing()
    print("chosen", replicas, "replicas, tune", tune, "ms per 32 steps", ms, "kernels", k,
          flush=True)
    b.close()


def training(n=65536, batch=4096):
    import torch
    import plum_gb300 as pg
    rng = np.random.default_rng(0)
    x = rng.gamma(2.0, 3.0, size=(n, 96)).astype(np.float32)
    t = rng.normal(0.0, 3.0, n).astype(np.float32)
    sg = pg.Surrogate(seed=1)
    sg.set_norm(x.mean(0), 1.0 / (x.std(0) + 1e-3), 3.0)
    xd = torch.tensor(x, device="cuda")
    td = torch.tensor(t, device="cuda")
    torch.cuda.nvtx.range_push("train")
    sg.train(xd, td, batch=batch, epochs=1, lr=1e-3)
    torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_push("infer")
    out = sg.predict_device(xd)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print("train ok, mean |s| %.4f" % float(out.abs().mean()), flush=True)


def pressure(evaluations=3):
    import time
    import torch
    import plum_gb300 as pg
    from . import systems
    spec = systems.brush_ensemble(1, seed=20261203)[0]
    spec.site_charge = 0.5
    d = os.path.join(tempfile.gettempdir(), "plum_prof_pressure")
    if not os.path.exists(os.path.join(d, "run.in")):
        systems.write_brush(d, spec, seed=20261203)
    s = pg.System(d)
    for _ in range(2):
        s.pressure_slit()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("pressure")
    t0 = time.perf_counter()
    for _ in range(evaluations):
        out = s.pressure_slit()
    dt = (time.perf_counter() - t0) / max(1, evaluations)
    torch.cuda.nvtx.range_pop()
    print("pressure ok: beads %d, k vectors %d, %.3f ms per evaluation, sums %s"
          % (s.n_bead, s.info.n_kvec, 1e3 * dt, out), flush=True)
    s.close()


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    what = argv[0] if argv else "da"
    if what == "da":
        delayed_acceptance(argv[1] if len(argv) > 1 else "bulk_20000_pinned",
                           int(argv[2]) if len(argv) > 2 else 16)
    elif what == "chosen":
        chosen(int(argv[1]) if len(argv) > 1 else 64)
    elif what == "train":
        training()
    elif what == "pressure":
        pressure(int(argv[1]) if len(argv) > 1 else 3)
    else:
        raise SystemExit("usage: python -m plum_gb300.profile_cases "
                         "{da [workload] [replicas] | chosen [replicas] | train | "
                         "pressure [evaluations]}")


if __name__ == "__main__":
    main()
