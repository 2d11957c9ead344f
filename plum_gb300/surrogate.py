"""Training data, training and storage of the learned energy-change surrogate.

Data come from the plain step loop (System.collect_surrogate_data: the exact
FP64 energy change of every pivot, crankshaft and reptation move of seeded
trajectories, with its descriptor); training runs the tensor-core forward/
backward and Adam kernels (Surrogate.train). Several contexts collect at once,
one host thread each: their step loops are latency-bound, so they share the
GPU well.

    python -m plum_gb300.surrogate --workload bulk_20000 --samples 2000000 \\
        --out plum_gb300/data/surrogate_bulk_20000.npz
"""
from __future__ import annotations

import argparse
import os
import tempfile
import threading
import time

import numpy as np

from . import FORM_FP64, Surrogate, System, systems

# Targets are clipped: any change above this is rejected in practice, and
# overlaps (up to 1e8) would otherwise dominate the loss.
CLIP = 20.0


def normalisation(desc):
    """Per-feature mean and inverse spread, the same for the before and after
    channels (statistics over the descriptors and their swaps)."""
    import torch
    h = desc.shape[1] // 2
    both = torch.cat([desc[:, :h], desc[:, h:]], dim=0).double()
    mu = both.mean(dim=0)
    sd = both.std(dim=0)
    mu = torch.cat([mu, mu]).float().cpu().numpy()
    isd = (1.0 / torch.clamp(torch.cat([sd, sd]), min=0.05)).float().cpu().numpy()
    return mu, isd


def targets(de, clip=CLIP):
    """Clipped float32 targets and the output scale (their spread)."""
    import torch
    t = torch.clamp(de, -clip, clip).float()
    return t, float(max(t.std().item(), 1e-3))


def collect(dirpath, samples, n_ctx=8, seed=1000, moves_per_call=20000, form=FORM_FP64,
            runin="run.in"):
    """About `samples` (descriptor, exact dE) pairs from n_ctx independently
    seeded plain-loop contexts, each on its own host thread. Returns CUDA
    tensors desc [k][96], de [k] and the wall time. The output buffers are
    allocated up front, so the threads make no CUDA calls of their own
    besides the library's (whose step loops capture CUDA graphs)."""
    import torch
    per = (samples + n_ctx - 1) // n_ctx
    cap = per + moves_per_call
    bufs = [(torch.empty((cap, 96), dtype=torch.float32, device="cuda"),
             torch.empty(cap, dtype=torch.float64, device="cuda")) for _ in range(n_ctx)]
    ctxs = []
    for i in range(n_ctx):
        s = System(dirpath, runin=runin, form=form)
        s.seed(seed + i)
        ctxs.append(s)
    torch.cuda.synchronize()
    got = [0] * n_ctx
    errs = []

    def work(i):
        try:
            s, (bd, be) = ctxs[i], bufs[i]
            while got[i] < per:
                d, _ = s.collect_surrogate_data(moves_per_call, moves_per_call,
                                                out=(bd[got[i]:], be[got[i]:]))
                got[i] += d.shape[0]
        except Exception as ex:  # reported below
            errs.append(ex)

    t0 = time.time()
    th = [threading.Thread(target=work, args=(i,)) for i in range(n_ctx)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.time() - t0
    for s in ctxs:
        s.close()
    if errs:
        raise errs[0]
    desc = torch.cat([b[0][:min(g, per)] for b, g in zip(bufs, got)])
    de = torch.cat([b[1][:min(g, per)] for b, g in zip(bufs, got)])
    return desc, de, wall


def fit(desc, de, epochs=20, batch=4096, lr=1e-3, seed=1, holdout=0.05, device=0):
    """Trains a surrogate on (desc, de); returns it with its statistics on a
    held-out part (RMSE against the exact change, clipped range)."""
    import torch
    n = desc.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g).to(desc.device)
    n_test = max(1, int(holdout * n))
    test, train = perm[:n_test], perm[n_test:]
    x_tr = desc[train].contiguous()
    t_tr, y_scale = targets(de[train])
    mu, isd = normalisation(x_tr)
    sg = Surrogate(seed=seed, device=device)
    sg.set_norm(mu, isd, y_scale)
    t0 = time.time()
    losses = sg.train(x_tr, t_tr.contiguous(), batch=batch, epochs=epochs, lr=lr, seed=seed)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    pred = sg.predict_device(desc[test].contiguous()).double()
    exact = de[test]
    inside = exact.abs() < CLIP
    err = (pred - exact)[inside]
    stats = {"n_train": int(train.numel()), "n_test": int(n_test), "epochs": epochs,
             "batch": batch, "lr": lr, "loss_first": float(losses[0]),
             "loss_last": float(losses[-1]), "train_seconds": train_s,
             "rmse_vs_fp64": float(err.pow(2).mean().sqrt().item()),
             "exact_std": float(exact[inside].std().item()),
             "test_fraction_clipped": float(1.0 - inside.double().mean().item())}
    return sg, stats


def save(sg, path, **meta):
    mu, isd, y_scale = sg.norm
    np.savez_compressed(path, params=sg.params(), mu=mu, isd=isd, y_scale=np.float32(y_scale),
                        **{k: np.asarray(v) for k, v in meta.items()})


def load(path, device=0):
    z = np.load(path)
    sg = Surrogate(seed=0, device=device)
    sg.set_params(z["params"])
    sg.set_norm(z["mu"], z["isd"], float(z["y_scale"]))
    return sg


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="bulk_20000_pinned")
    ap.add_argument("--samples", type=int, default=2000000)
    ap.add_argument("--contexts", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    spec = systems.CONFIGS[a.workload]
    with tempfile.TemporaryDirectory() as d:
        systems.write_bulk(d, spec, seed=20261203)
        desc, de, gen_s = collect(d, a.samples, n_ctx=a.contexts, seed=1000 + a.seed)
    sg, st = fit(desc, de, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed)
    st.update(workload=a.workload, samples=int(desc.shape[0]), collect_seconds=gen_s)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    save(sg, a.out, **{k: v for k, v in st.items()})
    print({k: (round(v, 5) if isinstance(v, float) else v) for k, v in st.items()})


if __name__ == "__main__":
    main()
