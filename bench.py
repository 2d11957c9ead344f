#!/usr/bin/env python
"""Benchmark of the Monte Carlo energy-difference hot path on one GB300.

Workload (default ``bulk_20000_pinned``): 100 chains x 100 beads (charge -1)
plus 10,000 +1 counterions, periodic cube L = 80, LJ eps = sigma = 1 cut at
2.5, harmonic bonds k = 400 r0 = 1, lB = 3, Ewald alpha = (5.6/L)^2 with the
real-space cut-off at L/2 and |n| <= 12 per axis (7,812 half-space k-vectors),
move mix ion 0.3 / COM 0.1 / pivot 0.2 / crankshaft 0.2 / reptation 0.2.
Seeded synthetic initial configuration (self-avoiding chains, uniform ions,
no pair closer than 0.8 sigma), written in the reference's input formats.

A "step" is a batch of Monte Carlo moves run on the device. Reported:
  value        moves/s of the precision form (FP32 pair/k arithmetic, FP64
               accumulators, FP64 recompute every 1e4 moves), device time
  plain_fp64   moves/s of the plain FP64 form on the same system
  e2e          moves/s through the C ABI with host buffers: the recorded
               mt19937 stream copied in and the per-move logs copied out
               inside the timed region
  samples      Rg-decorrelated samples/s (tau_int of the chain-averaged Rg^2
               series, Sokal window c = 5) when --samples-seconds > 0
  roofline     FP32 pipe: algorithmic FLOPs per move x moves/s over the FP32
               FMA peak measured on this GPU by a probe kernel
  cpu_baseline the FP64 CPU restatement of the reference (the reference
               itself cannot hold 20,000 particles: O(N^2) std::map storage)
               on a bounded sample of moves, one core

``--impl reference`` times the reference's CPU path (oracle/_ref where the
reference compiled, else the CPU restatement) with one process per host core.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC moves/s and Rg-decorrelated samples/s: plain FP64 vs chosen form, 1 GB300"


def mt19937_stream(seed: int, n: int):
    """std::mt19937 output words for `seed` (classic init_genrand seeding)."""
    import numpy as np
    key = np.zeros(624, dtype=np.uint32)
    x = seed & 0xFFFFFFFF
    key[0] = x
    for i in range(1, 624):
        x = (1812433253 * (x ^ (x >> 30)) + i) & 0xFFFFFFFF
        key[i] = x
    bg = np.random.MT19937()
    bg.state = {"bit_generator": "MT19937", "state": {"key": key, "pos": 624}}
    return bg.random_raw(n).astype(np.uint32)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                mhz.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(mhz)}


def tau_int(x, c=5.0):
    """Integrated autocorrelation time with Sokal's automatic window."""
    import numpy as np
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    if n < 8:
        return float("nan")
    x = x - x.mean()
    f = np.fft.rfft(x, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n]
    if acf[0] <= 0:
        return float("nan")
    rho = acf / acf[0]
    tau = 0.5
    for w in range(1, n):
        tau += rho[w]
        if w >= c * tau:
            break
    return float(tau)


def chain_rg2(pos, mol_start):
    """Rg^2 of every chain (simulation.cc:406-434: (1/n^2) sum_{j<k} r_jk^2 on
    unwrapped coordinates = mean squared distance from the centre of mass)."""
    import numpy as np
    sizes = np.diff(mol_start)
    out = []
    for n in np.unique(sizes[sizes > 1]):
        starts = mol_start[:-1][sizes == n]
        idx = starts[:, None] + np.arange(n)[None, :]
        x = pos[idx]
        out.append(((x - x.mean(axis=1, keepdims=True)) ** 2).sum(axis=2).mean(axis=1))
    return np.concatenate(out)


def tau_pooled(X, c=5.0):
    """Integrated autocorrelation time (in samples) of many series at once
    (columns of X): the autocorrelation is averaged over the columns, then
    Sokal's window; when the window would pass a third of the series, an
    exponential fitted to the decay to 1/e stands in (method says which)."""
    import numpy as np
    X = np.asarray(X, np.float64)
    T = X.shape[0]
    if T < 16:
        return float("nan"), "too short"
    Y = X - X.mean(axis=0, keepdims=True)
    f = np.fft.rfft(Y, 2 * T, axis=0)
    acf = np.fft.irfft(f * np.conj(f), axis=0)[:T].mean(axis=1)
    acf /= np.arange(T, 0, -1)  # unbiased per lag
    if acf[0] <= 0:
        return float("nan"), "flat"
    rho = acf / acf[0]
    tau = 0.5
    for w in range(1, T):
        tau += rho[w]
        if w >= c * tau:
            if w <= T // 3:
                return float(tau), "sokal"
            break
    k = int(np.argmax(rho < math.exp(-1.0)))
    if k < 2:
        return float("nan"), "no decay"
    lags = np.arange(k)
    slope = np.polyfit(lags, np.log(np.maximum(rho[:k], 1e-12)), 1)[0]
    return float(-1.0 / slope), "exponential fit"


def measure_taus(batches, steps_done, mol_start, seconds, every, burn):
    """tau_int of the chains' Rg^2 (moves per replica) for several batches
    started from the same configurations: each is first brought to `burn`
    steps per replica, then all are advanced in turn by `every` steps and
    sampled, so every series covers the same stretch of its trajectory
    (the chains still relax from their initial walks, which biases a tau
    estimate; equal stretches bias them alike)."""
    import numpy as np
    for b, done in zip(batches, steps_done):
        if burn > done:
            b.run(burn - done)
    reps = [[b.replica(r) for r in range(b.n)] for b in batches]
    X = [[] for _ in batches]
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end:
        for i, b in enumerate(batches):
            b.run(every)
            X[i].append(np.concatenate([chain_rg2(r.positions(), mol_start) for r in reps[i]]))
    out = []
    for x in X:
        tau, how = tau_pooled(np.array(x))
        out.append({"tau_moves_per_replica": tau * every, "tau_samples": tau, "method": how,
                    "samples": len(x), "chains": len(x[0]) if x else 0,
                    "moves_per_sample": every, "burn_in_moves": burn})
    return out


def alg_flops_per_move(n_bead, mean_moved, n_k, frac_in_rc, mean_bonds):
    """Algorithmic FP32 work per attempted move, with the weights fixed before
    measuring: 20 per (moved, other) pair for distance and wrap, 8 per image
    check (one image per pair when r_c = L/2), 25 per in-cut-off erfc term,
    12 per in-cut-off LJ pair (negligible at these densities), 16 per (moved
    bead, half-space k) phase pair, 10 per k for the |S|^2 change, 15 per bond.
    Counted once per pair (new configuration), as the reference's algorithm
    does; the kernel evaluates both old and new."""
    pairs = mean_moved * (n_bead - 1)
    return (pairs * (20 + 8) + pairs * frac_in_rc * 25 + mean_moved * n_k * 16
            + n_k * 10 + 15 * mean_bonds)


def run_reference_arm(args, rank, world):
    """The reference's CPU path on the host cores: one process per core, each
    timing a bounded sample of moves on its own copy of the workload."""
    if rank != 0:
        return 0
    d = make_workload(args.workload)
    cores = max(1, min(os.cpu_count() or 1, 16))
    moves = args.ref_moves
    code = (
        "import sys,time; sys.path.insert(0,%r)\n"
        "from oracle import bindings as ob\n"
        "o=ob.Oracle(%r, seed=int(sys.argv[1]), fast_init=True)\n"
        "t=time.time(); o.run(%d); print(time.time()-t)\n" % (ROOT, d, moves))
    steps = []
    for s in range(args.warmup + args.steps):
        procs = [subprocess.Popen([sys.executable, "-c", code, str(1000 + s * 97 + p)],
                                  stdout=subprocess.PIPE, text=True) for p in range(cores)]
        t = [float(p.communicate()[0].strip().splitlines()[-1]) for p in procs]
        if s >= args.warmup:
            steps.append(cores * moves / max(t))
    v = statistics.mean(steps)
    # the restatement is timed (the reference itself cannot hold 20,000
    # particles: O(N^2) pair-energy maps), so the baseline is the port
    kind = "port"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "moves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "moves_per_step": moves * cores,
                       "note": "the reference cannot hold this system; the FP64 CPU "
                               "restatement of its algorithm is timed"},
            "cpu_baseline": {"value": v, "unit": "moves/s", "cores": cores, "kind": kind,
                             "sample": "%d moves per process per step" % moves},
            "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def make_workload(name, seed=20261203):
    from plum_gb300 import systems
    d = os.path.join(tempfile.gettempdir(), "plum_bench_%s_%d" % (name, seed))
    if not os.path.exists(os.path.join(d, "run.in")):
        systems.write_bulk(d, systems.CONFIGS[name], seed=seed)
    return d


def make_brush_ensemble(n, seed=20261203):
    """The confined-brush replicas of uneven size (systems.brush_ensemble)."""
    from plum_gb300 import systems
    dirs = []
    for i, spec in enumerate(systems.brush_ensemble(n, seed)):
        d = os.path.join(tempfile.gettempdir(), "plum_bench_brush_%d_%d" % (seed, i))
        if not os.path.exists(os.path.join(d, "run.in")):
            systems.write_brush(d, spec, seed=seed + i)
        dirs.append(d)
    return dirs


def cbmc_growth_steps(device, reps=200):
    """Trial energies of configurational-bias growth steps on the
    grand-canonical box (L = 50, 40 neutral chains of 30 beads, 2,000 salt
    pairs, 32 trials per grown bead): the precision form's one launch against
    the plain form's FP64 kernels, device time per growth step from CUDA
    events, and the largest FP32 error over the steps."""
    import numpy as np
    import plum_gb300 as pg
    from plum_gb300 import systems
    d = os.path.join(tempfile.gettempdir(), "plum_bench_muvt_L50")
    if not os.path.exists(os.path.join(d, "run.in")):
        systems.write_muvt(d, systems.MuVTSpec(salt_first=True), seed=20261203)
    s64 = pg.System(d, form=pg.FORM_FP64, device=device)
    s32 = pg.System(d, form=pg.FORM_FP32, device=device)
    rng = np.random.default_rng(11)
    T, L = 32, 50.0
    err, rel, t32, t64, n_l = 0.0, 0.0, [], [], None
    for cl in (1, 8, 15, 22, 29):
        start = rng.uniform(0, L, 3)
        st = rng.normal(size=(cl, 3))
        chain = start + np.cumsum(st / np.linalg.norm(st, axis=1)[:, None], axis=0)
        dd = rng.normal(size=(T, 3))
        b1 = chain[-1] + dd / np.linalg.norm(dd, axis=1)[:, None]
        u64 = s64.cbmc_trials(b1, None, chain, None, -1)
        u32 = s32.cbmc_trials(b1, None, chain, None, -1)
        live = u64 < 1e8
        if live.any():
            rel = max(rel, float((np.abs(u32[live] - u64[live])
                                  / np.maximum(1.0, np.abs(u64[live]))).max()))
        small = np.abs(u64) < 50
        if small.any():
            err = max(err, float(np.abs(u32[small] - u64[small]).max()))
        a, n_l = s32.cbmc_time(b1, None, chain, None, -1, reps=reps)
        b, n64 = s64.cbmc_time(b1, None, chain, None, -1, reps=reps)
        t32.append(a)
        t64.append(b)
    ms32, ms64 = statistics.mean(t32), statistics.mean(t64)
    out = {"workload": "muvt_L50: 40 chains x 30 beads (neutral), 2,000 salt pairs, 5,200 beads",
           "trials_per_growth_step": T, "grown_beads": [1, 8, 15, 22, 29],
           "fp32_one_launch_ms": ms32, "fp32_launches": n_l,
           "fp64_ms": ms64, "fp64_launches": n64,
           "fp32_trial_sites_per_s": T / (ms32 / 1e3),
           "fp32_vs_fp64": ms64 / ms32, "max_abs_err_vs_fp64_kT_where_u_below_50": err,
           "max_rel_err_vs_fp64": rel}
    s32.close()
    s64.close()
    return out


def cpu_baseline_sample(d, moves):
    code = ("import sys,time; sys.path.insert(0,%r)\n"
            "from oracle import bindings as ob\n"
            "o=ob.Oracle(%r, seed=7, fast_init=True)\n"
            "t=time.time(); o.run(%d); print(time.time()-t)\n" % (ROOT, d, moves))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    t = float(out.stdout.strip().splitlines()[-1])
    return moves / t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bulk_20000_pinned")
    ap.add_argument("--moves-per-step", type=int, default=2000)
    ap.add_argument("--plain-moves-per-step", type=int, default=200)
    ap.add_argument("--samples-seconds", type=float, default=150.0,
                    help="seconds of Rg sampling (both forms together) for tau_int (0: skip)")
    ap.add_argument("--cpu-moves", type=int, default=20)
    ap.add_argument("--ref-moves", type=int, default=10)
    ap.add_argument("--tune", default=None,
                    help="with --only batch: item_pairs,k_tile,grid,min_blocks instead of autotuning")
    ap.add_argument("--groups", type=int, default=2, choices=[1, 2],
                    help="step chains per batch (two: halves in two graph branches)")
    ap.add_argument("--tau-replicas", type=int, default=16,
                    help="replicas whose chains' Rg^2 series give tau_int")
    ap.add_argument("--replicas", type=int, default=64,
                    help="replicas of the workload in the batched form (the chosen form)")
    ap.add_argument("--batch-steps", type=int, default=256)
    ap.add_argument("--da-margin", type=float, default=12.0,
                    help="delayed-acceptance dead zone in k_BT (stage one rejects only moves "
                         "the surrogate puts above it)")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="time the batched precision form without delayed acceptance")
    ap.add_argument("--only", default=None, choices=[None, "fp32", "fp64", "batch", "cbmc"],
                    help="profiling runs: time one form only, no baselines or e2e")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    from plum_gb300 import replicas

    import numpy as np
    import torch
    import plum_gb300 as pg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.only == "batch":
        if args.workload.startswith("brush_"):
            dirs = make_brush_ensemble(int(args.workload.split("_")[1]))
        else:
            dirs = [make_workload(args.workload, seed=20261203 + r) for r in range(args.replicas)]
        t0 = time.perf_counter()
        b = pg.Batch(dirs, device=local)
        setup_s = time.perf_counter() - t0
        b.seed(77)
        if args.tune:
            tune = tuple(int(x) for x in args.tune.split(","))
            b.set_tune(*tune)
        else:
            tune = b.autotune(8)
        for _ in range(args.warmup):
            b.run(args.batch_steps)
        ms_all = []
        for _ in range(args.steps):
            b.run(args.batch_steps)
            ms_all.append(b.last_timing()[0])
        ms = statistics.mean(ms_all)
        n_bead = sum(b.replica(r).n_bead for r in range(len(dirs)))
        print(json.dumps({"profile_run": "batch", "workload": args.workload,
                          "replicas": len(dirs), "beads_total": int(n_bead),
                          "steps": args.batch_steps, "ms_per_batch": ms,
                          "moves_per_s": len(dirs) * args.batch_steps / (ms / 1e3),
                          "autotuned_items": tune, "setup_s": setup_s,
                          "kernel_ms_per_launch": dict(zip(
                              ("delta", "serial", "descriptor", "inference"),
                              [float(x) for x in b.time_kernels(8)]))}), flush=True)
        return 0
    if args.only == "cbmc":
        print(json.dumps({"profile_run": "cbmc", **cbmc_growth_steps(local)}), flush=True)
        return 0
    d = make_workload(args.workload)
    M = args.moves_per_step
    s32 = pg.System(d, form=pg.FORM_FP32, device=local)
    s64 = pg.System(d, form=pg.FORM_FP64, device=local)
    info = s32.info
    s32.seed(1234 + rank)
    s64.seed(1234 + rank)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")


    if args.only:
        s = s32 if args.only == "fp32" else s64
        for _ in range(args.warmup + args.steps):
            s.run(M)
        torch.cuda.synchronize()
        ms, k = s.last_timing()
        print(json.dumps({"profile_run": args.only, "moves_per_step": M, "last_ms": ms,
                          "moves_per_s": M / (ms / 1e3)}), flush=True)
        return 0

    # the chosen form: replicas of the workload in one batch (precision form)
    # with delayed acceptance by the learned surrogate when its weights exist
    R, BS = args.replicas, args.batch_steps
    batch = pg.Batch([make_workload(args.workload, seed=20261203 + r) for r in range(R)],
                     device=local)
    batch.seed(replicas.replica_seed(rank))
    sg, sg_meta = None, None
    wpath = os.path.join(ROOT, "plum_gb300", "data", "surrogate_%s.npz" % args.workload)
    if os.path.exists(wpath) and not args.no_surrogate:
        from plum_gb300 import surrogate as S
        sg = S.load(wpath, device=local)
        sg.set_margin(args.da_margin)
        z = np.load(wpath)
        sg_meta = {k: (z[k].item() if z[k].ndim == 0 else None) for k in z.files
                   if k not in ("params", "mu", "isd")}
        batch.set_surrogate(sg)
    # work-item sizes of the batched energy change, timed on these replicas;
    # then the replicas' step chains in two graph branches (halves)
    tune = batch.autotune(16)
    batch.set_groups(args.groups)
    for _ in range(args.warmup):
        batch.run(BS)
        s32.run(M)
        s64.run(args.plain_moves_per_step)
    da0 = np.array(batch.da_stats()) if sg is not None else None

    sampler = ClockSampler(local)
    sampler.start()
    dev_ms, kernels = [], 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")   # lets a profiler select the timed region
    for _ in range(args.steps):
        flush.zero_()          # L2 flush between steps (outside the step's events)
        torch.cuda.synchronize()
        batch.run(BS)
        ms, k = batch.last_timing()
        dev_ms.append(ms)
        kernels += k
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    value, step_ms = replicas.job_rate(statistics.mean(dev_ms), R * BS, world, dist)
    da = None
    if sg is not None:
        mv, ps, ac = (np.array(batch.da_stats()) - da0).tolist()
        da = {"surrogate_moves": mv, "stage1_pass": ps / max(mv, 1),
              "surrogate_move_acceptance": ac / max(mv, 1),
              "exact_evaluations_skipped": (mv - ps) / float(R * BS * args.steps),
              "margin_kT": args.da_margin,
              "weights": os.path.relpath(wpath, ROOT), "training": sg_meta}
        cs = batch.cell_stats()
        da["descriptor_cell_lists"] = {"replicas": cs[0], "valid_after_timed_steps": cs[1],
                                       "most_beads_that_changed_cell": cs[2],
                                       "capacity_for_them": cs[3]}
    # per-kernel CUDA-event durations over a few more steps (plain launches)
    kern_ms = batch.time_kernels(32)

    # the same replicas (same starts and seeds) without the surrogate:
    # FP32 + batched
    nb = pg.Batch([make_workload(args.workload, seed=20261203 + r) for r in range(R)],
                  device=local)
    nb.seed(replicas.replica_seed(rank))
    tune_nb = nb.autotune(16)
    nb.set_groups(args.groups)
    for _ in range(2):
        nb.run(BS)
    nb_ms = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        nb.run(BS)
        nb_ms.append(nb.last_timing()[0])
    batched32 = R * BS / (statistics.mean(nb_ms) / 1e3)
    kern_ms_nb = nb.time_kernels(32)

    # Rg decorrelation of both dynamics: delayed acceptance changes the
    # acceptance of chain moves, hence tau in moves; the plain Metropolis
    # dynamics is shared by the FP64 and FP32 forms (their decisions differ
    # with the flip fraction below)
    # tau_int is a property of one replica's dynamics, not of the batch size:
    # it is measured on the first TR replicas (same starts and seeds) so the
    # sampling time yields series many tau long
    mol_start = s64.topology()[0]
    tau_da = tau_plain = None
    TR = min(args.tau_replicas, R)
    if args.samples_seconds > 0:
        def tau_batch(net):
            b = pg.Batch([make_workload(args.workload, seed=20261203 + r) for r in range(TR)],
                         device=local)
            b.seed(replicas.replica_seed(rank))
            b.set_tune(*tune)
            if net is not None:
                b.set_surrogate(net)
            return b
        if sg is not None:
            tau_da, tau_plain = measure_taus([tau_batch(sg), tau_batch(None)], [0, 0], mol_start,
                                             args.samples_seconds, 1000, 20000)
        else:
            tau_plain, = measure_taus([tau_batch(None)], [0], mol_start, args.samples_seconds,
                                      1000, 20000)

    # precision form against FP64 on identical trial moves
    from plum_gb300 import precision
    prec = precision.compare(s64, s32, s64.topology()[0], n=200, seed=5)
    cbmc = cbmc_growth_steps(local)

    # one replica of the precision form alone
    f_ms = []
    for _ in range(3):
        s32.run(M)
        f_ms.append(s32.last_timing()[0])
    single32 = M / (statistics.mean(f_ms) / 1e3)

    # plain FP64 on the same system
    p_ms = []
    for _ in range(max(3, args.steps // 2)):
        s64.run(args.plain_moves_per_step)
        p_ms.append(s64.last_timing()[0])
    plain = args.plain_moves_per_step / (statistics.mean(p_ms) / 1e3)

    # e2e through the C ABI with host buffers (stream in, logs out)
    n_e2e = M
    words = n_e2e * (24 + 4 * 100)
    stream = mt19937_stream(99 + rank, words)
    e2e_t = []
    for _ in range(3):
        t1 = time.perf_counter()
        used, mt, ac, et = s32.run_moves(stream, n_e2e)
        e2e_t.append(time.perf_counter() - t1)
    e2e = n_e2e / statistics.median(e2e_t)
    h2d = stream.nbytes
    d2h = n_e2e * (4 + 4 + 8)

    # algorithmic work per move (mean moved beads from the move mix)
    prob = (0.3, 0.1, 0.2, 0.2, 0.2)
    L = 100
    crank_mean = sum(max(0, ((L - f) * u) // 1 - 1) for f in range(L - 1)
                     for u in (0.25, 0.5, 0.75)) / (3 * (L - 1))
    mean_moved = prob[0] * 1 + (prob[1] + prob[2] + prob[4]) * L + prob[3] * crank_mean
    mean_bonds = (1 - prob[0]) * (L - 1)
    frac_in = (4.0 / 3.0) * math.pi * info.real_cutoff ** 3 / (info.box[0] ** 3)
    W = alg_flops_per_move(info.n_bead, mean_moved, info.n_kvec, min(1.0, frac_in), mean_bonds)
    peak, peak64 = pg.probe_peaks(local)
    # dominant kernel: the batched energy change; per launch it evaluates the
    # moves that reach the exact change (all of them without the surrogate)
    evaluated = R * (1.0 - (da["exact_evaluations_skipped"] if da else 0.0))
    achieved = W * evaluated / (kern_ms[0] / 1e3) / 1e12

    samples = None
    if tau_plain is not None:
        tp = tau_plain["tau_moves_per_replica"]
        td = tau_da["tau_moves_per_replica"] if tau_da else tp
        chosen = value / (2 * td)
        plain_s = plain / (2 * tp)
        samples = {"definition": "moves/s / (2 tau_int), tau_int of the chains' Rg^2 in moves per "
                                 "system (Sokal window, c = 5, autocorrelation pooled over all "
                                 "chains of %d replicas with the same starts and seeds as the "
                                 "first %d of the throughput batch)" % (TR, TR),
                   "tau_replicas": TR,
                   "tau_plain": tau_plain, "tau_chosen_form": tau_da,
                   "plain_fp64_samples_per_s": plain_s,
                   "batched_fp32_samples_per_s": batched32 / (2 * tp),
                   "chosen_form_samples_per_s": chosen,
                   "chosen_vs_plain_fp64": chosen / plain_s}

    cpu = None
    if rank == 0:
        try:
            v = cpu_baseline_sample(d, args.cpu_moves)
            cpu = {"value": v, "unit": "moves/s", "cores": 1, "kind": "port",
                   "sample": "%d moves of the FP64 CPU restatement on this workload "
                             "(the reference cannot hold 20,000 particles)" % args.cpu_moves}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": "moves/s", "cores": 1, "kind": "port",
                   "sample": "failed: %s" % e}

    drift = s32.drift()
    line = {
        "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "n_bead": info.n_bead, "n_kvec_half": info.n_kvec,
                   "real_cutoff": info.real_cutoff, "replicas": R, "steps_per_batch": BS,
                   "moves_per_step": R * BS,
                   "form": "batched replicas, precision form (FP32 pair/k, FP64 S(k) and "
                           "totals, FP64 recompute every 1e4 moves)" +
                           (", delayed acceptance with the learned surrogate" if sg else ""),
                   "l2": "flushed between steps (256 MB write)", "parallelism": "replicas",
                   "autotuned_items": {"pairs_per_item": tune[0], "k_per_tile": tune[1],
                                       "grid": tune[2], "resident_blocks_per_sm": tune[3]},
                   "step_chains": args.groups},
        "batched_fp32_no_surrogate": {"value": batched32, "unit": "moves/s",
                                      "ms_per_step": statistics.mean(nb_ms),
                                      "autotuned_items": tune_nb},
        "delayed_acceptance": da,
        "kernel_ms_per_launch": {
            "chosen_form": dict(zip(("delta", "serial", "descriptor", "inference"),
                                    [float(x) for x in kern_ms])),
            "no_surrogate": dict(zip(("delta", "serial", "descriptor", "inference"),
                                     [float(x) for x in kern_ms_nb]))},
        "precision_vs_fp64": prec,
        "cbmc_trials_grand_canonical": cbmc,
        "single_replica_fp32": {"value": single32, "unit": "moves/s", "moves_per_step": M},
        "plain_fp64": {"value": plain, "unit": "moves/s",
                       "moves_per_step": args.plain_moves_per_step},
        "speedup_vs_plain_fp64": value / plain,
        "e2e": {"value": e2e, "unit": "moves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "path": "plum_run_moves: one replica, precision form, recorded mt19937 stream "
                        "copied in and per-move logs copied out in the timed region"},
        "gpu_launches": int(kernels),
        "roofline": {"bound": "fp32", "kernel": "k_batch_delta32",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "launch_ms": float(kern_ms[0]), "moves_per_launch": evaluated,
                     "peak_source": "FP32 FMA probe kernel on this GPU (measured; the "
                                    "measured-peaks file has no FP32 entry)",
                     "fp64_peak_tflops": peak64,
                     "alg_flops_per_move": W},
        "samples": samples,
        "drift_fp32": {"last": list(drift[:4]), "max_abs_total": drift[4]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "wall_s": wall,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
