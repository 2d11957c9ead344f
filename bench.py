#!/usr/bin/env python
"""Benchmark of the Monte Carlo energy-difference hot path on one GB300.

Workload (default ``bulk_20000_pinned``): 100 chains x 100 beads (charge -1)
plus 10,000 +1 counterions, periodic cube L = 80, LJ eps = sigma = 1 cut at
2.5, harmonic bonds k = 400 r0 = 1, lB = 3, Ewald alpha = (5.6/L)^2 with the
real-space cut-off at L/2 and |n| <= 12 per axis (7,812 half-space k-vectors),
move mix ion 0.3 / COM 0.1 / pivot 0.2 / crankshaft 0.2 / reptation 0.2.
Seeded synthetic initial configurations (self-avoiding chains, uniform ions,
no pair closer than 0.8 sigma), written in the reference's input formats.

A "step" is a batch of Monte Carlo moves run on the device. Reported:
  value        moves/s of the chosen form: 64 replicas in one batch, precision
               form (FP32 pair/k arithmetic, FP64 S(k) and totals), delayed
               acceptance with the learned surrogate, and each replica's full
               FP64 recompute every 1e4 of its moves (staggered over the
               replicas, inside the timed region); device time
  e2e          the same through the public batch call with every replica's
               running energies copied to the host after every step
  plain_fp64   moves/s of the plain FP64 form on one system, with its own
               FP64-pipe roofline and an e2e through plum_run_moves (the
               recorded mt19937 stream copied in, per-move logs copied out)
  precision_on_chain
               FP32 against FP64 energy changes of the chain's own proposals
               (both forms fed one recorded stream) on the 1,000-particle
               bulk system, this workload and a confined-brush replica: error
               and the fraction of Metropolis decisions that flip
  equilibrium  burn-in of 16 replicas with the chosen form, tau_int of the
               chains' Rg^2 (Sokal window, c = 5) for the chosen form and the
               plain Metropolis dynamics, and the chosen form's mean energy
               and Rg^2 against plain FP64 runs from the same equilibrated
               starts (2 standard errors of the paired differences)
  samples      Rg-decorrelated samples/s = moves/s / (2 tau_int)
  roofline     FP32 pipe of the batched energy-change kernel: algorithmic
               FLOPs per move x moves per launch / launch time, over the FP32
               FMA peak measured on this GPU by a probe kernel
  cpu_baseline the FP64 CPU restatement of the reference (the reference
               itself cannot hold 20,000 particles: O(N^2) std::map storage)
               on a bounded sample of moves, one core

``--impl reference`` times the reference's CPU path (the CPU restatement, one
process per host core). ``--only MODE`` runs one profiling case instead.
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

# DRAM bytes per evaluated move of the batched energy-change kernel on this
# workload: dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture
# (64 replicas, every move evaluated: 44 MB per launch of 64 moves)
TRAFFIC_PER_EXACT_MOVE = 44.0e6 / 64


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


def paired_check(x, y, k=2.0, other="plain_fp64"):
    """Per-replica means x (chosen form) and y (the other arm: plain FP64, or
    plain Metropolis dynamics) paired by their starting configuration: the
    mean difference against k standard errors of the paired differences."""
    import numpy as np
    diff = np.asarray(x, np.float64) - np.asarray(y, np.float64)
    se = float(diff.std(ddof=1) / math.sqrt(len(diff)))
    return {"chosen_mean": float(np.mean(x)), other + "_mean": float(np.mean(y)),
            "paired_difference": float(diff.mean()), "standard_error": se,
            "within_2_se": bool(abs(diff.mean()) <= k * se)}


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


def _write_brush(job):
    from plum_gb300 import systems
    d, spec, seed = job
    systems.write_brush(d, spec, seed=seed)
    return d


def make_brush_ensemble(n, seed=20261203, only=None):
    """The confined-brush replicas of uneven size (systems.brush_ensemble);
    `only` picks one replica index. Missing ones are written by a process
    pool (spawned, so it never forks a process that holds a CUDA context)."""
    import concurrent.futures
    import multiprocessing
    from plum_gb300 import systems
    dirs, todo = [], []
    for i, spec in enumerate(systems.brush_ensemble(n, seed)):
        if only is not None and i != only:
            continue
        d = os.path.join(tempfile.gettempdir(), "plum_bench_brush_%d_%d" % (seed, i))
        if not os.path.exists(os.path.join(d, "run.in")):
            todo.append((d, spec, seed + i))
        dirs.append(d)
    if len(todo) > 1:
        workers = max(1, min(len(todo), os.cpu_count() or 1, 16))
        with concurrent.futures.ProcessPoolExecutor(
                workers, mp_context=multiprocessing.get_context("spawn")) as ex:
            list(ex.map(_write_brush, todo))
    else:
        for job in todo:
            _write_brush(job)
    return dirs


def shipped_surrogate(workload, device, margin):
    """The surrogate trained for this workload (plum_gb300/data), or None."""
    import numpy as np
    wpath = os.path.join(ROOT, "plum_gb300", "data", "surrogate_%s.npz" % workload)
    if not os.path.exists(wpath):
        return None, None, wpath
    from plum_gb300 import surrogate as S
    sg = S.load(wpath, device=device)
    sg.set_margin(margin)
    z = np.load(wpath)
    meta = {k: (z[k].item() if z[k].ndim == 0 else None) for k in z.files
            if k not in ("params", "mu", "isd")}
    return sg, meta, wpath


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


def precision_on_chain(d, device, n, seed, label):
    """FP32 against FP64 energy changes on the chain's own proposals: a plain
    (FP64) and a precision (FP32) context of the same system run the same
    recorded mt19937 stream with per-step energy-change logs, so they propose
    the same moves until their first differing decision (a flip; after it the
    chains diverge and the comparison stops, the flipping proposal included).
    For uniform u the decisions u < exp(-beta dE32) and u < exp(-beta dE64)
    differ with probability |min(1, e^{-beta dE32}) - min(1, e^{-beta dE64})|;
    its mean over the proposals is the expected flip fraction."""
    import numpy as np
    import plum_gb300 as pg
    s64 = pg.System(d, form=pg.FORM_FP64, device=device)
    s32 = pg.System(d, form=pg.FORM_FP32, device=device)
    beta = s64.run_params().beta
    ms = s64.topology()[0]
    max_len = int(np.diff(ms).max())
    stream = mt19937_stream(seed, n * (24 + 4 * max_len) + 65536)
    t0 = time.perf_counter()
    _, mt64, ac64, _, de64 = s64.run_moves_de(stream, n)
    _, mt32, ac32, _, de32 = s32.run_moves_de(stream, n)
    wall = time.perf_counter() - t0
    same = (mt64 == mt32) & (ac64 == ac32)
    first = n if same.all() else int(np.argmin(same))
    k = min(n, first + 1)
    mt, a, b = mt64[:k], de64[:k], de32[:k]
    live = (mt >= 0) & np.isfinite(a) & np.isfinite(b)

    def prob(x):
        return np.where(x >= 1e8, 0.0, np.exp(-beta * np.maximum(x, 0.0)))

    fin = live & (a < 1e8) & (b < 1e8)
    err = np.abs(b - a)
    rel = err / np.maximum(1.0, np.abs(a))
    flips = np.abs(prob(b) - prob(a))
    rel_sel = fin & (np.abs(a) <= 30.0 / beta)
    by_kind = {}
    for kind, name in enumerate(("ion", "com", "pivot", "crankshaft", "reptation")):
        sel = fin & (mt == kind)
        if sel.any():
            by_kind[name] = {"proposals": int(sel.sum()),
                             "de_abs_err_rms": float(np.sqrt((err[sel] ** 2).mean())),
                             "de_abs_err_max": float(err[sel].max()),
                             "de_rel_err_max": float(rel[sel].max()),
                             "expected_flip_fraction": float(flips[sel].mean())}
    out = {"system": label, "n_bead": int(s64.n_bead), "proposals": int(live.sum()),
           "steps_compared": int(k), "first_differing_decision": None if first == n else first,
           "overlap_agreement": float(((a[live] >= 1e8) == (b[live] >= 1e8)).mean()),
           "de_abs_err_rms": float(np.sqrt((err[fin] ** 2).mean())) if fin.any() else None,
           "de_abs_err_max": float(err[fin].max()) if fin.any() else None,
           "de_rel_err_max": float(rel[fin].max()) if fin.any() else None,
           "expected_flip_fraction": float(flips[live].mean()) if live.any() else None,
           # the proposals whose decision can go either way (|dE64| <= 30 kT:
           # acceptance probability above 1e-13); the errors above include
           # overlapping chain moves with dE near 1e7, where 1e-6 relative is
           # tens of kT but the acceptance probability is nil
           "relevant": {"proposals": int(rel_sel.sum()),
                        "de_abs_err_rms": float(np.sqrt((err[rel_sel] ** 2).mean()))
                        if rel_sel.any() else None,
                        "de_abs_err_max": float(err[rel_sel].max()) if rel_sel.any() else None,
                        "definition": "proposals with |dE64| <= 30 / beta"},
           "observed_flips": int(first < n), "by_kind": by_kind, "wall_s": wall,
           "definition": "dE of the FP32 form against the plain FP64 form on the same "
                         "proposals of one chain (recorded stream); relative error over "
                         "max(1, |dE64|); flip fraction = mean |p32 - p64| with "
                         "p = min(1, exp(-beta dE)), 0 at overlap"}
    s64.close()
    s32.close()
    return out


def equilibrium(args, device, sg, tune):
    """Statistics of the chosen form on the workload, against plain
    Metropolis and plain FP64, from common starting configurations.

    R replicas (the first R of the throughput batch: same starts) are burnt
    in with the chosen form; the trace of the mean energy and Rg^2 and the
    energy drift over the last fifth of the burn-in say how close to
    equilibrium the starts are. From them:
      (a) the chosen form and the plain Metropolis dynamics in the precision
          form run side by side for the same number of moves (different
          seeds), sampled every `tau_every` moves: tau_int of the chains'
          Rg^2 (pooled over all chains, Sokal window c = 5, an exponential
          fit when the window does not close) and of the total energy, and
          the paired check of their per-replica means (same protocol;
          delayed acceptance keeps the stationary distribution, so from
          equilibrated starts the means agree, while a relaxing system's
          chosen-form series lags plain Metropolis's, since it accepts fewer
          moves: starts_equilibrated compares the burn-in's final drift over
          the series length with the check's standard error);
      (b) plain Metropolis in FP32 and in FP64 from the same starts with the
          same seeds: the two make the same decisions until a flipped one,
          so their trajectories (and Rg^2, exactly) agree until then; the
          replicas whose trajectories stayed identical and the largest
          energy difference are reported;
      (c) the chosen form's per-replica means against the FP64 runs' of (b):
          the direct check, valid when the starts are equilibrated (the
          burn-in drift says whether they are)."""
    import numpy as np
    import plum_gb300 as pg
    R = args.stat_replicas
    dirs = [make_workload(args.workload, seed=20261203 + r) for r in range(R)]
    out = {"replicas": R, "burn_in_moves_per_replica": args.burn}
    t0 = time.perf_counter()
    eq = pg.Batch(dirs, device=device)
    eq.seed(np.arange(9000, 9000 + R, dtype=np.uint32))
    eq.set_tune(*tune)
    eq.set_groups(2)
    if sg is not None:
        eq.set_surrogate(sg)
    done = 0
    trace = []
    while done < args.burn:
        step = min(args.burn - done, max(args.burn // 30, 1000))
        eq.run(step)
        done += step
        trace.append((done, float(eq.energies().sum(axis=1).mean()),
                      float(np.mean([eq.replica(r).observables()[0] for r in range(R)]))))
    snap = [eq.replica(r).positions() for r in range(R)]
    eq.close()
    out["burn_in_s"] = time.perf_counter() - t0
    out["burn_in_trace"] = {"moves": [t[0] for t in trace],
                            "mean_energy": [t[1] for t in trace],
                            "mean_rg2": [t[2] for t in trace]}
    k = max(1, len(trace) // 5)
    if len(trace) > k:
        de = trace[-1][1] - trace[-1 - k][1]
        dm = trace[-1][0] - trace[-1 - k][0]
        out["burn_in_energy_drift_per_1e5_moves"] = de / dm * 1e5
        out["burn_in_rg2_drift_per_1e5_moves"] = (trace[-1][2] - trace[-1 - k][2]) / dm * 1e5

    def series(net, seed0, moves, every):
        b = pg.Batch(dirs, device=device)
        b.seed(np.arange(seed0, seed0 + R, dtype=np.uint32))
        b.set_tune(*tune)
        b.set_groups(2)
        for r in range(R):
            b.replica(r).set_positions(snap[r])
        if net is not None:
            b.set_surrogate(net)
        reps = [b.replica(r) for r in range(R)]
        E, G, Gm = [], [], []
        t1 = time.perf_counter()
        for _ in range(moves // every):
            b.run(every)
            E.append(b.energies().sum(axis=1))
            rg = [rep.chain_observables()[:, 0] for rep in reps]
            G.append(np.concatenate(rg))
            Gm.append([x.mean() for x in rg])
        wall = time.perf_counter() - t1
        b.close()
        return np.array(E), np.array(G), np.array(Gm), wall

    res = {}
    for name, net, seed0 in (("chosen_form", sg, 11000), ("plain_dynamics_fp32", None, 13000)):
        E, G, Gm, wall = series(net, seed0, args.tau_moves, args.tau_every)
        tg, mg = tau_pooled(G)
        te, me = tau_pooled(E)
        res[name] = {"tau_rg2_moves": tg * args.tau_every, "tau_rg2_method": mg,
                     "tau_energy_moves": te * args.tau_every, "tau_energy_method": me,
                     "samples": int(len(E)), "moves_per_sample": args.tau_every,
                     "moves_per_replica": int(len(E) * args.tau_every), "chains": int(G.shape[1]),
                     "wall_s": wall, "mean_energy_per_replica": E.mean(axis=0).tolist(),
                     "mean_rg2_per_replica": Gm.mean(axis=0).tolist()}
    out["series"] = res
    ch, pl = res["chosen_form"], res["plain_dynamics_fp32"]
    out["chosen_vs_plain_dynamics"] = {
        "energy": paired_check(ch["mean_energy_per_replica"], pl["mean_energy_per_replica"],
                               other="plain_dynamics"),
        "rg2": paired_check(ch["mean_rg2_per_replica"], pl["mean_rg2_per_replica"],
                            other="plain_dynamics"),
        "definition": "(a): same starts, same number of moves, different seeds; per-replica "
                      "means, mean paired difference against 2 standard errors"}
    # Whether the starts are equilibrated: the energy change the burn-in's
    # final drift would give over the series, against the standard error of
    # (a). Delayed acceptance keeps the stationary distribution but accepts
    # fewer moves, so while the system still relaxes its series lags plain
    # Metropolis's and (a) and (c) measure the relaxation, not a bias.
    drift = out.get("burn_in_energy_drift_per_1e5_moves")
    if drift is not None:
        relax = abs(drift) * args.tau_moves / 1e5
        se_a = out["chosen_vs_plain_dynamics"]["energy"]["standard_error"]
        out["relaxation_over_series_kT"] = relax
        out["starts_equilibrated"] = bool(relax < 2.0 * se_a)

    # (b) FP32 and FP64 plain Metropolis, same starts and seeds
    t1 = time.perf_counter()
    Ep, Gp, same, worst = [], [], 0, 0.0
    for r in range(R):
        s64 = pg.System(dirs[r], form=pg.FORM_FP64, device=device)
        s32 = pg.System(dirs[r], form=pg.FORM_FP32, device=device)
        s64.set_positions(snap[r])
        s32.set_positions(snap[r])
        s64.seed(15000 + r)
        s32.seed(15000 + r)
        e, g, ident = [], [], True
        for _ in range(args.plain_stat_moves // args.plain_stat_every):
            s64.run(args.plain_stat_every)
            s32.run(args.plain_stat_every)
            e64, e32 = s64.energies().sum(), s32.energies().sum()
            g64, g32 = s64.observables()[0], s32.observables()[0]
            e.append(e64)
            g.append(g64)
            if ident:
                ident = g64 == g32
                worst = max(worst, abs(e64 - e32) / max(1.0, abs(e64)))
        same += int(ident)
        Ep.append(np.mean(e))
        Gp.append(np.mean(g))
        s64.close()
        s32.close()
    out["plain_fp64"] = {"moves_per_replica": args.plain_stat_moves,
                         "moves_per_sample": args.plain_stat_every,
                         "wall_s": time.perf_counter() - t1,
                         "mean_energy_per_replica": Ep, "mean_rg2_per_replica": Gp}
    out["fp32_vs_fp64_same_seeds"] = {
        "replicas_identical_trajectories": same, "replicas": R,
        "max_rel_energy_difference_while_identical": worst,
        "definition": "(b): a replica counts as identical when Rg^2 of the FP32 and FP64 "
                      "chains agreed exactly at every sample (no flipped decision)"}
    # (c) the direct check
    out["stat_check"] = {
        "energy": paired_check(ch["mean_energy_per_replica"], Ep),
        "rg2": paired_check(ch["mean_rg2_per_replica"], Gp),
        "definition": "(c): the chosen form's per-replica means over its series against the "
                      "plain FP64 runs' over theirs, each from the same starting configuration; "
                      "valid when the starts are equilibrated (see the burn-in drift)"}
    return out


def brush_ensemble_batch(args, local, flush):
    """The batching form on its own workload: the confined-brush replicas of
    uneven size (walls with 9-3 LJ and surface sites, slab Ewald with a 3H
    vacuum gap), one batch, autotuned items, no surrogate, each replica's FP64
    recompute every 1e4 of its moves inside the timed steps."""
    import numpy as np
    import torch
    import plum_gb300 as pg
    dirs = make_brush_ensemble(args.brush_replicas)
    t0 = time.perf_counter()
    b = pg.Batch(dirs, device=local)
    setup_s = time.perf_counter() - t0
    b.seed(np.arange(31000, 31000 + len(dirs), dtype=np.uint32))
    tune = b.autotune(8)
    for _ in range(2):
        b.run(args.batch_steps)
    ms, n_rc, rc_ms = [], 0, 0.0
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        b.run(args.batch_steps)
        ms.append(b.last_timing()[0])
        _, n, t = b.drift()
        n_rc += n
        rc_ms += t
    n_bead = [b.replica(r).n_bead for r in range(len(dirs))]
    drift_tab, _, _ = b.drift()
    etot = b.energies().sum(axis=1)
    kern = b.time_kernels(8)
    b.close()
    return {"value": len(dirs) * args.batch_steps / (statistics.mean(ms) / 1e3),
            "unit": "moves/s", "replicas": len(dirs), "beads_total": int(sum(n_bead)),
            "beads_min_max": [int(min(n_bead)), int(max(n_bead))],
            "ms_per_step": statistics.mean(ms), "steps_per_batch": args.batch_steps,
            "autotuned_items": tune, "setup_s": setup_s,
            "kernel_ms_per_launch": {"delta": float(kern[0]), "serial": float(kern[1])},
            "recomputes_in_timed_steps": n_rc,
            "recompute_share_of_timed_device_time": rc_ms / max(sum(ms), 1e-9),
            "drift_max_rel_total": float((drift_tab[:, 4] / np.maximum(1.0, np.abs(etot))).max()),
            "workload": "%d confined brush replicas: H in [30, 60], Lx = Ly = 32, 16-64 grafted "
                        "chains of 20-80 beads, charge fraction f in [0.1, 1], 9-3 walls with "
                        "64 LJ sites each, slab Ewald (3H gap)" % len(dirs)}


def precision_cases(args, local):
    """precision_on_chain for the three bulk/confined configurations: the
    1,000-particle bulk system (reference Ewald rule: multi-image real
    space), the benchmark workload and the first confined-brush replica."""
    return [precision_on_chain(make_workload("bulk_1000"), local, args.precision_moves, 21,
                               "bulk_1000 (10 x 50 chains + 500 ions, L = 40, r_c = 28, 460 k)"),
            precision_on_chain(make_workload(args.workload), local, args.precision_moves, 22,
                               args.workload),
            precision_on_chain(make_brush_ensemble(256, only=0)[0], local,
                               args.precision_moves, 23,
                               "brush replica 0 of the 256-replica ensemble")]


def profile_case(args, local):
    """--only MODE: one profiling case, no baselines. Every mode prints one
    JSON line; the cases with an NVTX range let a profiler select the
    launches of interest (ncu --nvtx --nvtx-include "<range>/")."""
    import numpy as np
    import torch
    import plum_gb300 as pg
    if args.only in ("fp32", "fp64"):
        d = make_workload(args.workload)
        s = pg.System(d, form=pg.FORM_FP32 if args.only == "fp32" else pg.FORM_FP64,
                      device=local)
        s.seed(1234)
        M = args.moves_per_step
        for _ in range(args.warmup + args.steps):
            s.run(M)
        torch.cuda.synchronize()
        ms, k = s.last_timing()
        kern = s.time_kernels(min(M, 64))
        print(json.dumps({"profile_run": args.only, "moves_per_step": M, "last_ms": ms,
                          "moves_per_s": M / (ms / 1e3),
                          "kernel_ms_per_launch": {"delta": float(kern[0]),
                                                   "serial": float(kern[1])}}), flush=True)
        return 0
    if args.only == "total":
        # the full FP64 recompute of one replica of the workload
        d = make_workload(args.workload)
        s = pg.System(d, form=pg.FORM_FP32, device=local)
        for _ in range(3):
            s.total_energy()
        torch.cuda.synchronize()
        t = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            s.total_energy()
            t.append(time.perf_counter() - t0)
        print(json.dumps({"profile_run": "total", "workload": args.workload,
                          "ms_per_recompute": 1e3 * statistics.median(t)}), flush=True)
        return 0
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
        if args.real_term != "auto":
            b.set_real_term(args.real_term == "table")
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
                          "pair_loop": "shared h(u) table, paired evaluations" if b.real_term()
                          else "one evaluation at a time",
                          "kernel_ms_per_launch": dict(zip(
                              ("delta", "serial", "descriptor", "inference"),
                              [float(x) for x in b.time_kernels(8)]))}), flush=True)
        return 0
    if args.only == "chosen":
        # the measured form: replicas with the shipped surrogate, autotuned
        # items, two step chains; one batch of 32 steps in the range "chosen"
        sg, _, _ = shipped_surrogate(args.workload, local, args.da_margin)
        b = pg.Batch([make_workload(args.workload, seed=20261203 + r)
                      for r in range(args.replicas)], device=local)
        b.seed(77)
        if sg is not None:
            b.set_surrogate(sg)
        tune = b.autotune(16)
        b.set_groups(args.groups)
        b.run(256)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("chosen")
        b.run(32)
        torch.cuda.nvtx.range_pop()
        ms, k = b.last_timing()
        print(json.dumps({"profile_run": "chosen", "replicas": args.replicas, "tune": tune,
                          "ms_per_32_steps": ms, "kernels": k}), flush=True)
        return 0
    if args.only == "da":
        # a small surrogate trained on 6,000 collected moves, then 16
        # replicas with delayed acceptance: the third batch of 32 steps runs
        # in the range "da", the same without the surrogate in "plain"
        from plum_gb300 import surrogate as S
        d = make_workload(args.workload)
        desc, de, _ = S.collect(d, 6000, n_ctx=1, moves_per_call=10000)
        sg, _ = S.fit(desc, de, epochs=5, batch=1024)
        b = pg.Batch([make_workload(args.workload, seed=20261203 + i) for i in range(16)],
                     device=local)
        b.seed(77)
        res = {}
        for label, net in (("da", sg), ("plain", None)):
            b.set_surrogate(net)
            for i in range(3):
                if i == 2:
                    torch.cuda.nvtx.range_push(label)
                b.run(32)
                if i == 2:
                    torch.cuda.nvtx.range_pop()
            res[label] = b.last_timing()[0]
        print(json.dumps({"profile_run": "da", "ms_per_32_steps": res}), flush=True)
        return 0
    if args.only == "train":
        # one epoch of surrogate training on 65,536 random descriptors in
        # batches of 4,096 (range "train"), then one inference pass ("infer")
        rng = np.random.default_rng(0)
        x = rng.gamma(2.0, 3.0, size=(65536, 96)).astype(np.float32)
        t = rng.normal(0.0, 3.0, 65536).astype(np.float32)
        sg = pg.Surrogate(seed=1)
        sg.set_norm(x.mean(0), 1.0 / (x.std(0) + 1e-3), 3.0)
        xd = torch.tensor(x, device="cuda")
        td = torch.tensor(t, device="cuda")
        torch.cuda.nvtx.range_push("train")
        sg.train(xd, td, batch=4096, epochs=1, lr=1e-3)
        torch.cuda.nvtx.range_pop()
        torch.cuda.nvtx.range_push("infer")
        out = sg.predict_device(xd)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"profile_run": "train", "mean_abs_s": float(out.abs().mean())}),
              flush=True)
        return 0
    if args.only == "pressure":
        # the wall-force pressure of the first brush replica with charged
        # surface sites (+-0.5): two warm-up evaluations, then `steps` in
        # the range "pressure"
        from plum_gb300 import systems
        spec = systems.brush_ensemble(1, seed=20261203)[0]
        spec.site_charge = 0.5
        d = os.path.join(tempfile.gettempdir(), "plum_bench_pressure")
        if not os.path.exists(os.path.join(d, "run.in")):
            systems.write_brush(d, spec, seed=20261203)
        s = pg.System(d, device=local)
        for _ in range(2):
            s.pressure_slit()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("pressure")
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            s.pressure_slit()
        dt = (time.perf_counter() - t0) / max(1, args.steps)
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"profile_run": "pressure", "n_bead": int(s.n_bead),
                          "n_kvec": int(s.info.n_kvec), "ms_per_evaluation": 1e3 * dt}),
              flush=True)
        return 0
    if args.only == "cbmc":
        print(json.dumps({"profile_run": "cbmc", **cbmc_growth_steps(local)}), flush=True)
        return 0
    if args.only == "precision":
        print(json.dumps({"profile_run": "precision",
                          "cases": precision_cases(args, local)}), flush=True)
        return 0
    if args.only == "stats":
        sg, _, _ = shipped_surrogate(args.workload, local, args.da_margin)
        tune = tuple(int(x) for x in args.tune.split(",")) if args.tune else (4096, 256, 608, 4)
        print(json.dumps({"profile_run": "stats", **equilibrium(args, local, sg, tune)}),
              flush=True)
        return 0
    raise SystemExit("unknown profiling mode %r" % args.only)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bulk_20000_pinned")
    ap.add_argument("--moves-per-step", type=int, default=2000)
    ap.add_argument("--plain-moves-per-step", type=int, default=200)
    ap.add_argument("--cpu-moves", type=int, default=20)
    ap.add_argument("--ref-moves", type=int, default=10)
    ap.add_argument("--tune", default=None,
                    help="item_pairs,k_tile,grid,min_blocks instead of autotuning")
    ap.add_argument("--groups", type=int, default=2, choices=[1, 2],
                    help="step chains per batch (two: halves in two graph branches)")
    ap.add_argument("--replicas", type=int, default=64,
                    help="replicas of the workload in the batched form (the chosen form)")
    ap.add_argument("--batch-steps", type=int, default=256)
    ap.add_argument("--da-margin", type=float, default=12.0,
                    help="delayed-acceptance dead zone in k_BT (stage one rejects only moves "
                         "the surrogate puts above it)")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="time the batched precision form without delayed acceptance")
    ap.add_argument("--precision-moves", type=int, default=10000,
                    help="proposals per configuration for the FP32-vs-FP64 comparison")
    ap.add_argument("--stats", type=int, default=1, help="0: skip the equilibrium block")
    ap.add_argument("--brush-replicas", type=int, default=256,
                    help="replicas of the confined-brush ensemble measured after the "
                         "headline (0: skip)")
    ap.add_argument("--stat-replicas", type=int, default=16)
    ap.add_argument("--burn", type=int, default=500000,
                    help="burn-in moves per replica (chosen form) before the statistics")
    ap.add_argument("--tau-moves", type=int, default=750000,
                    help="moves per replica of each tau series")
    ap.add_argument("--tau-every", type=int, default=2500)
    ap.add_argument("--plain-stat-moves", type=int, default=20000,
                    help="moves per replica of the plain FP64 statistics runs")
    ap.add_argument("--plain-stat-every", type=int, default=1000)
    ap.add_argument("--real-term", default="auto", choices=["auto", "table", "fit"],
                    help="pair loop of the batched kernel: the autotuner's pick, the shared "
                         "h(u) table with paired evaluations, or one evaluation at a time")
    ap.add_argument("--only", default=None,
                    choices=[None, "fp32", "fp64", "total", "batch", "chosen", "da", "train",
                             "pressure", "cbmc", "precision", "stats"],
                    help="profiling runs: one case only, no baselines or e2e")
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
    if args.only:
        return profile_case(args, local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    d = make_workload(args.workload)
    M = args.moves_per_step
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    # the chosen form: replicas of the workload in one batch (precision form,
    # FP64 recompute every 1e4 moves per replica) with delayed acceptance by
    # the learned surrogate when its weights exist
    R, BS = args.replicas, args.batch_steps
    dirs = [make_workload(args.workload, seed=20261203 + r) for r in range(R)]
    batch = pg.Batch(dirs, device=local)
    batch.seed(replicas.replica_seed(rank))
    sg, sg_meta, wpath = (None, None, None)
    if not args.no_surrogate:
        sg, sg_meta, wpath = shipped_surrogate(args.workload, local, args.da_margin)
    if sg is not None:
        batch.set_surrogate(sg)
    # work-item sizes of the batched energy change, timed on these replicas;
    # then the replicas' step chains in two graph branches (halves)
    tune = batch.autotune(16)
    if args.real_term != "auto":
        batch.set_real_term(args.real_term == "table")
    real_term = ("shared h(u) table, paired evaluations" if batch.real_term()
                 else "one evaluation at a time")
    batch.set_groups(args.groups)
    for _ in range(args.warmup):
        batch.run(BS)
    da0 = np.array(batch.da_stats()) if sg is not None else None

    sampler = ClockSampler(local)
    sampler.start()
    dev_ms, kernels, n_rc, rc_ms = [], 0, 0, 0.0
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
        _, n, t = batch.drift()
        n_rc += n
        rc_ms += t
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    value, step_ms = replicas.job_rate(statistics.mean(dev_ms), R * BS, world, dist)
    drift_tab, _, _ = batch.drift()
    etot = batch.energies().sum(axis=1)
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
    # the same form with the recompute every 1e5 moves per replica: the timed
    # step time without its recomputes plus a tenth of their measured time
    step_wo = (sum(dev_ms) - rc_ms) / len(dev_ms)
    per_rc = rc_ms / max(n_rc, 1)
    value_1e5 = R * BS / ((step_wo + R * BS / 1e5 * per_rc) / 1e3) if n_rc else value
    recompute = {"every_moves_per_replica": 10000, "recomputes_in_timed_steps": n_rc,
                 "device_ms_in_timed_steps": rc_ms,
                 "share_of_timed_device_time": rc_ms / max(sum(dev_ms), 1e-9),
                 "ms_per_recompute": rc_ms / max(n_rc, 1),
                 "drift_last_max_abs_total": float(np.abs(drift_tab[:, :4].sum(axis=1)).max()),
                 "drift_max_abs_total": float(drift_tab[:, 4].max()),
                 "drift_max_rel_total": float((drift_tab[:, 4]
                                               / np.maximum(1.0, np.abs(etot))).max()),
                 "recomputes_per_replica_so_far": [int(x) for x in drift_tab[:, 5]],
                 "value_without_recomputes": R * BS / (step_wo / 1e3),
                 "value_recompute_every_1e5": value_1e5,
                 "value_recompute_every_1e5_definition":
                     "derived: the timed steps' device time without their recomputes plus "
                     "one tenth of the recompute time per step (a 1e5 cadence); the drift "
                     "over 1e4 moves is drift_max_rel_total"}

    # e2e through the public batch call: every step, every replica's running
    # energies come back to the host (the result a user samples)
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        t1 = time.perf_counter()
        batch.run(BS)
        e = batch.energies()
        e2e_t.append(time.perf_counter() - t1)
    e2e = R * BS / statistics.mean(e2e_t)
    e2e_d2h = int(e.nbytes)

    # per-kernel CUDA-event durations over a few more steps (plain launches)
    kern_ms = batch.time_kernels(32)
    batch.close()

    # the same replicas (same starts and seeds) without the surrogate:
    # FP32 + batched
    nb = pg.Batch(dirs, device=local)
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
    nb.close()
    brush = None
    if args.brush_replicas > 0:
        try:
            brush = brush_ensemble_batch(args, local, flush)
        except Exception as e:  # a secondary line: report the failure, keep the headline
            brush = {"error": "%s: %s" % (type(e).__name__, e)}

    # plain FP64 on one system of the workload: moves/s, per-kernel times and
    # an e2e through plum_run_moves (recorded stream in, logs out)
    s64 = pg.System(d, form=pg.FORM_FP64, device=local)
    s64.seed(1234 + rank)
    info = s64.info
    for _ in range(2):
        s64.run(args.plain_moves_per_step)
    p_ms = []
    for _ in range(max(3, args.steps // 2)):
        s64.run(args.plain_moves_per_step)
        p_ms.append(s64.last_timing()[0])
    plain = args.plain_moves_per_step / (statistics.mean(p_ms) / 1e3)
    kern64 = s64.time_kernels(64)
    n64 = args.plain_moves_per_step
    stream64 = mt19937_stream(99 + rank, n64 * (24 + 4 * 100))
    s64.run_moves(stream64, n64)
    t64 = []
    for _ in range(3):
        t1 = time.perf_counter()
        s64.run_moves(stream64, n64)
        t64.append(time.perf_counter() - t1)
    e2e64 = n64 / statistics.median(t64)
    s64.close()

    # one replica of the precision form alone, and its e2e (recorded stream)
    s32 = pg.System(d, form=pg.FORM_FP32, device=local)
    s32.seed(1234 + rank)
    s32.run(M)
    f_ms = []
    for _ in range(3):
        s32.run(M)
        f_ms.append(s32.last_timing()[0])
    single32 = M / (statistics.mean(f_ms) / 1e3)
    stream32 = mt19937_stream(98 + rank, M * (24 + 4 * 100))
    t32 = []
    for _ in range(3):
        t1 = time.perf_counter()
        s32.run_moves(stream32, M)
        t32.append(time.perf_counter() - t1)
    e2e32 = M / statistics.median(t32)
    s32.close()

    # FP32 against FP64 on the chain's own proposals (configs 0, 1, 2)
    prec = precision_cases(args, local)
    cbmc = cbmc_growth_steps(local)

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
    achieved64 = W / (kern64[0] / 1e3) / 1e12

    eqm = None
    if args.stats:
        eqm = equilibrium(args, local, sg, tune)
    samples = None
    if eqm is not None:
        tc = eqm["series"]["chosen_form"]["tau_rg2_moves"]
        tp = eqm["series"]["plain_dynamics_fp32"]["tau_rg2_moves"]
        chosen = value / (2 * tc)
        plain_s = plain / (2 * tp)
        samples = {"definition": "moves/s / (2 tau_int), tau_int of the chains' Rg^2 in moves "
                                 "per system (Sokal window, c = 5, autocorrelation pooled over "
                                 "all chains of the equilibrium block's replicas, after its "
                                 "burn-in)",
                   "tau_chosen_form": {"moves": tc,
                                       "method": eqm["series"]["chosen_form"]["tau_rg2_method"]},
                   "tau_plain_dynamics": {"moves": tp, "method": eqm["series"][
                       "plain_dynamics_fp32"]["tau_rg2_method"]},
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

    line = {
        "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "n_bead": info.n_bead, "n_kvec_half": info.n_kvec,
                   "real_cutoff": info.real_cutoff, "replicas": R, "steps_per_batch": BS,
                   "moves_per_step": R * BS,
                   "form": "batched replicas, precision form (FP32 pair/k, FP64 S(k) and "
                           "totals), each replica's full FP64 recompute every 1e4 of its "
                           "moves inside the timed steps" +
                           (", delayed acceptance with the learned surrogate" if sg else ""),
                   "l2": "flushed between steps (256 MB write)", "parallelism": "replicas",
                   "autotuned_items": {"pairs_per_item": tune[0], "k_per_tile": tune[1],
                                       "grid": tune[2], "resident_blocks_per_sm": tune[3],
                                       "pair_loop": real_term},
                   "step_chains": args.groups},
        "fp64_recompute": recompute,
        "batched_fp32_no_surrogate": {"value": batched32, "unit": "moves/s",
                                      "ms_per_step": statistics.mean(nb_ms),
                                      "autotuned_items": tune_nb},
        "batched_brush_ensemble": brush,
        "delayed_acceptance": da,
        "kernel_ms_per_launch": {
            "chosen_form": dict(zip(("delta", "serial", "descriptor", "inference"),
                                    [float(x) for x in kern_ms])),
            "no_surrogate": dict(zip(("delta", "serial", "descriptor", "inference"),
                                     [float(x) for x in kern_ms_nb])),
            "plain_fp64": {"delta": float(kern64[0]), "serial": float(kern64[1])}},
        "precision_on_chain": prec,
        "cbmc_trials_grand_canonical": cbmc,
        "single_replica_fp32": {"value": single32, "unit": "moves/s", "moves_per_step": M,
                                "e2e": {"value": e2e32, "unit": "moves/s",
                                        "h2d_bytes_per_step": int(stream32.nbytes),
                                        "d2h_bytes_per_step": M * (4 + 4 + 8)}},
        "plain_fp64": {"value": plain, "unit": "moves/s", "dtype": "f64",
                       "moves_per_step": args.plain_moves_per_step,
                       "e2e": {"value": e2e64, "unit": "moves/s",
                               "h2d_bytes_per_step": int(stream64.nbytes),
                               "d2h_bytes_per_step": n64 * (4 + 4 + 8),
                               "path": "plum_run_moves: the recorded mt19937 stream copied in "
                                       "and per-move logs (type, accept, total energy) copied "
                                       "out in the timed region"},
                       "roofline": {"bound": "fp64", "kernel": "k_delta64",
                                    "achieved": achieved64, "peak": peak64, "unit": "TFLOP/s",
                                    "frac": achieved64 / peak64,
                                    "launch_ms": float(kern64[0]),
                                    "peak_source": "FP64 FMA probe kernel on this GPU"}},
        "speedup_vs_plain_fp64": value / plain,
        "e2e": {"value": e2e, "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": e2e_d2h,
                "path": "plum_batch_run of the chosen form (FP64 recomputes included) and "
                        "plum_batch_energies every step: all replicas' running energies "
                        "copied to the host; a Monte Carlo step takes no host input (the "
                        "replicas' generators and configurations stay on the device; the "
                        "configurations were uploaded when the batch was created)"},
        "gpu_launches": int(kernels),
        "roofline": {"bound": "fp32", "kernel": "k_batch_delta32",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": TRAFFIC_PER_EXACT_MOVE * evaluated,
                     "traffic_source": "DRAM bytes (dram__bytes_read.sum + dram__bytes_write"
                                       ".sum) of one ncu capture of this kernel on this "
                                       "workload, per evaluated move, times the moves one "
                                       "launch evaluates",
                     "launch_ms": float(kern_ms[0]), "moves_per_launch": evaluated,
                     "peak_source": "FP32 FMA probe kernel on this GPU (measured; the "
                                    "measured-peaks file has no FP32 entry)",
                     "fp64_peak_tflops": peak64,
                     "alg_flops_per_move": W},
        "equilibrium": eqm,
        "samples": samples,
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
