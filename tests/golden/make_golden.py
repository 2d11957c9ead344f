"""Generates the golden fixtures under tests/golden/<case>/ by running the
reference itself (oracle/_ref/libplumref.so: the unmodified reference sources
linked with oracle/ref_harness.cc) on seeded inputs written by
plum_gb300.systems.

Each case directory holds the three reference-format inputs (run.in,
input_crd.dat, input_top.dat) and ref.npz with, from the reference:
  energies      running totals {pair, ewald, bond, ext} after initialisation
  ewald         potential_ewald_coul.cc:38-115 derived values
  de_mol/de_trial/de_moved/de_out
                ForceField::EnergyDifference on seeded trial configurations
  run_seed, run_type, run_accept, run_draws, run_etot
                a seeded run of the reference's step loop
  run_coords, run_obs, run_rhoz
                final coordinates, observables, rho(z) after the run
  rng_words     the reference generator's first outputs for run_seed

Run from the repository root:  python tests/golden/make_golden.py
[moves] [cbmc] [long | long:<case>] [stats] [gc] [outputs] (needs the reference checkout;
the fixtures themselves are committed). "long" adds long.npz, a 1e5-step
run, to the cases in LONG_CASES (about 40 min each at the reference's
speed); "stats" writes the STAT_CASES with stats.npz, 8 seeded 6e4-step
reference runs each (about 15 min on 8 cores); "outputs" writes the
OUTPUT_CASES: the reference's own output files of a sampled run.
"""
from __future__ import annotations

import os
import shutil
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from oracle import bindings as ob  # noqa: E402
from plum_gb300 import systems  # noqa: E402
from _moves import kind_trials  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "bulk_small": dict(kind="bulk", seed=7, run_seed=123, steps=600,
                       spec=systems.BulkSpec(n_chain=4, chain_len=20, n_ion=80, box=15.0)),
    "bulk_wca": dict(kind="bulk", seed=8, run_seed=321, steps=600,
                     spec=systems.BulkSpec(n_chain=3, chain_len=16, n_ion=48, box=13.0,
                                           lj_cutoff=-1.0, use_bond=False,
                                           move_prob=(0.4, 0.1, 0.2, 0.1, 0.2))),
    "bulk_medium": dict(kind="bulk", seed=9, run_seed=77, steps=400,
                        spec=systems.BulkSpec(n_chain=10, chain_len=20, n_ion=200, box=20.0)),
    "slab_wca": dict(kind="brush", seed=3, run_seed=99, steps=600,
                     spec=systems.BrushSpec(n_graft=4, chain_len=8, lxy=10.0, height=12.0,
                                            n_sites=6, wall_cut=-1.0, charge_frac=0.7)),
    "slab_lj": dict(kind="brush", seed=4, run_seed=98, steps=600,
                    spec=systems.BrushSpec(n_graft=5, chain_len=10, lxy=12.0, height=16.0,
                                           n_sites=8, wall_cut=2.5, charge_frac=0.5)),
    # the other potentials of the reference's pair and external surface
    # (potential_hard_sphere.cc, potential_hard_wall.cc, potential_well_wall.cc);
    # radii below the generators' minimum separation of 0.8 and no surface
    # sites (the external energy counts every bead, the sites included)
    "hs_bulk": dict(kind="bulk", seed=10, run_seed=55, steps=600,
                    spec=systems.BulkSpec(n_chain=4, chain_len=12, n_ion=48, box=13.0),
                    over=dict(pair_kind="HardSphere", hs_radii=(("P", 0.35), ("C", 0.3)))),
    "slab_hardwall": dict(kind="brush", seed=11, run_seed=56, steps=600,
                          spec=systems.BrushSpec(n_graft=4, chain_len=8, lxy=10.0, height=12.0,
                                                 n_sites=0, charge_frac=0.6),
                          over=dict(ext_kind="HardWall",
                                    wall_radii=(("P", 0.5), ("L", 0.0), ("C", 0.5)))),
    "slab_wellwall": dict(kind="brush", seed=12, run_seed=57, steps=600,
                          spec=systems.BrushSpec(n_graft=4, chain_len=8, lxy=10.0, height=12.0,
                                                 n_sites=0, charge_frac=0.6),
                          over=dict(ext_kind="WellWall", well_width=2.0, well_depth=-0.7,
                                    wall_radii=(("P", 0.5), ("L", 0.0), ("C", 0.5)))),
    # the 1,000-particle bulk polyelectrolyte at its own size (10 x 50 chains,
    # 500 counterions, L = 40, alpha = (5/L)^2) with the reference's own Ewald
    # rule: real cut-off 28 > L/2 (several image cells per pair) and 460
    # k-vectors; the generator seed is the one the benchmark workload uses
    "bulk_1000": dict(kind="bulk", seed=20261203, run_seed=12345, steps=400, kinds=True,
                      spec=systems.CONFIGS["bulk_1000"]),
    # the smallest replica of the 256-replica confined-brush ensemble
    # (systems.brush_ensemble(256, 20261203); its index is stored as
    # ref.npz["ensemble"][2]) at full size: 16 grafted chains of 26 beads,
    # 64 LJ surface sites per wall, 9-3 walls, slab Ewald with the dipole
    # correction
    "brush_ens_smallest": dict(kind="brush", seed=None, run_seed=4321, steps=300, kinds=True,
                               spec=None, ensemble=(256, 20261203)),
}


def ensemble_member(n, seed, pick="smallest"):
    """(index, spec, generator seed) of one replica of the confined-brush
    ensemble, the seed as the benchmark writes it (seed + index)."""
    specs = systems.brush_ensemble(n, seed)
    size = [s.n_graft * s.chain_len * (1.0 + s.charge_frac) for s in specs]
    i = int(np.argmin(size)) if pick == "smallest" else int(pick)
    return i, specs[i], seed + i


CBMC_CASES = {
    "muvt_neutral": dict(seed=21, spec=systems.MuVTSpec(box=14.0, n_chain=4, chain_len=10,
                                                         n_salt=30, trials=8)),
    "muvt_charged": dict(seed=22, spec=systems.MuVTSpec(box=14.0, n_chain=3, chain_len=6,
                                                         bead_charge=-1.0, n_salt=12, trials=8)),
}


def make_cbmc_case(name, cfg, n_eval=24):
    """BeadsEnergy (cbmc.cc:5-151) of seeded trial sites: inserting (growing
    a chain from a random first bead) and deleting (regrowing an existing
    chain), from the reference itself."""
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    spec = cfg["spec"]
    systems.write_muvt(d, spec, seed=cfg["seed"])
    R = ob.Ref(d, seed=1)
    L, qb, trials, _ = R.gc_info()
    L = int(L)
    charged = qb != 0
    rng = np.random.default_rng(cfg["seed"] + 7)
    sizes = np.array([R.mol_size(m) for m in range(R.n_mol)])
    start = np.concatenate([[0], np.cumsum(sizes)])
    coords = R.coords()
    chain_mols = [m for m in range(R.n_mol) if sizes[m] > 1]
    rows = []
    for k in range(n_eval):
        if k % 2 == 0:
            delete_id = -1
            cl = int(rng.integers(0, L))
            first = rng.uniform(0, spec.box, size=3)
            steps = rng.normal(size=(max(cl, 1), 3))
            steps /= np.linalg.norm(steps, axis=1)[:, None]
            chain = first + np.cumsum(np.vstack([[0, 0, 0], steps[:max(cl - 1, 0)]]), axis=0)[:cl]
            chain_ci = rng.uniform(0, spec.box, size=(cl, 3))
        else:
            delete_id = int(chain_mols[rng.integers(len(chain_mols))])
            cl = int(rng.integers(0, L))
            chain = coords[start[delete_id]:start[delete_id] + cl]
            chain_ci = np.array([coords[start[delete_id + 1 + i]] for i in range(cl)]) \
                if charged else np.zeros((cl, 3))
        base = chain[-1] if cl > 0 else rng.uniform(0, spec.box, size=3)
        v = rng.normal(size=3)
        b1 = base + 1.0 * v / np.linalg.norm(v)
        b2 = rng.uniform(0, spec.box, size=3)
        u = R.beads_energy(b1, b2 if charged else None, chain if cl else None,
                           chain_ci if (charged and cl) else None, delete_id)
        rows.append((delete_id, cl, b1, b2, chain, chain_ci, u))
    R.close()
    for f in os.listdir(d):
        if f not in ("run.in", "input_crd.dat", "input_top.dat"):
            os.remove(os.path.join(d, f))
    out = {"delete_id": np.array([r[0] for r in rows], np.int32),
           "cl": np.array([r[1] for r in rows], np.int32),
           "b1": np.array([r[2] for r in rows]), "b2": np.array([r[3] for r in rows]),
           "chain": np.concatenate([np.asarray(r[4]).reshape(-1, 3) for r in rows]),
           "chain_ci": np.concatenate([np.asarray(r[5]).reshape(-1, 3) for r in rows]),
           "u": np.array([r[6] for r in rows]), "charged": np.array(int(charged)),
           "gc_len": np.array(L)}
    np.savez_compressed(os.path.join(d, "cbmc.npz"), **out)
    print(name, "beads", int(start[-1]), "u range", out["u"].min(), out["u"].max())


def coarse_rhoz(rz, width=50):
    """rho(z) [n_bins, 3] at 0.02 resolution averaged over groups of `width`
    bins (1 sigma); a ragged last group is dropped."""
    n = (len(rz) // width) * width
    return rz[:n].reshape(-1, width, 3).mean(axis=1)


# the wall-force pressure (pressure.cc:404-488) of a slit with charged wall
# sites, so that its Ewald columns are not zero: the reference's p_tensor
# after evaluations at three configurations (the start, then after `steps` and
# 2 `steps` steps), with those configurations
PRESSURE_CASE = dict(name="slab_charged_sites", seed=13, run_seed=61, steps=300,
                     spec=systems.BrushSpec(n_graft=4, chain_len=8, lxy=10.0, height=12.0,
                                            n_sites=8, wall_cut=2.5, charge_frac=0.6,
                                            site_charge=0.5))


def make_pressure_case(cfg=PRESSURE_CASE):
    d = os.path.join(HERE, cfg["name"])
    if os.path.isdir(d):
        shutil.rmtree(d)
    systems.write_brush(d, cfg["spec"], seed=cfg["seed"])
    R = ob.Ref(d, seed=cfg["run_seed"])
    coords, pt = [], []
    for k in range(3):
        if k:
            R.run(cfg["steps"])
        coords.append(R.coords())
        pt.append(R.pressure_force_slit())
    R.close()
    for f in os.listdir(d):
        if f not in ("run.in", "input_crd.dat", "input_top.dat"):
            os.remove(os.path.join(d, f))
    np.savez_compressed(os.path.join(d, "pressure.npz"), coords=np.array(coords),
                        p_tensor=np.array(pt), steps=np.array(cfg["steps"]),
                        run_seed=np.array(cfg["run_seed"]))
    print(cfg["name"], "p_tensor[9:12]", np.array(pt)[:, 9:12])


LONG_CASES = {"bulk_small": 2024, "slab_wca": 2025}


def make_long_case(name, seed, steps=100000, every=100):
    """A 1e5-step seeded run of the reference's step loop on an existing
    case's inputs: long.npz with the move-type, accept and draw-count
    sequences, the running total after every `every` steps, samples of the
    observables (Rg^2 averaged over chains, end-to-end^2) and of rho(z)
    (averaged into 1-sigma bins, coarse_rhoz) at the same points, the final
    full-resolution rho(z) and the final coordinates. Sampling between chunks of
    the loop reads the state only, so the sequences are those of one run."""
    import tempfile
    src = os.path.join(HERE, name)
    with tempfile.TemporaryDirectory() as d:
        for f in ("run.in", "input_crd.dat", "input_top.dat"):
            shutil.copy(os.path.join(src, f), os.path.join(d, f))
        R = ob.Ref(d, seed=seed)
        mts, acs, drs, ets, obs, rz = [], [], [], [], [], []
        for _ in range(steps // every):
            mt, ac, dr, et = R.run(every)
            mts.append(mt)
            acs.append(ac)
            drs.append(dr)
            ets.append(et[-1])
            obs.append(R.observables())
            rz.append(coarse_rhoz(R.rhoz()))
        out = {"run_seed": np.array(seed), "every": np.array(every),
               "run_type": np.concatenate(mts).astype(np.int8),
               "run_accept": np.concatenate(acs).astype(np.int8),
               "run_draws": np.concatenate(drs).astype(np.uint16),
               "run_etot_sampled": np.array(ets), "run_obs_sampled": np.array(obs),
               "run_rhoz_coarse": np.array(rz).astype(np.float32),
               "run_rhoz": R.rhoz(), "run_coords": R.coords()}
        R.close()
    np.savez_compressed(os.path.join(src, "long.npz"), **out)
    print(name, "long run accept", out["run_accept"].mean())


GC_CASES = {
    "gcx_neutral": dict(seed=31, run_seed=5, steps=400, over={},
                        spec=systems.MuVTSpec(box=12.0, n_chain=4, chain_len=6, n_salt=15,
                                              trials=8, chem_pot=2.0, salt_first=True)),
    # rigid bonds: with the spring potential on, the reference's per-molecule
    # bond energy arrays gain one entry per inserted chain while a charged
    # species adds 1 + L molecules (potential_bond.cc:29-41), so its later
    # bookkeeping reads past their end
    "gcx_charged": dict(seed=32, run_seed=5, steps=400, over={"use_bond": False},
                        spec=systems.MuVTSpec(box=12.0, n_chain=3, chain_len=4, bead_charge=-1.0,
                                              n_salt=8, trials=8, chem_pot=2.0,
                                              salt_first=True)),
}


def _gc_run(name):
    """One reference run with grand-canonical exchanges (a fresh worker
    process: the reference keeps gasdev's cached deviate in statics)."""
    import tempfile
    cfg = GC_CASES[name]
    src = os.path.join(HERE, name)
    with tempfile.TemporaryDirectory() as d:
        for f in ("run.in", "input_crd.dat", "input_top.dat"):
            shutil.copy(os.path.join(src, f), os.path.join(d, f))
        R = ob.Ref(d, seed=cfg["run_seed"])
        mt, ac, dr, et = R.run(cfg["steps"])
        out = dict(run_seed=np.array(cfg["run_seed"]), run_type=mt.astype(np.int8),
                   run_accept=ac.astype(np.int8), run_draws=dr.astype(np.int32), run_etot=et,
                   run_coords=R.coords(), run_n_mol=np.array(R.L.pr_n_mol(R.h)))
        R.close()
    return out


def make_gc_cases():
    """Grand-canonical runs (Simulation::GCMove with configurational-bias
    insertion and deletion) of the reference: gc.npz with the move-type,
    accept and draw-count sequences, running totals and final coordinates."""
    import multiprocessing as mp
    for name, cfg in GC_CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        systems.write_muvt(d, cfg["spec"], seed=cfg["seed"], **cfg["over"])
    with mp.get_context("spawn").Pool(len(GC_CASES)) as pool:
        res = pool.map(_gc_run, list(GC_CASES))
    for name, out in zip(GC_CASES, res):
        np.savez_compressed(os.path.join(HERE, name, "gc.npz"), **out)
        mt, ac = out["run_type"], out["run_accept"]
        print(name, "exchanges", int((mt >= 5).sum()), "accepted", int(ac[mt >= 5].sum()),
              "molecules", int(out["run_n_mol"]))


STAT_CASES = {
    "stat_bulk": dict(kind="bulk", seed=11,
                      spec=systems.BulkSpec(n_chain=2, chain_len=10, n_ion=20, box=9.0)),
    "stat_slab": dict(kind="brush", seed=12,
                      spec=systems.BrushSpec(n_graft=3, chain_len=6, lxy=8.0, height=10.0,
                                             n_sites=4, wall_cut=-1.0, charge_frac=0.7)),
}
STAT_SEEDS = [101, 102, 103, 104, 105, 106, 107, 108]
STAT_STEPS, STAT_EVERY, STAT_BURN = 60000, 100, 10000


def _stat_run(args):
    """One seeded reference run of a statistics case (a worker process)."""
    name, seed = args
    import tempfile
    src = os.path.join(HERE, name)
    with tempfile.TemporaryDirectory() as d:
        for f in ("run.in", "input_crd.dat", "input_top.dat"):
            shutil.copy(os.path.join(src, f), os.path.join(d, f))
        R = ob.Ref(d, seed=seed)
        E, G, Z = [], [], []
        for k in range(STAT_STEPS // STAT_EVERY):
            _, _, _, et = R.run(STAT_EVERY)
            E.append(et[-1])
            G.append(R.observables()[0])
            if (k + 1) * STAT_EVERY > STAT_BURN:
                Z.append(coarse_rhoz(R.rhoz()))
        R.close()
    return np.array(E), np.array(G), np.mean(Z, axis=0)


def make_stat_cases(workers=8):
    """Equilibrium statistics of the reference: 8 independently seeded runs
    of STAT_STEPS steps per case, sampled every STAT_EVERY steps (total
    energy, chain-averaged Rg^2) and, after STAT_BURN steps, rho(z) averaged
    per run in 1-sigma bins. stats.npz holds the series and per-run means."""
    import multiprocessing as mp
    for name, cfg in STAT_CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        if cfg["kind"] == "bulk":
            systems.write_bulk(d, cfg["spec"], seed=cfg["seed"])
        else:
            systems.write_brush(d, cfg["spec"], seed=cfg["seed"])
    tasks = [(name, s) for name in STAT_CASES for s in STAT_SEEDS]
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_stat_run, tasks)
    for name in STAT_CASES:
        rows = [r for (n, _), r in zip(tasks, res) if n == name]
        np.savez_compressed(os.path.join(HERE, name, "stats.npz"),
                            seeds=np.array(STAT_SEEDS), steps=np.array(STAT_STEPS),
                            every=np.array(STAT_EVERY), burn=np.array(STAT_BURN),
                            energy=np.array([r[0] for r in rows]),
                            rg2=np.array([r[1] for r in rows]),
                            rhoz=np.array([r[2] for r in rows]))
        print(name, "runs", len(rows))


def make_case(name, cfg, n_de=24):
    import time
    t0 = time.time()
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    spec, seed = cfg["spec"], cfg["seed"]
    out = {}
    if cfg.get("ensemble"):
        idx, spec, seed = ensemble_member(*cfg["ensemble"])
        out["ensemble"] = np.array([cfg["ensemble"][0], cfg["ensemble"][1], idx])
    if cfg["kind"] == "bulk":
        systems.write_bulk(d, spec, seed=seed, **cfg.get("over", {}))
    else:
        systems.write_brush(d, spec, seed=seed, **cfg.get("over", {}))
    R = ob.Ref(d, seed=cfg["run_seed"])
    out["energies"] = R.energies()
    out["ewald"] = R.ewald_info()
    sizes = np.array([R.mol_size(m) for m in range(R.n_mol)])
    start = np.concatenate([[0], np.cumsum(sizes)])
    rng = np.random.default_rng(seed + 1000)
    c = R.coords()
    mols, trials, moveds, outs = [], [], [], []
    movable = [m for m in range(R.n_mol) if sizes[m] > 1] + \
              [m for m in range(R.n_mol) if sizes[m] == 1][-20:]
    for k in range(n_de):
        m = int(movable[rng.integers(len(movable))])
        cur = c[start[m]:start[m + 1]]
        n = sizes[m]
        moved = np.zeros(n, np.int32)
        if n == 1:
            moved[:] = 1
        else:
            lo = int(rng.integers(0, n))
            hi = int(rng.integers(lo + 1, n + 1))
            moved[lo:hi] = 1
        trial = cur + moved[:, None] * rng.normal(scale=0.25, size=cur.shape)
        mols.append(m)
        trials.append(trial)
        moveds.append(moved)
        outs.append(R.delta_energy(m, trial, moved))
    kinds = [-1] * len(mols)
    if cfg.get("kinds"):
        first = spec.n_sites * 2 if cfg["kind"] == "brush" else 0
        for kind, m, trial, moved in kind_trials(c, start, sizes, rng, move_size=spec.move_size,
                                                 bond=spec.r0, first_mol=first):
            kinds.append(kind)
            mols.append(m)
            trials.append(trial)
            moveds.append(moved)
            outs.append(R.delta_energy(m, trial, moved))
    # When the pair (or pair + external) change reaches 1e8 the reference
    # returns before the Ewald part (force_field.cc:411-422), so the Ewald
    # potential's dE member still holds the previous call's value: the
    # component is recorded as 0, the change the early return adds. (The
    # bond and Ewald terms cannot lift a total below 1e8 to it.)
    outs = [np.array([o[0], o[1], 0.0 if o[0] >= 1e8 else o[2]]) for o in outs]
    out["de_kind"] = np.array(kinds, np.int32)
    out["de_mol"] = np.array(mols, np.int32)
    out["de_start"] = start.astype(np.int32)
    out["de_trial"] = np.concatenate(trials)
    out["de_moved"] = np.concatenate(moveds)
    out["de_out"] = np.array(outs)
    out["rng_words"] = R.rng_words(4000)
    out["run_seed"] = np.array(cfg["run_seed"])
    mt, ac, dr, et = R.run(cfg["steps"])
    out["run_type"], out["run_accept"], out["run_draws"], out["run_etot"] = mt, ac, dr, et
    out["run_coords"] = R.coords()
    out["run_obs"] = R.observables()
    out["run_rhoz"] = R.rhoz()
    out["run_recompute"] = R.recompute()
    R.close()
    for f in os.listdir(d):
        if f not in ("run.in", "input_crd.dat", "input_top.dat"):
            os.remove(os.path.join(d, f))
    np.savez_compressed(os.path.join(d, "ref.npz"), **out)
    print(name, "beads", int(start[-1]), "accept", ac.mean(), "types", np.bincount(mt + 1),
          "%.0f s" % (time.time() - t0))


# Output files: the reference's Simulation::Run with sampling and writing on
# an existing case's inputs, run.in items 4-8 replaced (steps, equilibration
# steps, sampling / stat / trajectory frequencies).
OUTPUT_CASES = {"outputs_bulk_small": dict(src="bulk_small", seed=77, steps=3000, steps_eq=1000,
                                           sample_freq=10, stat_freq=500, traj_freq=1000),
                # walls, dipole, grafted chains and charged surface sites: the stat
                # file carries the wall-force pressure (its LJ columns are
                # undefined in the reference: PairForce reads an uninitialised
                # local, potential_truncated_lj.cc:95-100)
                "outputs_slab_charged_sites": dict(src="slab_charged_sites", seed=61, steps=2000,
                                                   steps_eq=500, sample_freq=10, stat_freq=500,
                                                   traj_freq=1000),
                # grand-canonical exchange of a charged species: the stat file's
                # molecule count, density and exchange acceptance columns
                "outputs_gcx_charged": dict(src="gcx_charged", seed=5, steps=1200, steps_eq=200,
                                            sample_freq=10, stat_freq=400, traj_freq=600)}
OUTPUT_FILES = ("out_stat.dat", "out_traj_p.xyz", "out_traj_c.xyz", "out_traj_a.xyz",
                "out_traj_n.xyz", "out_lastcrd.dat", "out_lastcrd.dat2", "out_lasttop.dat",
                "out_lastrhoZ.dat", "out_lastrhoZ.dat2")


def output_runin(src_runin, cfg):
    """The case's run.in with the run name "out" and the run-control items
    of the output case (lines 3-8 of the positional grammar)."""
    lines = open(src_runin).read().splitlines()
    keys = {2: "out", 3: cfg["steps"], 4: cfg["steps_eq"], 5: cfg["sample_freq"],
            6: cfg["stat_freq"], 7: cfg["traj_freq"]}
    for i, v in keys.items():
        flag = lines[i].split()[0]
        lines[i] = "%s %s" % (flag, v)
    return "\n".join(lines) + "\n"


def make_output_cases(only=None):
    import tempfile
    for name, cfg in OUTPUT_CASES.items():
        if only and name not in only:
            continue
        src = os.path.join(HERE, cfg["src"])
        dst = os.path.join(HERE, name)
        os.makedirs(dst, exist_ok=True)
        with open(os.path.join(dst, "run.in"), "w") as f:
            f.write(output_runin(os.path.join(src, "run.in"), cfg))
        with tempfile.TemporaryDirectory() as d:
            for f in ("input_crd.dat", "input_top.dat"):
                shutil.copy(os.path.join(src, f), os.path.join(d, f))
            shutil.copy(os.path.join(dst, "run.in"), os.path.join(d, "run.in"))
            R = ob.Ref(d, seed=cfg["seed"])
            R.run_full()
            coords = R.coords()
            R.close()  # the destructor's last writes
            for f in OUTPUT_FILES:
                shutil.copy(os.path.join(d, f), os.path.join(dst, f))
            # the sampling (and the pressure routine it calls every tenth
            # sample) must leave the trajectory alone: the plain step loop
            # from the same seed ends in the same coordinates
            P = ob.Ref(d, seed=cfg["seed"])
            P.run(cfg["steps"])
            assert np.array_equal(P.coords(), coords), "sampling changed the trajectory"
            P.close()
        print(name, "written:", ", ".join(OUTPUT_FILES))


if __name__ == "__main__":
    ob.build()
    which = sys.argv[1:] or ["moves", "cbmc"]
    if "moves" in which:
        for name, cfg in CASES.items():
            make_case(name, cfg)
    for name, cfg in CASES.items():
        if "case:" + name in which:
            make_case(name, cfg)
    if "cbmc" in which:
        for name, cfg in CBMC_CASES.items():
            make_cbmc_case(name, cfg)
    for name, seed in LONG_CASES.items():
        if "long" in which or "long:" + name in which:
            make_long_case(name, seed)
    if "stats" in which:
        make_stat_cases()
    if "gc" in which:
        make_gc_cases()
    if "outputs" in which:
        make_output_cases()
    picked = [w.split(":", 1)[1] for w in which if w.startswith("outputs:")]
    if picked:
        make_output_cases(picked)
    if "pressure" in which:
        make_pressure_case()
