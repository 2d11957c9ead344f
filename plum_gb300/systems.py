"""Seeded synthetic systems written in the reference's own input formats.

The reference (nuwapi/Plum) reads a positional ``run.in`` on stdin
(simulation.cc:30-50, force_field.cc:64-195 and the potentials'
ReadParameters), a coordinate file (simulation.cc:582-608: two header lines,
then ``mol_id symbol x y z q`` rows) and a topology file (simulation.cc:610-646).
This module writes exactly those three files, so the same inputs drive the
reference, the CPU oracle and this package.

Workloads (all seeded):

* ``bulk_nvt``: linear chains of charged beads (symbol ``P``) plus monovalent
  counterions (``C``) in a periodic cube. Chains are self-avoiding random
  walks with bond length 1 sigma and no two beads closer than 0.8 sigma;
  ions are uniform with the same exclusion.
* ``brush``: one confined replica: end-grafted chains (first bead ``L`` near
  z=0), counterions, random LJ surface sites (phantom molecules ``S``) between
  walls at z=0 and z=H, periodic in x and y.

A trailing extension block (keys prefixed ``plum_``) can pin the Ewald
real-space cutoff and the k-vector range. The reference never reads past its
last potential block, so such files stay valid reference inputs.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional

import numpy as np


@dataclasses.dataclass
class BulkSpec:
    n_chain: int = 10
    chain_len: int = 50
    n_ion: int = 500          # +1 counterions
    box: float = 40.0
    bead_charge: float = -1.0
    lj_cutoff: float = 2.5
    lj_sigma: float = 1.0
    lj_eps: float = 1.0
    lB: float = 3.0
    alpha_times_L: float = 5.0  # alpha (reference units, ul^-2) = (alpha_times_L / L)^2
    k_bond: float = 400.0
    r0: float = 1.0
    move_size: float = 1.0
    move_prob: tuple = (0.3, 0.1, 0.2, 0.2, 0.2)  # bead, COM, pivot, crank, reptation
    steps: int = 100000
    # None keeps the reference's automatic Ewald rule (potential_ewald_coul.cc:56-75)
    real_cutoff: Optional[float] = None
    kmax: Optional[int] = None
    kcut2: Optional[float] = None
    use_ewald: bool = True
    use_bond: bool = True
    min_sep: float = 0.8


# Named workloads. Ewald parameters follow the reference's automatic rule
# unless a workload pins them (the "r_c = L/2, |n| <= kmax" form).
CONFIGS = {
    # 10 x 50 chains + 500 ions, L = 40, alpha = (5/L)^2
    "bulk_1000": BulkSpec(),
    # same system with the Ewald parameters pinned to r_c = L/2, |n| <= 7
    "bulk_1000_pinned": BulkSpec(real_cutoff=20.0, kmax=7, kcut2=-1.0),
    # 100 x 100 chains + 10000 ions, L = 80, alpha = (5.6/L)^2
    "bulk_20000": BulkSpec(n_chain=100, chain_len=100, n_ion=10000, box=80.0,
                           alpha_times_L=5.6),
    # same system with r_c = L/2 and |n| <= 12
    "bulk_20000_pinned": BulkSpec(n_chain=100, chain_len=100, n_ion=10000, box=80.0,
                                  alpha_times_L=5.6, real_cutoff=40.0, kmax=12,
                                  kcut2=-1.0),
}


class _Grid:
    """Cell list for overlap rejection while placing beads."""

    def __init__(self, box, cell):
        self.box = np.asarray(box, dtype=np.float64)
        self.nc = np.maximum(1, np.floor(self.box / cell).astype(int))
        self.cell = self.box / self.nc
        self.cells = {}

    def _key(self, p):
        w = p - self.box * np.floor(p / self.box)
        return tuple((np.floor(w / self.cell).astype(int)) % self.nc)

    def ok(self, p, r, periodic):
        k = self._key(p)
        r2 = r * r
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    kk = ((k[0] + dx) % self.nc[0], (k[1] + dy) % self.nc[1],
                          (k[2] + dz) % self.nc[2])
                    for q in self.cells.get(kk, ()):
                        d = q - p
                        for a in range(3):
                            if periodic[a]:
                                d[a] -= self.box[a] * round(d[a] / self.box[a])
                        if d @ d < r2:
                            return False
        return True

    def add(self, p):
        self.cells.setdefault(self._key(p), []).append(np.array(p, dtype=np.float64))


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def bulk_coordinates(spec: BulkSpec, seed: int):
    """Seeded self-avoiding chains followed by counterions.

    Returns (mol_ids, symbols, xyz[n,3], q[n]) in file order: chain beads first
    (molecule by molecule), then one molecule per ion."""
    rng = np.random.default_rng(seed)
    L = spec.box
    box = np.array([L, L, L])
    grid = _Grid(box, max(spec.min_sep, 1.0))
    per = (True, True, True)
    mol, sym, xyz, q = [], [], [], []
    for c in range(spec.n_chain):
        for attempt in range(1000):
            beads = []
            p = rng.uniform(0, L, size=3)
            if not grid.ok(p, spec.min_sep, per):
                continue
            beads.append(p)
            local = _Grid(box, max(spec.min_sep, 1.0))
            local.add(p)
            okc = True
            for b in range(1, spec.chain_len):
                for t in range(200):
                    cand = beads[-1] + spec.r0 * _unit(rng)
                    if grid.ok(cand, spec.min_sep, per) and local.ok(cand, spec.min_sep, per):
                        break
                else:
                    okc = False
                    break
                beads.append(cand)
                local.add(cand)
            if okc:
                break
        else:
            raise RuntimeError("could not grow chain %d" % c)
        for p in beads:
            grid.add(p)
            mol.append(c)
            sym.append("P")
            xyz.append(p)
            q.append(spec.bead_charge)
    for i in range(spec.n_ion):
        for t in range(100000):
            p = rng.uniform(0, L, size=3)
            if grid.ok(p, spec.min_sep, per):
                break
        else:
            raise RuntimeError("could not place ion %d" % i)
        grid.add(p)
        mol.append(spec.n_chain + i)
        sym.append("C")
        xyz.append(p)
        q.append(+1.0)
    return np.array(mol), sym, np.array(xyz), np.array(q, dtype=np.float64)


def write_crd(path, mol, sym, xyz, q):
    with open(path, "w") as f:
        f.write("%d\n \n" % len(mol))
        for m, s, p, c in zip(mol, sym, xyz, q):
            f.write("%d %s %.17g %.17g %.17g %g\n" % (m, s, p[0], p[1], p[2], c))


def write_top(path, n_bead, n_mol, box, bonds=()):
    with open(path, "w") as f:
        f.write("TotNoOfBeads: %d\nTotNoOfMolec: %d\n" % (n_bead, n_mol))
        for a, L in zip("XYZ", box):
            f.write("Box_Length_%s: %.17g\n" % (a, L))
        f.write("bonds:\n")
        for m, i, j in bonds:
            f.write("%d %d %d\n" % (m, i, j))
        f.write("-1\nangles:\n-1\ndiheds\n-1\n")


def runin_text(*, crd="input_crd.dat", top="input_top.dat", run_name="output",
               steps=1000, steps_eq=0, sample_freq=10**9, npbc=3, beta=1.0,
               move_size=1.0, phantom=0, coion=0, grafted=0, grafted_counterion=0,
               move_prob=(0.3, 0.1, 0.2, 0.2, 0.2), use_pair=True, lj_cutoff=2.5,
               lj_table=(("P", 1.0, 1.0), ("C", 1.0, 1.0)), use_ewald=True, lB=3.0,
               alpha=0.015625, dipole=False, use_bond=True, k_bond=400.0, r0=1.0,
               use_rigid=True, rigid=1.0, use_ext=False, wall_cut=-1.0,
               wall_table=(), use_gc=False, gc=None, real_cutoff=None, kmax=None,
               kcut2=None, pair_kind="TruncatedLJ", hs_radii=(), ext_kind="TruncatedLJWall",
               wall_radii=(), well_width=1.0, well_depth=-1.0) -> str:
    """A run.in in the reference's positional grammar. pair_kind
    "HardSphere" reads hs_radii ((symbol, radius), ...) instead of the LJ
    table (potential_hard_sphere.cc:20-36); ext_kind "HardWall" / "WellWall"
    read wall_radii (and the well's width and depth) instead of the 9-3 wall
    table (potential_hard_wall.cc:15-33, potential_well_wall.cc:15-40)."""
    L = []
    a = L.append
    a("s1_input_coordinate_file %s" % crd)
    a("s1_input_topology_file %s" % top)
    a("s1_prefix_of_output_file_names %s" % run_name)
    a("s1_total_simulation_steps %d" % steps)
    a("s1_equilibrium_steps %d" % steps_eq)
    a("s1_sampling_frequency %d" % sample_freq)
    a("s1_sampling_print_frequency %d" % sample_freq)
    a("s1_trajectory_print_frequency %d" % sample_freq)
    a("s1_PBC_dimensions %d" % npbc)
    a("s1_beta %.17g" % beta)
    a("s1_MC_move_size %.17g" % move_size)
    a("s1_calc_chem_pot 0")
    a("s1_number_of_surface_sites %d" % phantom)
    a("s1_number_of_surf_counterions %d" % coion)
    a("s1_number_of_grafted_chains %d" % grafted)
    a("s1_number_of_grafted_counterion %d" % grafted_counterion)
    for name, p in zip(("bead_translation", "COM_translation", "pivot", "crankshaft",
                        "random_reptation"), move_prob):
        a("s1_prob_%s %.17g" % (name, p))
    a("s1_vp_bin_resolution_in_ul 10")
    a("s1_bead_size_virial_pressure 1")
    a("s2_use_short_range_potential %d" % int(use_pair))
    a("s2_use_Ewald_potential %d" % int(use_ewald))
    a("s2_use_bond_potential %d" % int(use_bond))
    a("s2_use_rigid_bond %d" % int(use_rigid))
    a("s2_use_angle_potential 0")
    a("s2_use_dihedral_potential 0")
    a("s2_use_external_potential %d" % int(use_ext))
    a("s2_use_grand_canonical_MC_move %d" % int(use_gc))
    if use_gc:
        for k in ("chem_pot", "deBroglie", "gc_freq", "chain_len", "bead_charge",
                  "bead_symbol", "cbmc_trials"):
            a("s3_gc_%s %s" % (k, gc[k]))
    if use_pair and pair_kind == "HardSphere":
        a("s3_short_range_potential_type HardSphere")
        for i, (s, rad) in enumerate(hs_radii):
            a("s3_bead_type_%d %s" % (i + 1, s))
            a("s3_radius_for_bead_type_%d %.17g" % (i + 1, rad))
        a("s3_end_flag end")
    elif use_pair:
        a("s3_short_range_potential_type TruncatedLJ")
        a("s3_LJ_cutoff %.17g" % lj_cutoff)
        for i, (s, sg, ep) in enumerate(lj_table):
            a("s3_bead_type_%d %s" % (i + 1, s))
            a("s3_sigma_for_bead_type_%d %.17g" % (i + 1, sg))
            a("s3_epsilon_for_bead_type_%d %.17g" % (i + 1, ep))
        a("s3_end_flag end")
    if use_ewald:
        a("s3_Ewald_potential_type Coul")
        a("s3_Bjerrum_length %.17g" % lB)
        a("s3_dielectric_constant 80")
        a("s3_Ewald_alpha %.17g" % alpha)
        a("s3_use_dipole_correction %d" % int(dipole))
    if use_bond:
        a("s3_bond_potential_type Spring")
        a("s3_spring_constant %.17g" % k_bond)
        a("s3_equilibrium_length %.17g" % r0)
    if use_rigid:
        a("s3_rigid_bond_length %.17g" % rigid)
    if use_ext and ext_kind in ("HardWall", "WellWall"):
        a("s3_external_potential_type %s" % ext_kind)
        if ext_kind == "WellWall":
            a("s3_well_width %.17g" % well_width)
            a("s3_well_depth %.17g" % well_depth)
        for i, (s, rad) in enumerate(wall_radii):
            a("s3_bead_type_%d %s" % (i + 1, s))
            a("s3_radius_for_bead_type_%d %.17g" % (i + 1, rad))
        a("s3_end_flag end")
    elif use_ext:
        a("s3_external_potential_type TruncatedLJWall")
        a("s3_LJ_cutoff %.17g" % wall_cut)
        a("s3_wall_sigma 1")
        a("s3_wall_epsilon 1")
        for i, (s, sg, ep) in enumerate(wall_table):
            a("s3_bead_type_%d %s" % (i + 1, s))
            a("s3_sigma_for_bead_type_%d %.17g" % (i + 1, sg))
            a("s3_epsilon_for_bead_type_%d %.17g" % (i + 1, ep))
        a("s3_end_flag end")
    if real_cutoff is not None:
        a("plum_ewald_real_cutoff %.17g" % real_cutoff)
    if kmax is not None:
        a("plum_ewald_kmax %d" % kmax)
    if kcut2 is not None:
        a("plum_ewald_kcut2 %.17g" % kcut2)
    return "\n".join(L) + "\n"


def write_bulk(dirpath: str, spec: BulkSpec, seed: int, runin="run.in", **over) -> str:
    """Writes run.in, input_crd.dat and input_top.dat for a bulk system.

    Returns the run.in path."""
    os.makedirs(dirpath, exist_ok=True)
    mol, sym, xyz, q = bulk_coordinates(spec, seed)
    n_mol = spec.n_chain + spec.n_ion
    write_crd(os.path.join(dirpath, "input_crd.dat"), mol, sym, xyz, q)
    write_top(os.path.join(dirpath, "input_top.dat"), len(mol), n_mol,
              (spec.box, spec.box, spec.box))
    kw = dict(steps=spec.steps, move_size=spec.move_size, move_prob=spec.move_prob,
              lj_cutoff=spec.lj_cutoff,
              lj_table=(("P", spec.lj_sigma, spec.lj_eps), ("C", spec.lj_sigma, spec.lj_eps)),
              use_ewald=spec.use_ewald, lB=spec.lB,
              alpha=(spec.alpha_times_L / spec.box) ** 2, use_bond=spec.use_bond,
              k_bond=spec.k_bond, r0=spec.r0, rigid=spec.r0,
              real_cutoff=spec.real_cutoff, kmax=spec.kmax, kcut2=spec.kcut2)
    kw.update(over)
    with open(os.path.join(dirpath, runin), "w") as f:
        f.write(runin_text(**kw))
    return os.path.join(dirpath, runin)


@dataclasses.dataclass
class BrushSpec:
    """One confined replica: end-grafted chains between walls at z=0 and z=H."""
    n_graft: int = 16
    chain_len: int = 20
    lxy: float = 32.0
    height: float = 40.0
    charge_frac: float = 0.5     # probability that a chain bead carries -1
    n_sites: int = 64            # LJ surface sites per wall (phantom molecules)
    site_charge: float = 0.0     # sites carry +q, -q, +q, ... along each wall
    graft_z: float = 1.0
    wall_cut: float = -1.0       # <0: purely repulsive 9-3 wall
    lj_cutoff: float = 2.5
    lB: float = 3.0
    alpha_times_L: float = 5.0   # alpha = (alpha_times_L / lxy)^2
    k_bond: float = 400.0
    r0: float = 1.0
    move_size: float = 1.0
    move_prob: tuple = (0.3, 0.1, 0.2, 0.2, 0.2)
    min_sep: float = 0.8
    real_cutoff: Optional[float] = None
    kmax: Optional[int] = None
    kcut2: Optional[float] = None


def brush_ensemble(n: int, seed: int):
    """n confined brush replicas of uneven size: wall gap H uniform in
    [30, 60] sigma, Lx = Ly = 32 sigma, grafted chains uniform in {16..64} of
    length uniform in {20..80}, bead charge -1 with probability f, f uniform
    in [0.1, 1], +1 counterions, 64 LJ surface sites per wall and the 9-3
    walls. The slab Ewald box follows the reference's rule (3H when 3H > 150,
    else H + 150; potential_ewald_coul.cc:43-49)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(BrushSpec(n_graft=int(rng.integers(16, 65)),
                             chain_len=int(rng.integers(20, 81)),
                             lxy=32.0, height=float(rng.uniform(30.0, 60.0)),
                             charge_frac=float(rng.uniform(0.1, 1.0)), n_sites=64))
    return out


def brush_coordinates(spec: BrushSpec, seed: int):
    """Phantom surface sites (symbol S, both walls), grafted chains (first bead
    L at z = graft_z), then +1 counterions neutralising the chain charge."""
    rng = np.random.default_rng(seed)
    L, H = spec.lxy, spec.height
    box = np.array([L, L, H])
    per = (True, True, False)
    grid = _Grid(box, max(spec.min_sep, 1.0))
    mol, sym, xyz, q = [], [], [], []
    m = 0
    for w in (0.0, H):
        for i in range(spec.n_sites):
            p = np.array([rng.uniform(0, L), rng.uniform(0, L), w])
            mol.append(m), sym.append("S"), xyz.append(p)
            q.append(spec.site_charge * (1.0 if i % 2 == 0 else -1.0))
            m += 1
    zlo, zhi = spec.min_sep, H - spec.min_sep
    nneg = 0
    for c in range(spec.n_graft):
        for attempt in range(1000):
            p = np.array([rng.uniform(0, L), rng.uniform(0, L), spec.graft_z])
            if not grid.ok(p, spec.min_sep, per):
                continue
            beads = [p]
            local = _Grid(box, max(spec.min_sep, 1.0))
            local.add(p)
            okc = True
            for b in range(1, spec.chain_len):
                for t in range(400):
                    cand = beads[-1] + spec.r0 * _unit(rng)
                    if zlo < cand[2] < zhi and grid.ok(cand, spec.min_sep, per) and \
                            local.ok(cand, spec.min_sep, per):
                        break
                else:
                    okc = False
                    break
                beads.append(cand)
                local.add(cand)
            if okc:
                break
        else:
            raise RuntimeError("could not graft chain %d" % c)
        for b, p in enumerate(beads):
            grid.add(p)
            ch = -1.0 if rng.uniform() < spec.charge_frac else 0.0
            nneg += ch < 0
            mol.append(m), sym.append("L" if b == 0 else "P"), xyz.append(p), q.append(ch)
        m += 1
    for i in range(nneg):
        for t in range(100000):
            p = np.array([rng.uniform(0, L), rng.uniform(0, L), rng.uniform(zlo, zhi)])
            if grid.ok(p, spec.min_sep, per):
                break
        else:
            raise RuntimeError("could not place counterion %d" % i)
        grid.add(p)
        mol.append(m), sym.append("C"), xyz.append(p), q.append(1.0)
        m += 1
    return np.array(mol), sym, np.array(xyz), np.array(q, dtype=np.float64), nneg


def write_brush(dirpath: str, spec: BrushSpec, seed: int, runin="run.in", **over) -> str:
    """Writes run.in, input_crd.dat and input_top.dat for one brush replica."""
    os.makedirs(dirpath, exist_ok=True)
    mol, sym, xyz, q, nneg = brush_coordinates(spec, seed)
    n_mol = int(mol.max()) + 1
    write_crd(os.path.join(dirpath, "input_crd.dat"), mol, sym, xyz, q)
    write_top(os.path.join(dirpath, "input_top.dat"), len(mol), n_mol,
              (spec.lxy, spec.lxy, spec.height))
    lj = (("P", 1.0, 1.0), ("L", 1.0, 1.0), ("C", 1.0, 1.0), ("S", 1.0, 1.0))
    wall = (("P", 1.0, 1.0), ("L", 1.0, 1.0), ("C", 1.0, 1.0), ("S", 1.0, 0.0))
    kw = dict(npbc=2, move_size=spec.move_size, move_prob=spec.move_prob,
              phantom=2 * spec.n_sites, coion=0, grafted=spec.n_graft,
              grafted_counterion=nneg, lj_cutoff=spec.lj_cutoff, lj_table=lj,
              lB=spec.lB, alpha=(spec.alpha_times_L / spec.lxy) ** 2, dipole=True,
              k_bond=spec.k_bond, r0=spec.r0, rigid=spec.r0, use_ext=True,
              wall_cut=spec.wall_cut, wall_table=wall, real_cutoff=spec.real_cutoff,
              kmax=spec.kmax, kcut2=spec.kcut2)
    kw.update(over)
    with open(os.path.join(dirpath, runin), "w") as f:
        f.write(runin_text(**kw))
    return os.path.join(dirpath, runin)


@dataclasses.dataclass
class MuVTSpec:
    """Grand-canonical bulk box: chains of the exchanged species (each
    followed by its counterions when charged) plus fixed +-1 salt pairs."""
    box: float = 50.0
    n_chain: int = 40
    chain_len: int = 30
    bead_charge: float = 0.0     # charge of each chain bead (0: neutral species)
    n_salt: int = 2000           # +1/-1 pairs
    lj_cutoff: float = 2.5
    lB: float = 3.0
    alpha_times_L: float = 5.0
    k_bond: float = 400.0
    r0: float = 1.0
    chem_pot: float = 0.0
    trials: int = 32
    gc_freq: int = 2             # the reference draws insert/delete when rand % gc_freq == 0
    move_prob: tuple = (0.5, 0.1, 0.2, 0.0, 0.2)
    min_sep: float = 0.8
    # Salt before the exchanged chains, declared as the run's "surface
    # counterions" (coion). The reference's deletion indexes the exchanged
    # species as the molecules after phantom + coion + grafted +
    # grafted_counterion (cbmc.cc:340-346) while insertion appends at the end
    # (cbmc.cc:294-312), so any other molecule after the chains is read as a
    # chain once one has been inserted; exchange runs need this layout.
    salt_first: bool = False


def muvt_coordinates(spec: MuVTSpec, seed: int):
    rng = np.random.default_rng(seed)
    L = spec.box
    box = np.array([L, L, L])
    grid = _Grid(box, max(spec.min_sep, 1.0))
    per = (True, True, True)
    mol, sym, xyz, q = [], [], [], []
    m = 0

    def place():
        for t in range(100000):
            p = rng.uniform(0, L, size=3)
            if grid.ok(p, spec.min_sep, per):
                grid.add(p)
                return p
        raise RuntimeError("could not place a bead")

    def salt():
        nonlocal m
        for i in range(spec.n_salt):
            mol.append(m), sym.append("C"), xyz.append(place()), q.append(1.0)
            m += 1
            mol.append(m), sym.append("A"), xyz.append(place()), q.append(-1.0)
            m += 1

    if spec.salt_first:
        salt()
    for c in range(spec.n_chain):
        for attempt in range(1000):
            p = rng.uniform(0, L, size=3)
            if not grid.ok(p, spec.min_sep, per):
                continue
            beads = [p]
            local = _Grid(box, max(spec.min_sep, 1.0))
            local.add(p)
            ok = True
            for b in range(1, spec.chain_len):
                for t in range(200):
                    cand = beads[-1] + spec.r0 * _unit(rng)
                    if grid.ok(cand, spec.min_sep, per) and local.ok(cand, spec.min_sep, per):
                        break
                else:
                    ok = False
                    break
                beads.append(cand)
                local.add(cand)
            if ok:
                break
        else:
            raise RuntimeError("could not grow chain %d" % c)
        for p in beads:
            grid.add(p)
            mol.append(m), sym.append("P"), xyz.append(p), q.append(spec.bead_charge)
        m += 1
        if spec.bead_charge != 0:
            for b in range(spec.chain_len):
                mol.append(m), sym.append("P"), xyz.append(place()), q.append(-spec.bead_charge)
                m += 1
    if not spec.salt_first:
        salt()
    return np.array(mol), sym, np.array(xyz), np.array(q, dtype=np.float64)


def write_muvt(dirpath: str, spec: MuVTSpec, seed: int, runin="run.in", **over) -> str:
    os.makedirs(dirpath, exist_ok=True)
    mol, sym, xyz, q = muvt_coordinates(spec, seed)
    write_crd(os.path.join(dirpath, "input_crd.dat"), mol, sym, xyz, q)
    write_top(os.path.join(dirpath, "input_top.dat"), len(mol), int(mol.max()) + 1,
              (spec.box,) * 3)
    gc = {"chem_pot": spec.chem_pot, "deBroglie": 1, "gc_freq": spec.gc_freq,
          "chain_len": spec.chain_len, "bead_charge": int(spec.bead_charge),
          "bead_symbol": "P", "cbmc_trials": spec.trials}
    kw = dict(move_prob=spec.move_prob, lj_cutoff=spec.lj_cutoff,
              lj_table=(("P", 1.0, 1.0), ("C", 1.0, 1.0), ("A", 1.0, 1.0)), lB=spec.lB,
              alpha=(spec.alpha_times_L / spec.box) ** 2, k_bond=spec.k_bond, r0=spec.r0,
              rigid=spec.r0, use_gc=True, gc=gc,
              coion=2 * spec.n_salt if spec.salt_first else 0)
    kw.update(over)
    with open(os.path.join(dirpath, runin), "w") as f:
        f.write(runin_text(**kw))
    return os.path.join(dirpath, runin)
