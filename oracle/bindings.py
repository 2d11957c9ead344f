"""ctypes bindings for the CPU checkers built by oracle/Makefile.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by
bench.py's CPU-baseline leg. The product package never imports this module.

* ``Ref``    -- the unmodified reference sources linked with ref_harness.cc
               (oracle/_ref/libplumref.so).
* ``Oracle`` -- the project's FP64 CPU restatement (oracle/_ref/liboracle.so).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libplumref.so")
ORACLE_SO = os.path.join(HERE, "_ref", "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


# Where the reference checkout is read from (only to build the checker
# libplumref.so); PLUM_REF_DIR overrides it. Absent on machines that only run
# the prebuilt checkers.
REF_DIR = os.environ.get("PLUM_REF_DIR", "/root/reference")


def build(ref_dir: str = REF_DIR, quiet: bool = True) -> None:
    """Runs oracle/Makefile (the reference part only if its sources exist)."""
    out = subprocess.run(["make", "-C", HERE, "-j4", "REF=%s" % ref_dir],
                         capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (out.stdout, out.stderr))


def have_ref() -> bool:
    return os.path.exists(REF_SO)


_ref_lib = None
_orc_lib = None


def _load_ref():
    global _ref_lib
    if _ref_lib is None:
        L = C.CDLL(REF_SO)
        L.pr_create.restype = C.c_void_p
        L.pr_create.argtypes = [C.c_char_p, C.c_char_p, C.c_uint]
        L.pr_destroy.argtypes = [C.c_void_p]
        for f in ("pr_n_mol", "pr_n_bead"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int
        L.pr_mol_size.argtypes = [C.c_void_p, C.c_int]
        L.pr_mol_size.restype = C.c_int
        L.pr_energies.argtypes = [C.c_void_p, _dp]
        L.pr_coords.argtypes = [C.c_void_p, _dp]
        L.pr_ewald_info.argtypes = [C.c_void_p, _dp]
        L.pr_pair_terms.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp]
        L.pr_self_energy.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.pr_self_energy.restype = C.c_double
        L.pr_bond_energy.argtypes = [C.c_void_p, C.c_int]
        L.pr_bond_energy.restype = C.c_double
        L.pr_ext_energy.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.pr_ext_energy.restype = C.c_double
        L.pr_dipole_energy.argtypes = [C.c_void_p]
        L.pr_dipole_energy.restype = C.c_double
        L.pr_recompute.argtypes = [C.c_void_p, _dp]
        L.pr_delta_energy.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _dp]
        L.pr_run.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _dp]
        L.pr_run.restype = C.c_int
        L.pr_observables.argtypes = [C.c_void_p, _dp]
        L.pr_rhoz.argtypes = [C.c_void_p, _dp, C.c_int]
        L.pr_rhoz.restype = C.c_int
        L.pr_rng_words.argtypes = [C.c_void_p, C.c_uint, _up]
        L.pr_beads_energy.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int]
        L.pr_beads_energy.restype = C.c_double
        L.pr_gc_info.argtypes = [C.c_void_p, _dp]
        L.pr_run_full.argtypes = [C.c_void_p]
        L.pr_pressure_force_slit.argtypes = [C.c_void_p, _dp]
        L.pr_wall_force.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.pr_wall_force.restype = C.c_double
        L.pr_ewald_force_z.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp]
        L.pr_chem_pot.argtypes = [C.c_void_p]
        L.pr_chem_pot.restype = C.c_double
        _ref_lib = L
    return _ref_lib


def _load_oracle():
    global _orc_lib
    if _orc_lib is None:
        L = C.CDLL(ORACLE_SO)
        L.po_create.restype = C.c_void_p
        L.po_create.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32, C.c_char_p, C.c_int]
        L.po_destroy.argtypes = [C.c_void_p]
        for f in ("po_n_bead", "po_n_mol", "po_n_kvec"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int
        L.po_ewald_info.argtypes = [C.c_void_p, _dp]
        L.po_total_energy.argtypes = [C.c_void_p, _dp]
        L.po_energies.argtypes = [C.c_void_p, _dp]
        L.po_delta_energy.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _dp]
        L.po_run.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _dp]
        L.po_run.restype = C.c_int
        L.po_run_stream.argtypes = [C.c_void_p, C.c_int, _up, C.c_long, _ip, _ip, _dp]
        L.po_run_stream.restype = C.c_long
        L.po_coords.argtypes = [C.c_void_p, _dp]
        L.po_set_coords.argtypes = [C.c_void_p, _dp]
        L.po_observables.argtypes = [C.c_void_p, _dp]
        L.po_rhoz.argtypes = [C.c_void_p, _dp, C.c_int]
        L.po_rhoz.restype = C.c_int
        L.po_mt19937.argtypes = [C.c_uint32, C.c_long, _up]
        L.po_set_fast_init.argtypes = [C.c_int]
        L.po_beads_energy.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int]
        L.po_beads_energy.restype = C.c_double
        L.po_pressure_force_slit.argtypes = [C.c_void_p, _dp]
        L.po_wall_force.argtypes = [C.c_void_p, C.c_int]
        L.po_wall_force.restype = C.c_double
        L.po_ewald_force_z.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.po_chem_pot.argtypes = [C.c_void_p]
        L.po_chem_pot.restype = C.c_double
        _orc_lib = L
    return _orc_lib


class _Base:
    def _steps(self, fn, n):
        mt = np.zeros(n, np.int32)
        ac = np.zeros(n, np.int32)
        dr = np.zeros(n, np.int32)
        et = np.zeros(n, np.float64)
        fn(self.h, n, mt, ac, dr, et)
        return mt, ac, dr, et


class Ref(_Base):
    """The reference's own code (oracle/_ref/libplumref.so)."""

    def __init__(self, dirpath: str, runin: str = "run.in", seed: int = 1):
        self.L = _load_ref()
        self.h = self.L.pr_create(dirpath.encode(), runin.encode(), seed)
        if not self.h:
            raise RuntimeError("reference could not read %s/%s" % (dirpath, runin))
        self.n_bead = self.L.pr_n_bead(self.h)
        self.n_mol = self.L.pr_n_mol(self.h)

    def close(self):
        if self.h:
            self.L.pr_destroy(self.h)
            self.h = None

    def __del__(self):
        if getattr(self, 'h', None):
            self.close()

    def energies(self):
        o = np.zeros(4)
        self.L.pr_energies(self.h, o)
        return o

    def recompute(self):
        o = np.zeros(4)
        self.L.pr_recompute(self.h, o)
        return o

    def coords(self):
        self.n_bead = self.L.pr_n_bead(self.h)  # grand-canonical moves change it
        o = np.zeros(3 * self.n_bead)
        self.L.pr_coords(self.h, o)
        return o.reshape(-1, 3)

    def ewald_info(self):
        o = np.zeros(15)
        self.L.pr_ewald_info(self.h, o)
        return o

    def mol_size(self, m):
        return self.L.pr_mol_size(self.h, m)

    def pair_terms(self, ma, ia, mb, ib):
        o = np.zeros(3)
        self.L.pr_pair_terms(self.h, ma, ia, mb, ib, o)
        return o

    def delta_energy(self, mol, trial, moved):
        o = np.zeros(3)
        self.L.pr_delta_energy(self.h, mol, np.ascontiguousarray(trial, np.float64).ravel(),
                               np.ascontiguousarray(moved, np.int32), o)
        return o

    def run(self, n):
        return self._steps(self.L.pr_run, n)

    def pressure_force_slit(self):
        """p_tensor[0..11] after one CalcPressureForceLJELSlit."""
        o = np.zeros(12)
        self.L.pr_pressure_force_slit(self.h, o)
        return o

    def wall_force(self, mol, bead):
        return self.L.pr_wall_force(self.h, mol, bead)

    def ewald_force_z(self, ma, ia, mb, ib):
        o = np.zeros(2)
        self.L.pr_ewald_force_z(self.h, ma, ia, mb, ib, o)
        return o

    def chem_pot(self):
        """CalcChemicalPotentialF's Widom average (consumes the generator)."""
        return self.L.pr_chem_pot(self.h)

    def run_full(self):
        """The reference's Simulation::Run with its sampling and output
        files (into the case directory); close() runs its destructor, which
        makes the last writes."""
        self.L.pr_run_full(self.h)

    def observables(self):
        o = np.zeros(5)
        self.L.pr_observables(self.h, o)
        return o

    def rhoz(self, cap=1 << 20):
        o = np.zeros(cap)
        nb = self.L.pr_rhoz(self.h, o, cap)
        return o[:3 * nb].reshape(nb, 3)

    def rng_words(self, n):
        o = np.zeros(n, np.uint32)
        self.L.pr_rng_words(self.h, n, o)
        return o

    def gc_info(self):
        o = np.zeros(4)
        self.L.pr_gc_info(self.h, o)
        return o

    def beads_energy(self, b1, b2, chain, chain_ci, delete_id=-1):
        cl = 0 if chain is None else len(chain)
        a = lambda x: None if x is None else np.ascontiguousarray(x, np.float64).ravel()
        keep = [a(b2), a(chain), a(chain_ci)]
        ptr = lambda x: None if x is None else x.ctypes.data_as(C.c_void_p)
        return self.L.pr_beads_energy(self.h, a(b1), ptr(keep[0]), cl, ptr(keep[1]), ptr(keep[2]),
                                      delete_id)


class Oracle(_Base):
    """The FP64 CPU restatement (oracle/_ref/liboracle.so)."""

    def __init__(self, dirpath: str, runin: str = "run.in", seed: int = 1,
                 fast_init: bool = False):
        self.L = _load_oracle()
        err = C.create_string_buffer(512)
        self.L.po_set_fast_init(int(fast_init))
        self.h = self.L.po_create(dirpath.encode(), runin.encode(), seed, err, 512)
        self.L.po_set_fast_init(0)
        if not self.h:
            raise ValueError(err.value.decode())
        self.n_bead = self.L.po_n_bead(self.h)
        self.n_mol = self.L.po_n_mol(self.h)
        self.n_kvec = self.L.po_n_kvec(self.h)

    def close(self):
        if self.h:
            self.L.po_destroy(self.h)
            self.h = None

    def __del__(self):
        if getattr(self, 'h', None):
            self.close()

    def ewald_info(self):
        o = np.zeros(15)
        self.L.po_ewald_info(self.h, o)
        return o

    def total_energy(self):
        o = np.zeros(8)
        self.L.po_total_energy(self.h, o)
        return o

    def energies(self):
        o = np.zeros(4)
        self.L.po_energies(self.h, o)
        return o

    def delta_energy(self, mol, trial, moved):
        o = np.zeros(5)
        self.L.po_delta_energy(self.h, mol, np.ascontiguousarray(trial, np.float64).ravel(),
                               np.ascontiguousarray(moved, np.int32), o)
        return o

    def run(self, n):
        return self._steps(self.L.po_run, n)

    def run_stream(self, n, stream):
        mt = np.zeros(n, np.int32)
        ac = np.zeros(n, np.int32)
        et = np.zeros(n, np.float64)
        s = np.ascontiguousarray(stream, np.uint32)
        used = self.L.po_run_stream(self.h, n, s, len(s), mt, ac, et)
        return used, mt, ac, et

    def coords(self):
        self.n_bead = self.L.po_n_bead(self.h)  # grand-canonical moves change it
        o = np.zeros(3 * self.n_bead)
        self.L.po_coords(self.h, o)
        return o.reshape(-1, 3)

    def set_coords(self, xyz):
        self.L.po_set_coords(self.h, np.ascontiguousarray(xyz, np.float64).ravel())

    def observables(self):
        o = np.zeros(5)
        self.L.po_observables(self.h, o)
        return o

    def pressure_force_slit(self):
        """p_tensor[0..11] after one wall-force pressure evaluation
        (ForceField::CalcPressureForceLJELSlit, pressure.cc:400-488)."""
        o = np.zeros(12)
        self.L.po_pressure_force_slit(self.h, o)
        return o

    def wall_force(self, i):
        return self.L.po_wall_force(self.h, i)

    def chem_pot(self):
        """The Widom average of 50 test insertions (consumes the generator)."""
        return self.L.po_chem_pot(self.h)

    def ewald_force_z(self, a, b):
        o = np.zeros(2)
        self.L.po_ewald_force_z(self.h, a, b, o)
        return o

    def rhoz(self, cap=1 << 20):
        o = np.zeros(cap)
        nb = self.L.po_rhoz(self.h, o, cap)
        return o[:3 * nb].reshape(nb, 3)

    def beads_energy(self, b1, b2, chain, chain_ci, delete_id=-1):
        cl = 0 if chain is None else len(chain)
        a = lambda x: None if x is None else np.ascontiguousarray(x, np.float64).ravel()
        keep = [a(b2), a(chain), a(chain_ci)]
        ptr = lambda x: None if x is None else x.ctypes.data_as(C.c_void_p)
        return self.L.po_beads_energy(self.h, a(b1), ptr(keep[0]), cl, ptr(keep[1]),
                                      ptr(keep[2]), delete_id)


def mt19937(seed: int, n: int) -> np.ndarray:
    o = np.zeros(n, np.uint32)
    _load_oracle().po_mt19937(seed, n, o)
    return o
