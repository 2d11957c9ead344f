"""GB300 Monte Carlo energy engine for Plum-format polyelectrolyte systems.

The compute path is the CUDA library ``plum_gb300/_lib/libplumgpu.so`` (built
from ``plum_gb300/csrc`` for sm_103a). This module is a thin ctypes layer over
its C ABI (``include/plum_gpu.h``); it has no CPU implementation of any
energy term and raises if the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libplumgpu.so")

PLUM_OK = 0
PLUM_ERR_INPUT = 1
FORM_FP64 = 0
FORM_FP32 = 1
ERRORS = {1: "input", 2: "cuda", 3: "timeout", 4: "nonfinite", 5: "state", 6: "stream"}

_lib = None


class PlumError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s error (%d): %s" % (ERRORS.get(code, "unknown"), code, msg))
        self.code = code


class Info(C.Structure):
    _fields_ = [("n_bead", C.c_int), ("n_mol", C.c_int), ("n_type", C.c_int),
                ("n_kvec", C.c_int), ("npbc", C.c_int), ("form", C.c_int),
                ("box", C.c_double * 3), ("ewald_box", C.c_double * 3),
                ("real_cutoff", C.c_double), ("kcut2", C.c_double),
                ("alpha", C.c_double), ("lB", C.c_double),
                ("real_cell", C.c_int * 3), ("k_cell", C.c_int * 3)]


class RunInfo(C.Structure):
    """plum_run_info: the run-control items of run.in."""
    _fields_ = [("steps", C.c_long), ("steps_eq", C.c_long), ("sample_freq", C.c_long),
                ("stat_out_freq", C.c_long), ("traj_out_freq", C.c_long),
                ("beta", C.c_double), ("move_size", C.c_double), ("move_prob", C.c_double * 5),
                ("phantom", C.c_int), ("coion", C.c_int), ("grafted", C.c_int),
                ("grafted_counterion", C.c_int), ("calc_chem_pot", C.c_int),
                ("use_pair", C.c_int), ("use_ewald", C.c_int), ("use_bond", C.c_int),
                ("use_bond_rigid", C.c_int), ("use_ext", C.c_int), ("use_gc", C.c_int),
                ("gc_freq", C.c_int), ("rigid_bond", C.c_double), ("eq_bond", C.c_double),
                ("run_name", C.c_char * 256)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def lib():
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("plum_gb300 CUDA library not built: %s (run __graft_entry__.build())"
                              % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        L.plum_last_error.restype = C.c_char_p
        L.plum_ctx_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                      C.POINTER(C.c_void_p)]
        L.plum_ctx_destroy.argtypes = [C.c_void_p]
        L.plum_ctx_info.argtypes = [C.c_void_p, C.POINTER(Info)]
        L.plum_total_energy.argtypes = [C.c_void_p, _dp]
        L.plum_energies.argtypes = [C.c_void_p, _dp]
        L.plum_delta_energy.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _dp]
        L.plum_finalize.argtypes = [C.c_void_p, C.c_int]
        L.plum_run_moves.argtypes = [C.c_void_p, _up, C.c_long, C.c_int, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(C.c_long)]
        L.plum_run_moves_de.argtypes = [C.c_void_p, _up, C.c_long, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_long)]
        L.plum_seed.argtypes = [C.c_void_p, C.c_uint32]
        L.plum_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
        L.plum_get_positions.argtypes = [C.c_void_p, _dp]
        L.plum_set_positions.argtypes = [C.c_void_p, _dp]
        L.plum_observables.argtypes = [C.c_void_p, _dp]
        L.plum_rhoz.argtypes = [C.c_void_p, _dp, C.c_int, C.POINTER(C.c_int)]
        L.plum_pressure_slit.argtypes = [C.c_void_p, _dp]
        L.plum_get_topology.argtypes = [C.c_void_p, _ip, _dp, _ip]
        L.plum_last_timing.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                       C.POINTER(C.c_long)]
        L.plum_set_recompute.argtypes = [C.c_void_p, C.c_long]
        L.plum_drift.argtypes = [C.c_void_p, _dp]
        L.plum_probe_peaks.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.plum_batch_create.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                        C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.plum_batch_destroy.argtypes = [C.c_void_p]
        L.plum_batch_seed.argtypes = [C.c_void_p, C.c_uint32]
        L.plum_batch_seed_each.argtypes = [C.c_void_p, _up]
        L.plum_batch_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_long)]
        L.plum_batch_size.argtypes = [C.c_void_p]
        L.plum_batch_replica.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.plum_batch_last_timing.argtypes = [C.c_void_p, C.POINTER(C.c_double),
                                             C.POINTER(C.c_long)]
        L.plum_cbmc_trials.argtypes = [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_int, _dp]
        L.plum_cbmc_time.argtypes = [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                     C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.plum_sim_create.argtypes = [C.c_char_p, C.c_char_p, C.c_uint, C.c_int,
                                      C.POINTER(C.c_void_p)]
        L.plum_sim_destroy.argtypes = [C.c_void_p]
        L.plum_sim_translational_moves.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.plum_sim_run_steps.argtypes = [C.c_void_p, C.c_long]
        L.plum_sim_steps.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.plum_sim_n_bead.argtypes = [C.c_void_p]
        L.plum_gc_info.argtypes = [C.c_void_p, _dp]
        L.plum_append_molecules.argtypes = [C.c_void_p, C.c_int, _ip, _dp, _dp, _ip]
        L.plum_erase_molecules.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.plum_sim_positions.argtypes = [C.c_void_p, _dp]
        L.plum_sim_energies.argtypes = [C.c_void_p, _dp]
        L.plum_sim_enable_output.argtypes = [C.c_void_p, C.c_char_p]
        L.plum_sim_run.argtypes = [C.c_void_p]
        L.plum_sim_chem_pot.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.plum_sim_pressure.argtypes = [C.c_void_p, C.c_int, _dp]
        L.plum_sim_finish.argtypes = [C.c_void_p]
        L.plum_sim_write_checkpoint.argtypes = [C.c_void_p, C.c_char_p]
        L.plum_sim_read_checkpoint.argtypes = [C.c_void_p, C.c_char_p]
        _fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.plum_surrogate_create.argtypes = [C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]
        L.plum_surrogate_destroy.argtypes = [C.c_void_p]
        L.plum_surrogate_set_params.argtypes = [C.c_void_p, _fp]
        L.plum_surrogate_get_params.argtypes = [C.c_void_p, _fp]
        L.plum_surrogate_set_norm.argtypes = [C.c_void_p, _fp, _fp, C.c_float]
        L.plum_surrogate_set_margin.argtypes = [C.c_void_p, C.c_float]
        L.plum_surrogate_predict.argtypes = [C.c_void_p, _fp, C.c_long, _fp]
        L.plum_surrogate_predict_device.argtypes = [C.c_void_p, C.c_void_p, C.c_long, C.c_void_p]
        L.plum_surrogate_grad.argtypes = [C.c_void_p, _fp, _fp, C.c_long, _fp]
        L.plum_surrogate_adam_step.argtypes = [C.c_void_p, _fp, C.c_float]
        L.plum_surrogate_train.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_int,
                                           C.c_int, C.c_float, C.c_ulonglong, C.c_void_p]
        L.plum_collect_surrogate_data.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_void_p,
                                                  C.c_void_p, C.POINTER(C.c_long)]
        L.plum_move_descriptor.argtypes = [C.c_void_p, _dp]
        L.plum_batch_set_surrogate.argtypes = [C.c_void_p, C.c_void_p]
        L.plum_batch_time_kernels.argtypes = [C.c_void_p, C.c_int, _dp]
        L.plum_batch_set_tune.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.plum_batch_set_cells.argtypes = [C.c_void_p, C.c_int]
        L.plum_batch_descriptors.argtypes = [C.c_void_p, C.c_void_p]
        L.plum_batch_cell_stats.argtypes = [C.c_void_p, _ip]
        L.plum_batch_set_cell_cap.argtypes = [C.c_void_p, C.c_int]
        L.plum_batch_set_groups.argtypes = [C.c_void_p, C.c_int]
        L.plum_batch_autotune.argtypes = [C.c_void_p, C.c_int, _ip]
        L.plum_batch_da_stats.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
        L.plum_batch_set_recompute.argtypes = [C.c_void_p, C.c_long]
        L.plum_structure_factor.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.plum_batch_energies.argtypes = [C.c_void_p, _dp]
        L.plum_time_kernels.argtypes = [C.c_void_p, C.c_int, _dp]
        L.plum_batch_set_real_term.argtypes = [C.c_void_p, C.c_int]
        L.plum_batch_real_term.argtypes = [C.c_void_p]
        L.plum_h32_table.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.plum_h64_table.argtypes = [C.c_void_p, C.c_int]
        L.plum_run_params.argtypes = [C.c_void_p, C.POINTER(RunInfo)]
        L.plum_chain_observables.argtypes = [C.c_void_p, C.c_void_p, C.c_int,
                                             C.POINTER(C.c_int)]
        L.plum_batch_drift.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_long),
                                       C.POINTER(C.c_double)]
        _lib = L
    return _lib


def h32_table(scale=1.0, cut=0.0):
    """[bins, 4] cubic coefficients (in w = f/32, f the bin-local fraction) of
    the FP32 table of h(u'/scale), h(u) = erfc(sqrt u)/sqrt u, in bins of 1/32
    octave of u' from 2^-14 to 2^5; with cut > 0 the bins from u' = cut on
    are zero (the batch's cut table: scale = 16 / (alpha r_c^2), cut = 16)."""
    n = lib().plum_h32_table(None, 0, scale, cut)
    if n < 0:
        raise PlumError(PLUM_ERR_INPUT, lib().plum_last_error().decode())
    out = np.zeros(4 * n, np.float32)
    lib().plum_h32_table(_ptr(out), n, scale, cut)
    return out.reshape(n, 4)


def h64_table():
    """[bins, 10] degree-8 coefficients (and a zero) of the FP64 h(u) table
    (bins of 1/32 octave from u = 2^-12 to 2^5)."""
    n = lib().plum_h64_table(None, 0)
    out = np.zeros(10 * n, np.float64)
    lib().plum_h64_table(_ptr(out), n)
    return out.reshape(n, 10)


def probe_peaks(device: int = 0):
    """Measured (FP32, FP64) FMA throughput of the GPU in TFLOP/s."""
    a, b = C.c_double(0), C.c_double(0)
    _check(lib().plum_probe_peaks(device, C.byref(a), C.byref(b)))
    return a.value, b.value


def _check(rc):
    if rc != PLUM_OK:
        raise PlumError(rc, lib().plum_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dev(t, dtype):
    """Device pointer of a contiguous CUDA tensor of the given torch dtype."""
    if not (t.is_cuda and t.is_contiguous() and t.dtype == dtype):
        raise ValueError("expected a contiguous CUDA tensor of %s" % dtype)
    return C.c_void_p(t.data_ptr())


class System:
    """One system resident on a GPU, read from the reference's input files.

    Mirrors the reference's ForceField energy surface: ``total_energy``
    (InitializeEnergy), ``energies`` (Tot*Energy), ``energy_difference``
    (EnergyDifference) and ``finalize`` (FinalizeEnergies)."""

    def __init__(self, dirpath: str, runin: str = "run.in", form: int = FORM_FP64,
                 device: int = 0):
        L = lib()
        h = C.c_void_p()
        _check(L.plum_ctx_create(dirpath.encode(), runin.encode(), form, device, C.byref(h)))
        self.h = h
        info = Info()
        _check(L.plum_ctx_info(self.h, C.byref(info)))
        self.info = info
        self.n_bead = info.n_bead
        self.n_mol = info.n_mol

    def close(self):
        if getattr(self, "h", None):
            lib().plum_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def total_energy(self):
        o = np.zeros(8)
        _check(lib().plum_total_energy(self.h, o))
        return o

    def energies(self):
        o = np.zeros(4)
        _check(lib().plum_energies(self.h, o))
        return o

    def energy_difference(self, mol, trial, moved):
        o = np.zeros(5)
        _check(lib().plum_delta_energy(self.h, mol,
                                       np.ascontiguousarray(trial, np.float64).ravel(),
                                       np.ascontiguousarray(moved, np.int32), o))
        return o

    def finalize(self, accept: bool):
        _check(lib().plum_finalize(self.h, int(bool(accept))))

    def run_moves(self, stream, n_moves, logs=True):
        """Runs n_moves steps on the device consuming a recorded mt19937 stream."""
        s = np.ascontiguousarray(stream, np.uint32)
        mt = np.zeros(n_moves, np.int32) if logs else None
        ac = np.zeros(n_moves, np.int32) if logs else None
        et = np.zeros(n_moves, np.float64) if logs else None
        used = C.c_long(0)
        _check(lib().plum_run_moves(self.h, s, len(s), n_moves, _ptr(mt), _ptr(ac), _ptr(et),
                                    C.byref(used)))
        return used.value, mt, ac, et

    def run_moves_de(self, stream, n_moves):
        """run_moves that also logs each step's proposal energy change:
        (draws used, move types, accept flags, totals, dE [NaN: no move])."""
        s = np.ascontiguousarray(stream, np.uint32)
        mt = np.zeros(n_moves, np.int32)
        ac = np.zeros(n_moves, np.int32)
        et = np.zeros(n_moves, np.float64)
        de = np.zeros(n_moves, np.float64)
        used = C.c_long(0)
        _check(lib().plum_run_moves_de(self.h, s, len(s), n_moves, _ptr(mt), _ptr(ac), _ptr(et),
                                       _ptr(de), C.byref(used)))
        return used.value, mt, ac, et, de

    def seed(self, seed: int):
        _check(lib().plum_seed(self.h, seed))

    def time_kernels(self, n_moves):
        """n_moves device steps with CUDA events around each kernel: mean ms
        per launch of (energy change, serial step)."""
        o = np.zeros(2)
        _check(lib().plum_time_kernels(self.h, n_moves, o))
        return o

    def run(self, n_moves):
        acc = C.c_int(0)
        _check(lib().plum_run(self.h, n_moves, C.byref(acc)))
        return acc.value

    def _refresh_counts(self):
        info = Info()
        _check(lib().plum_ctx_info(self.h, C.byref(info)))
        self.info, self.n_bead, self.n_mol = info, info.n_bead, info.n_mol

    def append_molecules(self, sizes, xyz, q, types):
        """Appends molecules (sizes[m] beads each) after the last one."""
        sizes = np.ascontiguousarray(sizes, np.int32)
        _check(lib().plum_append_molecules(self.h, len(sizes), sizes,
                                           np.ascontiguousarray(xyz, np.float64).ravel(),
                                           np.ascontiguousarray(q, np.float64),
                                           np.ascontiguousarray(types, np.int32)))
        self._refresh_counts()

    def erase_molecules(self, first, count):
        _check(lib().plum_erase_molecules(self.h, first, count))
        self._refresh_counts()

    def positions(self):
        o = np.zeros(3 * self.n_bead)
        _check(lib().plum_get_positions(self.h, o))
        return o.reshape(-1, 3)

    def set_positions(self, xyz):
        _check(lib().plum_set_positions(self.h, np.ascontiguousarray(xyz, np.float64).ravel()))

    def topology(self):
        """(mol_start [n_mol+1], charge [n_bead], type index [n_bead])."""
        ms = np.zeros(self.n_mol + 1, np.int32)
        q = np.zeros(self.n_bead)
        ty = np.zeros(self.n_bead, np.int32)
        _check(lib().plum_get_topology(self.h, ms, q, ty))
        return ms, q, ty

    def observables(self):
        o = np.zeros(5)
        _check(lib().plum_observables(self.h, o))
        return o

    def run_params(self) -> RunInfo:
        """The run-control items of run.in (beta, move_size, move_prob, ...)."""
        o = RunInfo()
        _check(lib().plum_run_params(self.h, C.byref(o)))
        return o

    def chain_observables(self):
        """[chains, 5] per chain: Rg^2, Rg_x^2, Rg_y^2, Rg_z^2, end-to-end^2."""
        n = C.c_int(0)
        _check(lib().plum_chain_observables(self.h, None, 0, C.byref(n)))
        o = np.zeros((max(n.value, 1), 5))
        _check(lib().plum_chain_observables(self.h, _ptr(o), n.value, C.byref(n)))
        return o[:n.value]

    def structure_factor(self):
        """(S(k) [n_kvec] complex, k [n_kvec, 3] integer components): the
        running structure factor with the last accepted change applied."""
        nk = self.info.n_kvec
        sk = np.zeros(2 * max(nk, 1))
        kn = np.zeros(3 * max(nk, 1), np.int32)
        _check(lib().plum_structure_factor(self.h, _ptr(sk), _ptr(kn)))
        return sk[:2 * nk].view(np.complex128), kn[:3 * nk].reshape(-1, 3)

    def pressure_slit(self):
        """One evaluation of the wall-force pressure sums of a slit system:
        the increments of p_tensor[6..11] (LJ ions, polymers, wall-wall;
        Ewald ions, polymers, wall-wall)."""
        o = np.zeros(6)
        _check(lib().plum_pressure_slit(self.h, o))
        return o

    def rhoz(self):
        """One rho(z) sample [n_bins, 3] (chain beads, q >= 0 ions, q < 0 ions)."""
        nb = C.c_int(0)
        _check(lib().plum_rhoz(self.h, np.zeros(1), 0, C.byref(nb)))
        o = np.zeros(3 * nb.value)
        _check(lib().plum_rhoz(self.h, o, len(o), C.byref(nb)))
        return o.reshape(-1, 3)

    def cbmc_trials(self, b1, b2=None, chain=None, chain_ci=None, delete_mol=-1):
        """BeadsEnergy of trial sites b1[T,3] (and trial counterions b2[T,3] for a
        charged species) given the grown chain[cl,3] (and chain_ci[cl,3])."""
        b1 = np.ascontiguousarray(b1, np.float64).reshape(-1, 3)
        T = len(b1)
        keep = [None if x is None else np.ascontiguousarray(x, np.float64).ravel()
                for x in (b2, chain, chain_ci)]
        cl = 0 if chain is None else len(np.asarray(chain).reshape(-1, 3))
        u = np.zeros(T)
        _check(lib().plum_cbmc_trials(self.h, T, b1.ravel(), _ptr(keep[0]), cl, _ptr(keep[1]),
                                      _ptr(keep[2]), delete_mol, u))
        return u

    def cbmc_time(self, b1, b2=None, chain=None, chain_ci=None, delete_mol=-1, reps=50):
        """(ms per growth step, kernel launches per growth step) of
        cbmc_trials' kernels on these inputs, CUDA events on the device."""
        b1 = np.ascontiguousarray(b1, np.float64).reshape(-1, 3)
        keep = [None if x is None else np.ascontiguousarray(x, np.float64).ravel()
                for x in (b2, chain, chain_ci)]
        cl = 0 if chain is None else len(np.asarray(chain).reshape(-1, 3))
        ms, n = C.c_double(0), C.c_int(0)
        _check(lib().plum_cbmc_time(self.h, len(b1), b1.ravel(), _ptr(keep[0]), cl,
                                    _ptr(keep[1]), _ptr(keep[2]), delete_mol, reps,
                                    C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_recompute(self, every: int):
        _check(lib().plum_set_recompute(self.h, every))

    def drift(self):
        o = np.zeros(5)
        _check(lib().plum_drift(self.h, o))
        return o

    def last_timing(self):
        ms = C.c_double(0)
        k = C.c_long(0)
        _check(lib().plum_last_timing(self.h, C.byref(ms), C.byref(k)))
        return ms.value, k.value


    def move_descriptor(self):
        """Surrogate descriptor [96] of the pending trial move (after
        energy_difference, before finalize)."""
        o = np.zeros(96)
        _check(lib().plum_move_descriptor(self.h, o))
        return o

    def collect_surrogate_data(self, n_moves: int, cap: int, out=None):
        """Runs n_moves plain steps (as run) and returns (desc [k][96], dE [k])
        of the chain moves among them as CUDA tensors (k <= cap). `out`: a
        pair of preallocated tensors ([>= cap][96] float32, [>= cap] float64)
        to write into instead (they must be idle on the GPU)."""
        import torch
        if out is None:
            desc = torch.empty((cap, 96), dtype=torch.float32, device="cuda")
            de = torch.empty(cap, dtype=torch.float64, device="cuda")
            torch.cuda.current_stream().synchronize()
        else:
            desc, de = out
            if desc.shape[0] < cap or de.shape[0] < cap:
                raise ValueError("output tensors smaller than cap")
        k = C.c_long(0)
        _check(lib().plum_collect_surrogate_data(self.h, n_moves, cap, _dev(desc, torch.float32),
                                                 _dev(de, torch.float64), C.byref(k)))
        return desc[:k.value], de[:k.value]


class Surrogate:
    """The learned energy-change surrogate (include/plum_gpu.h,
    plum_surrogate_*): BF16 tensor-core forward/backward and Adam on the GPU."""

    N_IN = 96

    def __init__(self, seed: int = 1, device: int = 0):
        h = C.c_void_p()
        _check(lib().plum_surrogate_create(device, seed, C.byref(h)))
        self.h = h
        self.n_params = lib().plum_surrogate_nparams()

    def close(self):
        if getattr(self, "h", None):
            lib().plum_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        o = np.zeros(self.n_params, np.float32)
        _check(lib().plum_surrogate_get_params(self.h, o))
        return o

    def set_params(self, p):
        _check(lib().plum_surrogate_set_params(self.h, np.ascontiguousarray(p, np.float32)))

    def set_norm(self, mu, isd, y_scale):
        self.norm = (np.asarray(mu, np.float32), np.asarray(isd, np.float32), float(y_scale))
        _check(lib().plum_surrogate_set_norm(self.h, np.ascontiguousarray(mu, np.float32),
                                             np.ascontiguousarray(isd, np.float32), y_scale))

    def set_margin(self, margin):
        """Dead zone of delayed acceptance: s' = sign(s) max(|s| - margin, 0)."""
        self.margin = float(margin)
        _check(lib().plum_surrogate_set_margin(self.h, margin))

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 96)
        o = np.zeros(len(x), np.float32)
        _check(lib().plum_surrogate_predict(self.h, x, len(x), o))
        return o

    def predict_device(self, x):
        import torch
        out = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        torch.cuda.synchronize()
        _check(lib().plum_surrogate_predict_device(self.h, _dev(x, torch.float32), x.shape[0],
                                                   _dev(out, torch.float32)))
        return out

    def grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 96)
        t = np.ascontiguousarray(t, np.float32)
        o = np.zeros(self.n_params + 1, np.float32)
        _check(lib().plum_surrogate_grad(self.h, x, t, len(x), o))
        return o[:-1], float(o[-1])

    def adam_step(self, g, lr):
        _check(lib().plum_surrogate_adam_step(self.h, np.ascontiguousarray(g, np.float32), lr))

    def train(self, x, t, batch=4096, epochs=1, lr=1e-3, seed=0):
        """Adam on CUDA tensors x [n][96] (float32), t [n] (float32)."""
        import torch
        losses = np.zeros(max(epochs, 1))
        torch.cuda.synchronize()
        _check(lib().plum_surrogate_train(self.h, _dev(x, torch.float32), _dev(t, torch.float32),
                                          x.shape[0], batch, epochs, lr, seed,
                                          losses.ctypes.data_as(C.c_void_p)))
        return losses[:epochs]


class _Replica(System):
    """A replica context owned by a Batch (not destroyed by this object)."""

    def __init__(self, h):
        self.h = h
        info = Info()
        _check(lib().plum_ctx_info(self.h, C.byref(info)))
        self.info = info
        self.n_bead = info.n_bead
        self.n_mol = info.n_mol

    def close(self):
        self.h = None


class Batch:
    """Independent replicas (possibly of different systems) advanced together
    in the precision form: one move per replica per step."""

    def __init__(self, dirs, runins=None, form: int = FORM_FP32, device: int = 0):
        n = len(dirs)
        runins = runins or ["run.in"] * n
        d = (C.c_char_p * n)(*[x.encode() for x in dirs])
        r = (C.c_char_p * n)(*[x.encode() for x in runins])
        h = C.c_void_p()
        _check(lib().plum_batch_create(n, d, r, form, device, C.byref(h)))
        self.h = h
        self.n = n

    def close(self):
        if getattr(self, "h", None):
            lib().plum_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def seed(self, seed):
        if np.ndim(seed) == 0:
            _check(lib().plum_batch_seed(self.h, int(seed)))
        else:
            _check(lib().plum_batch_seed_each(self.h, np.ascontiguousarray(seed, np.uint32)))

    def run(self, n_steps):
        acc = C.c_long(0)
        _check(lib().plum_batch_run(self.h, n_steps, C.byref(acc)))
        return acc.value

    def replica(self, r) -> System:
        h = C.c_void_p()
        _check(lib().plum_batch_replica(self.h, r, C.byref(h)))
        return _Replica(h)

    def last_timing(self):
        ms = C.c_double(0)
        k = C.c_long(0)
        _check(lib().plum_batch_last_timing(self.h, C.byref(ms), C.byref(k)))
        return ms.value, k.value

    def time_kernels(self, n_steps):
        """n_steps steps with per-kernel CUDA events: mean ms per launch of
        (delta, serial, descriptor, inference)."""
        o = np.zeros(4)
        _check(lib().plum_batch_time_kernels(self.h, n_steps, o))
        return o

    def set_tune(self, item_pairs=4096, k_tile=128, grid=0, min_blocks=2):
        _check(lib().plum_batch_set_tune(self.h, item_pairs, k_tile, grid, min_blocks))

    def set_cells(self, on=True):
        """Surrogate descriptors through the cell lists (default) or the
        all-pairs kernel; the same integers either way."""
        _check(lib().plum_batch_set_cells(self.h, 1 if on else 0))

    def set_groups(self, groups):
        """1 or 2 step chains (two graph branches on two streams)."""
        _check(lib().plum_batch_set_groups(self.h, groups))

    def set_cell_cap(self, cap):
        _check(lib().plum_batch_set_cell_cap(self.h, cap))

    def cell_stats(self):
        """(replicas with a cell list, of which valid, most beads in one
        replica's list of beads that changed cell, its capacity)."""
        o = np.zeros(4, np.int32)
        _check(lib().plum_batch_cell_stats(self.h, o))
        return tuple(int(x) for x in o)

    def descriptors(self):
        """[replicas, 96] descriptors of the replicas' last surrogate moves."""
        out = np.zeros((self.n, 96), np.float32)
        _check(lib().plum_batch_descriptors(self.h, _ptr(out)))
        return out

    def autotune(self, steps=16):
        """Times the energy-change kernel's work-item sizes on these replicas
        and keeps the fastest: (item_pairs, k_tile, grid, min_blocks)."""
        o = np.zeros(4, np.int32)
        _check(lib().plum_batch_autotune(self.h, steps, o))
        return tuple(int(x) for x in o)

    def set_surrogate(self, sg):
        """Delayed acceptance with the surrogate sg (None: off)."""
        self._sg = sg
        _check(lib().plum_batch_set_surrogate(self.h, None if sg is None else sg.h))

    def da_stats(self):
        """(surrogate moves, stage-one passes, accepted) since set_surrogate."""
        o = (C.c_long * 3)()
        _check(lib().plum_batch_da_stats(self.h, o))
        return tuple(o)

    def energies(self):
        """[replicas, 4] running totals (pair, ewald, bond, ext), gathered on
        the device and copied in one transfer."""
        o = np.zeros((self.n, 4))
        _check(lib().plum_batch_energies(self.h, o))
        return o

    def set_real_term(self, table=True):
        """Real-space Ewald term from the h(u) table (True) or the erfc fit."""
        _check(lib().plum_batch_set_real_term(self.h, 1 if table else 0))

    def real_term(self):
        """1: the h(u) table, 0: the erfc fit."""
        return int(lib().plum_batch_real_term(self.h))

    def set_recompute(self, every):
        """Full FP64 recompute of each replica every `every` of its moves
        (0: never; default 10,000), staggered over the replicas."""
        _check(lib().plum_batch_set_recompute(self.h, int(every)))

    def drift(self):
        """([replicas, 6] per replica: running-minus-recomputed pair, ewald,
        bond, ext at its last recompute, the largest |total drift| so far,
        its number of recomputes), recomputes in the last run, their device
        milliseconds)."""
        o = np.zeros((self.n, 6))
        n = C.c_long(0)
        ms = C.c_double(0)
        _check(lib().plum_batch_drift(self.h, o, C.byref(n), C.byref(ms)))
        return o, n.value, ms.value


class HostSimulation:
    """The reference-named C++ host classes (include/plum_host.hpp) driven
    through include/plum_host_capi.h: Simulation::TranslationalMove with host
    control flow and device energies, or the device step loop."""

    def __init__(self, dirpath: str, runin: str = "run.in", seed: int = 5489,
                 form: int = FORM_FP64):
        import os as _os
        text = open(_os.path.join(dirpath, runin)).read()
        h = C.c_void_p()
        _check(lib().plum_sim_create(dirpath.encode(), text.encode(), seed, form, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().plum_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def translational_moves(self, n):
        mt = np.zeros(n, np.int32)
        ac = np.zeros(n, np.int32)
        _check(lib().plum_sim_translational_moves(self.h, n, _ptr(mt), _ptr(ac)))
        return mt, ac

    def run_steps(self, n):
        _check(lib().plum_sim_run_steps(self.h, n))

    def steps(self, n):
        """n steps of the reference's loop with host control flow, exchanges
        included: (move type per step, accepted per step)."""
        mt = np.zeros(n, np.int32)
        ac = np.zeros(n, np.int32)
        _check(lib().plum_sim_steps(self.h, n, _ptr(mt), _ptr(ac)))
        return mt, ac

    def n_bead(self):
        return lib().plum_sim_n_bead(self.h)

    def positions(self, n_bead=None):
        n_bead = self.n_bead() if n_bead is None else n_bead
        o = np.zeros(3 * n_bead)
        _check(lib().plum_sim_positions(self.h, o))
        return o.reshape(-1, 3)

    def energies(self):
        o = np.zeros(4)
        _check(lib().plum_sim_energies(self.h, o))
        return o

    def enable_output(self, dirpath="."):
        """The reference's output files (stat, trajectories, last
        coordinates / topology / rho(z)) into dirpath."""
        _check(lib().plum_sim_enable_output(self.h, str(dirpath).encode()))

    def chem_pot(self):
        """Widom's average of 50 configurational-bias test insertions
        (ForceField::CalcChemicalPotentialF; consumes the generator)."""
        v = C.c_double(0)
        _check(lib().plum_sim_chem_pot(self.h, C.byref(v)))
        return v.value

    def pressure(self, evaluate=False):
        """(p_tensor[0..11], evaluations so far) of the host ForceField; with
        evaluate one more CalcPressureForceLJELSlit first."""
        o = np.zeros(13)
        _check(lib().plum_sim_pressure(self.h, int(bool(evaluate)), o))
        return o[:12], int(o[12])

    def run(self):
        """The steps of run.in (Simulation::Run): samples and writes where
        the reference does."""
        _check(lib().plum_sim_run(self.h))

    def finish(self):
        """The writes of the reference's destructor; closes the files."""
        _check(lib().plum_sim_finish(self.h))

    def write_checkpoint(self, path):
        """Step, generator state, counters, averages and the device state
        for an exact restart."""
        _check(lib().plum_sim_write_checkpoint(self.h, str(path).encode()))

    def read_checkpoint(self, path):
        _check(lib().plum_sim_read_checkpoint(self.h, str(path).encode()))
