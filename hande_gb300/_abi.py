"""ctypes mirror of the POD structs in include/hande_gpu.h and helpers that
pack a :class:`hande_gb300.systems.System` and calculation options into them.

The packed objects keep references to the numpy buffers their pointers refer
to, so they stay valid for as long as the Python object lives."""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from .systems import System

MAX_WORDS = 2
MAX_SPACES = 2

HGPU_OK = 0
STATUS_TEXT = {
    0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "spawned list overflow",
    4: "main list overflow", 5: "device wait timed out", 6: "CUDA error", 7: "no CUDA device",
    8: "unsupported option",
}

SYS_HUB_K = 1
SYS_READ_IN = 2

EXCIT_GEN = {
    "renorm": 0, "renorm_spin": 1, "no_renorm": 2, "no_renorm_spin": 3,
    "uniform_power_pitzer": 5, "power_pitzer_orderM": 5, "uniform_cauchy_schwarz": 8, "cauchy_schwarz_orderM": 8,
    "heat_bath_power_pitzer": 6, "power_pitzer_orderM_ij": 6, "heat_bath_cauchy_schwarz": 9,
    "heat_bath_power_pitzer_ref": 7, "power_pitzer_orderN": 7,
    "cauchy_schwarz_orderM_ij": 9,
    "heat_bath": 10, "heat_bath_uniform": 11, "heat_bath_single": 12,
}

PREC_FP64 = 0
PREC_MIXED = 1


class HgpuSystem(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("nbasis", C.c_int32), ("nel", C.c_int32), ("nalpha", C.c_int32),
        ("nbeta", C.c_int32), ("nwords", C.c_int32),
        ("orb_sym", C.POINTER(C.c_int32)), ("orb_ms", C.POINTER(C.c_int32)),
        ("sp_eigv", C.POINTER(C.c_double)),
        ("nkpoints", C.c_int32), ("sym_table", C.POINTER(C.c_int32)), ("inv_sym", C.POINTER(C.c_int32)),
        ("coulomb_k", C.c_double),
        ("norb", C.c_int32), ("nsym_pg", C.c_int32), ("h1", C.POINTER(C.c_double)),
        ("v2", C.POINTER(C.c_double)), ("nv2", C.c_int64), ("ecore", C.c_double),
        ("nbasis_sym_spin", C.POINTER(C.c_int32)), ("max_sym_spin", C.c_int32),
        ("sym_spin_basis_fns", C.POINTER(C.c_int32)),
    ]


class HgpuConfig(C.Structure):
    _fields_ = [
        ("tau", C.c_double), ("shift_damping", C.c_double), ("initial_shift", C.c_double),
        ("vary_shift_from", C.c_double), ("target_particles", C.c_double),
        ("initiator_pop", C.c_double), ("spawn_cutoff", C.c_double),
        ("pattempt_single", C.c_double), ("pattempt_double", C.c_double),
        ("D0_population", C.c_double),
        ("vary_shift_from_proje", C.c_int32), ("excit_gen", C.c_int32),
        ("real_amplitudes", C.c_int32), ("initiator_approx", C.c_int32), ("nspaces", C.c_int32),
        ("ncycles", C.c_int32), ("precision", C.c_int32), ("quadrature_initiator", C.c_int32),
        ("seed", C.c_int64), ("walker_length", C.c_int64), ("spawned_walker_length", C.c_int64),
        ("ref_det", C.c_uint64 * MAX_WORDS), ("pattempt_parallel", C.c_double),
        ("density_matrices", C.c_int32), ("density_matrix_report", C.c_int32),
        ("power_pitzer_min_weight", C.c_double),
        ("semi_stoch_space", C.c_int32), ("semi_stoch_size", C.c_int32),
        ("semi_stoch_start_iter", C.c_int64), ("semi_stoch_shift_iter", C.c_int64),
        ("semi_stoch_ci_level", C.c_int32), ("semi_stoch_combined", C.c_int32),
        ("shift_harmonic_forcing", C.c_double), ("target_reference", C.c_int32), ("reserved0", C.c_int32),
    ]


class HgpuReport(C.Structure):
    _fields_ = [
        ("iteration", C.c_int64), ("shift", C.c_double * MAX_SPACES),
        ("proj_energy", C.c_double * MAX_SPACES), ("D0_population", C.c_double * MAX_SPACES),
        ("nparticles", C.c_double * MAX_SPACES), ("vary_shift", C.c_int32 * MAX_SPACES),
        ("nstates", C.c_int64), ("nspawn_events", C.c_int64), ("rspawn", C.c_double),
        ("nattempts", C.c_int64), ("nspawned", C.c_int64), ("error_flags", C.c_int32),
        ("reserved0", C.c_int32), ("device_ms", C.c_double),
        ("rdm_energy", C.c_double), ("rdm_trace", C.c_double),
        ("nblooms", C.c_int64), ("tot_bloom", C.c_double), ("max_bloom", C.c_double),
    ]

    def as_dict(self, nspaces: int = 1) -> dict:
        r = {
            "iterations": int(self.iteration),
            "Shift": list(self.shift)[:nspaces],
            "\\sum H_0j N_j": list(self.proj_energy)[:nspaces],
            "N_0": list(self.D0_population)[:nspaces],
            "# H psips": list(self.nparticles)[:nspaces],
            "vary_shift": list(self.vary_shift)[:nspaces],
            "# states": int(self.nstates),
            "# spawn_events": int(self.nspawn_events),
            "R_spawn": float(self.rspawn),
            "attempts": int(self.nattempts),
            "spawned": int(self.nspawned),
            "error_flags": int(self.error_flags),
            "device_ms": float(self.device_ms),
            "blooms": int(self.nblooms),
            "bloom particles": float(self.tot_bloom),
            "max bloom": float(self.max_bloom),
        }
        if self.rdm_trace != 0.0:
            r["RDM energy num."] = float(self.rdm_energy)
            r["RDM trace"] = float(self.rdm_trace)
        return r


class HgpuLaunch(C.Structure):
    """Launch shape of a handle's kernels (hgpu_launch)."""
    _fields_ = [("spawn_chunk", C.c_int32), ("spawn_blocks", C.c_int32), ("stream_blocks", C.c_int32),
                ("sort_blocks", C.c_int32)]

    def as_tuple(self):
        return (int(self.spawn_chunk), int(self.spawn_blocks), int(self.stream_blocks), int(self.sort_blocks))


class HgpuState(C.Structure):
    _fields_ = [
        ("iteration", C.c_int64), ("shift", C.c_double * MAX_SPACES),
        ("vary_shift", C.c_int32 * MAX_SPACES), ("nparticles_old", C.c_double * MAX_SPACES),
        ("tau", C.c_double), ("seed", C.c_int64),
    ]


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return C.POINTER(ctype)()
    return a.ctypes.data_as(C.POINTER(ctype))


class PackedSystem:
    """An HgpuSystem plus the contiguous numpy buffers it points into."""

    def __init__(self, s: System):
        self.sys = s
        keep = []

        def arr(x, dt):
            if x is None:
                return None
            a = np.ascontiguousarray(np.asarray(x), dtype=dt)
            keep.append(a)
            return a

        st = HgpuSystem()
        st.kind = SYS_HUB_K if s.kind == "hubbard_k" else SYS_READ_IN
        st.nbasis = s.nbasis
        st.nel = s.nel
        st.nalpha = s.nalpha
        st.nbeta = s.nbeta
        st.nwords = s.nwords
        st.orb_sym = _ptr(arr(s.orb_sym, np.int32), C.c_int32)
        st.orb_ms = _ptr(arr(s.orb_ms, np.int32), C.c_int32)
        st.sp_eigv = _ptr(arr(s.sp_eigv, np.float64), C.c_double)
        if s.kind == "hubbard_k":
            st.nkpoints = s.nkpoints
            st.sym_table = _ptr(arr(s.sym_table.reshape(-1), np.int32), C.c_int32)
            st.inv_sym = _ptr(arr(s.inv_sym, np.int32), C.c_int32)
            st.coulomb_k = s.coulomb_k
        else:
            st.norb = s.norb
            st.nsym_pg = s.nsym_pg
            st.h1 = _ptr(arr(s.h1.reshape(-1), np.float64), C.c_double)
            st.v2 = _ptr(arr(s.v2, np.float64), C.c_double)
            st.nv2 = int(s.v2.size)
            st.ecore = s.ecore
            st.nbasis_sym_spin = _ptr(arr(s.nbasis_sym_spin.reshape(-1), np.int32), C.c_int32)
            st.max_sym_spin = int(s.sym_spin_basis_fns.shape[2])
            st.sym_spin_basis_fns = _ptr(arr(s.sym_spin_basis_fns.reshape(-1), np.int32), C.c_int32)
        self.struct = st
        self._keep = keep


def make_config(s: System, tau: float, *, ncycles: int = 10, seed: int = 7, init_pop: float = 10.0,
                target_population: float = 1e300, shift_damping: float = 0.05,
                initial_shift: float = 0.0, vary_shift_from: float = 0.0,
                vary_shift_from_proje: bool = False, real_amplitudes: bool = False,
                spawn_cutoff: float = 0.01, excit_gen: str = "renorm",
                pattempt_single: float = -1.0, pattempt_double: float = -1.0,
                pattempt_parallel: float = -1.0, density_matrices: bool = False,
                density_matrix_report: int = 0, power_pitzer_min_weight: float = 0.01, initiator: bool = False,
                initiator_threshold: float = 3.0, quadrature_initiator: bool = True, nspaces: int = 1,
                semi_stoch_space: int = 0,
                semi_stoch_size: int = 0, semi_stoch_start_iter: int = 1, semi_stoch_shift_iter: int = -1,
                semi_stoch_ci_level: int = 0, semi_stoch_combined: int = 0, shift_harmonic_forcing: float = 0.0,
                target_reference: bool = False,
                precision: int = PREC_FP64, state_size: int = 100000,
                spawned_state_size: int = 100000, reference=None) -> HgpuConfig:
    """Configuration with HANDE's qmc{} key names (src/lua_hande_calc.f90:1318-1331)."""
    cfg = HgpuConfig()
    cfg.tau = tau
    cfg.shift_damping = shift_damping
    cfg.initial_shift = initial_shift
    cfg.vary_shift_from = vary_shift_from
    cfg.target_particles = target_population
    cfg.initiator_pop = initiator_threshold
    cfg.spawn_cutoff = spawn_cutoff
    cfg.pattempt_single = pattempt_single
    cfg.pattempt_double = pattempt_double
    cfg.pattempt_parallel = pattempt_parallel
    cfg.density_matrices = int(bool(density_matrices))
    cfg.density_matrix_report = int(density_matrix_report)
    cfg.power_pitzer_min_weight = power_pitzer_min_weight
    cfg.semi_stoch_space = int(semi_stoch_space)
    cfg.semi_stoch_size = int(semi_stoch_size)
    cfg.semi_stoch_start_iter = int(semi_stoch_start_iter)
    cfg.semi_stoch_shift_iter = int(semi_stoch_shift_iter)
    cfg.semi_stoch_ci_level = int(semi_stoch_ci_level)
    cfg.semi_stoch_combined = int(semi_stoch_combined)
    cfg.shift_harmonic_forcing = float(shift_harmonic_forcing)
    cfg.target_reference = int(bool(target_reference))
    cfg.D0_population = init_pop
    cfg.vary_shift_from_proje = int(bool(vary_shift_from_proje))
    cfg.excit_gen = EXCIT_GEN[excit_gen] if isinstance(excit_gen, str) else int(excit_gen)
    cfg.real_amplitudes = int(bool(real_amplitudes))
    cfg.initiator_approx = int(bool(initiator))
    cfg.quadrature_initiator = int(bool(quadrature_initiator))
    cfg.nspaces = nspaces
    cfg.ncycles = ncycles
    cfg.precision = precision
    cfg.seed = seed
    cfg.walker_length = state_size
    cfg.spawned_walker_length = spawned_state_size
    occ = s.aufbau_occ() if reference is None else list(reference)
    f0 = s.encode(occ)
    for w in range(MAX_WORDS):
        cfg.ref_det[w] = int(f0[w]) if w < len(f0) else 0
    return cfg


def sdata_element_len(s: System, nspaces: int) -> int:
    return s.nwords + nspaces + 1
