"""ctypes front end of the CPU oracle (oracle/hande_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker of the GPU engine."""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from hande_gb300._abi import HgpuConfig, HgpuReport, HgpuState, HgpuSystem, PackedSystem, make_config

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with the committed Makefile (gcc, -ffp-contract=off)."""
    src = os.path.join(HERE, "hande_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [P(HgpuConfig), P(HgpuSystem)]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_initial_distribution.argtypes = [C.c_void_p]
        L.oracle_set_walkers.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_double), C.c_int64]
        L.oracle_get_walkers.restype = C.c_int64
        L.oracle_get_walkers.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_double), C.c_int64]
        L.oracle_run_cycles.argtypes = [C.c_void_p, C.c_int32]
        L.oracle_end_report.argtypes = [C.c_void_p, P(HgpuReport)]
        L.oracle_get_state.argtypes = [C.c_void_p, P(HgpuState)]
        L.oracle_set_state.argtypes = [C.c_void_p, P(HgpuState)]
        L.oracle_eval_excitations.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), C.c_int64, C.c_int64,
                                              P(C.c_int32), P(C.c_double), P(C.c_double), P(C.c_int32),
                                              P(C.c_int64)]
        L.oracle_annihilate_fixed.argtypes = [C.c_void_p, P(C.c_int64), C.c_int64, C.c_int64]
        L.oracle_hmatel.restype = C.c_double
        L.oracle_hmatel.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64)]
        L.oracle_sc0.restype = C.c_double
        L.oracle_sc0.argtypes = [C.c_void_p, P(C.c_int64)]
        L.oracle_rdm.restype = C.c_int64
        L.oracle_rdm.argtypes = [C.c_void_p, P(C.c_double), C.c_int64]
        L.oracle_rdm_energy.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.oracle_rdm_from_list.argtypes = [C.c_void_p]
        L.oracle_pattempt_parallel.restype = C.c_double
        L.oracle_pattempt_parallel.argtypes = [C.c_void_p]
        L.oracle_pattempt.restype = None
        L.oracle_determ_space.restype = C.c_int64
        L.oracle_determ_space.argtypes = [C.c_void_p, P(C.c_int64), C.c_int64]
        L.oracle_pattempt.argtypes = [C.c_void_p, P(C.c_double)]
        L.oracle_pgen.restype = C.c_double
        L.oracle_pgen.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int32)]
        L.oracle_total_attempts.restype = C.c_int64
        L.oracle_total_attempts.argtypes = [C.c_void_p]
        L.oracle_par_create.restype = C.c_void_p
        L.oracle_par_create.argtypes = [P(HgpuConfig), P(HgpuSystem), C.c_int]
        L.oracle_par_destroy.argtypes = [C.c_void_p]
        L.oracle_par_initial_distribution.argtypes = [C.c_void_p]
        L.oracle_par_run_cycles.argtypes = [C.c_void_p, C.c_int32]
        L.oracle_par_begin_report.argtypes = [C.c_void_p]
        L.oracle_par_end_report.argtypes = [C.c_void_p, P(HgpuReport)]
        L.oracle_par_snapshot.argtypes = [C.c_void_p, C.c_int]
        L.oracle_par_set_state.argtypes = [C.c_void_p, P(HgpuState)]
        L.oracle_par_get_state.argtypes = [C.c_void_p, P(HgpuState)]
        L.oracle_par_total_attempts.restype = C.c_int64
        L.oracle_par_total_attempts.argtypes = [C.c_void_p]
        L.oracle_par_get_walkers.restype = C.c_int64
        L.oracle_par_get_walkers.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_double), C.c_int64]
        L.oracle_uniform.restype = C.c_double
        L.oracle_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
        _lib = L
    return _lib


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64).ctypes.data_as(C.POINTER(C.c_int64))


class Oracle:
    """One CPU FCIQMC calculation (the same state the GPU handle holds)."""

    def __init__(self, system, cfg: HgpuConfig = None, **kw):
        self.system = system
        self.packed = PackedSystem(system)
        self.cfg = cfg if cfg is not None else make_config(system, **kw)
        self.R = max(1, self.cfg.nspaces)
        self.L = lib()
        self.h = self.L.oracle_create(C.byref(self.cfg), C.byref(self.packed.struct))
        if not self.h:
            raise RuntimeError("oracle_create failed")

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_distribution(self):
        self.L.oracle_initial_distribution(self.h)

    def set_walkers(self, states, pops, dat=None):
        states = np.ascontiguousarray(states, dtype=np.int64)
        pops = np.ascontiguousarray(pops, dtype=np.int64)
        n = pops.shape[0]
        d = None if dat is None else np.ascontiguousarray(dat, dtype=np.float64)
        rc = self.L.oracle_set_walkers(self.h, states.ctypes.data_as(C.POINTER(C.c_int64)),
                                       pops.ctypes.data_as(C.POINTER(C.c_int64)),
                                       None if d is None else d.ctypes.data_as(C.POINTER(C.c_double)), n)
        if rc:
            raise RuntimeError("oracle_set_walkers: %d" % rc)

    def walkers(self):
        n = self.L.oracle_get_walkers(self.h, None, None, None, 0)
        W = self.system.nwords
        st = np.zeros((n, W), dtype=np.int64)
        po = np.zeros((n, self.R), dtype=np.int64)
        da = np.zeros(n, dtype=np.float64)
        self.L.oracle_get_walkers(self.h, st.ctypes.data_as(C.POINTER(C.c_int64)),
                                  po.ctypes.data_as(C.POINTER(C.c_int64)),
                                  da.ctypes.data_as(C.POINTER(C.c_double)), n)
        return st, po, da

    def run_cycles(self, n):
        return self.L.oracle_run_cycles(self.h, n)

    def end_report(self) -> HgpuReport:
        r = HgpuReport()
        self.L.oracle_end_report(self.h, C.byref(r))
        return r

    def run_report(self) -> HgpuReport:
        self.run_cycles(self.cfg.ncycles)
        return self.end_report()

    def state(self) -> HgpuState:
        s = HgpuState()
        self.L.oracle_get_state(self.h, C.byref(s))
        return s

    def set_state(self, s: HgpuState):
        self.L.oracle_set_state(self.h, C.byref(s))

    def eval_excitations(self, parents, parent_pops, iteration):
        parents = np.ascontiguousarray(parents, dtype=np.int64)
        pp = np.ascontiguousarray(parent_pops, dtype=np.int64)
        n = pp.shape[0]
        orbs = np.zeros((n, 4), dtype=np.int32)
        pgen = np.zeros(n)
        hm = np.zeros(n)
        al = np.zeros(n, dtype=np.int32)
        ns = np.zeros(n, dtype=np.int64)
        self.L.oracle_eval_excitations(self.h, parents.ctypes.data_as(C.POINTER(C.c_int64)),
                                       pp.ctypes.data_as(C.POINTER(C.c_int64)), n, iteration,
                                       orbs.ctypes.data_as(C.POINTER(C.c_int32)),
                                       pgen.ctypes.data_as(C.POINTER(C.c_double)),
                                       hm.ctypes.data_as(C.POINTER(C.c_double)),
                                       al.ctypes.data_as(C.POINTER(C.c_int32)),
                                       ns.ctypes.data_as(C.POINTER(C.c_int64)))
        return orbs, pgen, hm, al, ns

    def annihilate_fixed(self, sdata, iteration):
        sdata = np.ascontiguousarray(sdata, dtype=np.int64)
        return self.L.oracle_annihilate_fixed(self.h, sdata.ctypes.data_as(C.POINTER(C.c_int64)),
                                              sdata.shape[0], iteration)

    def hmatel(self, f1, f2) -> float:
        return self.L.oracle_hmatel(self.h, _i64(f1), _i64(f2))

    def sc0(self, f) -> float:
        return self.L.oracle_sc0(self.h, _i64(f))

    def rdm(self):
        m = self.L.oracle_rdm(self.h, None, 0)
        out = np.zeros(m)
        self.L.oracle_rdm(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), m)
        n = int(round(np.sqrt(m)))
        return out.reshape(n, n)

    def rdm_energy(self):
        e, t = C.c_double(), C.c_double()
        self.L.oracle_rdm_energy(self.h, C.byref(e), C.byref(t))
        return e.value, t.value

    def rdm_from_list(self):
        self.L.oracle_rdm_from_list(self.h)

    def pattempt_parallel(self) -> float:
        return self.L.oracle_pattempt_parallel(self.h)

    def determ_space(self):
        n = self.L.oracle_determ_space(self.h, None, 0)
        d = np.zeros((n, self.system.nwords), dtype=np.int64)
        self.L.oracle_determ_space(self.h, d.ctypes.data_as(C.POINTER(C.c_int64)), n)
        return d

    def pattempt(self):
        out = (C.c_double * 2)()
        self.L.oracle_pattempt(self.h, out)
        return out[0], out[1]

    def pgen(self, f, orbs) -> float:
        o = np.ascontiguousarray(orbs, dtype=np.int32)
        return self.L.oracle_pgen(self.h, _i64(f), o.ctypes.data_as(C.POINTER(C.c_int32)))

    def total_attempts(self) -> int:
        return self.L.oracle_total_attempts(self.h)


class OraclePar:
    """One calculation hash-partitioned over `nthreads` ranks (threads), as the
    reference runs over MPI ranks (oracle_par_* in hande_oracle.c)."""

    def __init__(self, system, cfg: HgpuConfig, nthreads: int):
        self.L = lib()
        self.sys = system
        self.packed = PackedSystem(system)
        self.cfg = cfg
        self.nw = system.nwords
        self.R = cfg.nspaces
        self.h = self.L.oracle_par_create(C.byref(cfg), C.byref(self.packed.struct), int(nthreads))
        if not self.h:
            raise RuntimeError("oracle_par_create failed")

    def close(self):
        if self.h:
            self.L.oracle_par_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_distribution(self):
        self.L.oracle_par_initial_distribution(self.h)

    def begin_report(self):
        """The start of a report (each rank clears its RDM once accumulating);
        run_cycles does it itself when it was not called."""
        self.L.oracle_par_begin_report(self.h)

    def run_cycles(self, n):
        return self.L.oracle_par_run_cycles(self.h, int(n))

    def end_report(self) -> HgpuReport:
        r = HgpuReport()
        self.L.oracle_par_end_report(self.h, C.byref(r))
        return r

    def run_report(self) -> HgpuReport:
        self.run_cycles(self.cfg.ncycles)
        return self.end_report()

    def snapshot(self, restore: bool = False):
        rc = self.L.oracle_par_snapshot(self.h, int(bool(restore)))
        if rc:
            raise RuntimeError("oracle_par_snapshot: no snapshot")

    def total_attempts(self) -> int:
        return int(self.L.oracle_par_total_attempts(self.h))

    def state(self) -> HgpuState:
        s = HgpuState()
        self.L.oracle_par_get_state(self.h, C.byref(s))
        return s

    def set_state(self, s: HgpuState):
        self.L.oracle_par_set_state(self.h, C.byref(s))

    def walkers(self):
        n = self.L.oracle_par_get_walkers(self.h, None, None, None, 0)
        st = np.zeros((max(n, 1), self.nw), dtype=np.int64)
        po = np.zeros((max(n, 1), self.R), dtype=np.int64)
        da = np.zeros(max(n, 1), dtype=np.float64)
        self.L.oracle_par_get_walkers(self.h, _i64(st), _i64(po), da.ctypes.data_as(C.POINTER(C.c_double)), n)
        return st[:n], po[:n], da[:n]


def uniform(seed, c0, c1, c2, c3, which=0):
    return lib().oracle_uniform(seed, c0, c1, c2, c3, which)
