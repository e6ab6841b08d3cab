"""ctypes binding of the CUDA engine (libhande_gpu.so, C ABI in include/hande_gpu.h).

There is no CPU fallback: constructing an :class:`Engine` without the built
library or without a CUDA device raises."""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._abi import (STATUS_TEXT, HgpuConfig, HgpuLaunch, HgpuReport, HgpuState, HgpuSystem, PackedSystem,
                   make_config)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhande_gpu.so")

# Every entry point of include/hande_gpu.h (checked by the CPU test suite).
EXPORTS = [
    "hgpu_version", "hgpu_error_string", "hgpu_device_count", "hgpu_create", "hgpu_destroy",
    "hgpu_initial_distribution", "hgpu_upload_walkers", "hgpu_download_walkers", "hgpu_run_cycles",
    "hgpu_end_report", "hgpu_run_report", "hgpu_get_state", "hgpu_set_state", "hgpu_checkpoint",
    "hgpu_restore", "hgpu_eval_excitations", "hgpu_annihilate_fixed", "hgpu_eval_diagonal",
    "hgpu_profile_cycle", "hgpu_snapshot", "hgpu_self_annihilate_noalloc",
    "hgpu_batch_create", "hgpu_batch_run_cycles", "hgpu_batch_destroy", "hgpu_rdm_download",
    "hgpu_get_launch", "hgpu_set_launch",
]


class HgpuError(RuntimeError):
    def __init__(self, status: int, where: str, text: str = ""):
        self.status = status
        super().__init__("%s: %s (status %d)" % (where, text or STATUS_TEXT.get(status, "?"), status))


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libhande_gpu.so and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("CUDA engine library %s is missing: run hande_gb300.build.build()" % path)
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    L.hgpu_version.restype = C.c_int32
    L.hgpu_error_string.restype = C.c_char_p
    L.hgpu_error_string.argtypes = [C.c_int32]
    L.hgpu_device_count.restype = C.c_int32
    L.hgpu_create.argtypes = [P(HgpuConfig), P(HgpuSystem), P(vp)]
    L.hgpu_destroy.argtypes = [vp]
    L.hgpu_initial_distribution.argtypes = [vp]
    L.hgpu_upload_walkers.argtypes = [vp, P(C.c_int64), P(C.c_int64), P(C.c_double), C.c_int64]
    L.hgpu_download_walkers.argtypes = [vp, P(C.c_int64), P(C.c_int64), P(C.c_double), C.c_int64, P(C.c_int64)]
    L.hgpu_rdm_download.argtypes = [vp, P(C.c_double), C.c_int64, P(C.c_int64)]
    L.hgpu_run_cycles.argtypes = [vp, C.c_int32]
    L.hgpu_end_report.argtypes = [vp, P(HgpuReport)]
    L.hgpu_run_report.argtypes = [vp, P(HgpuReport)]
    L.hgpu_get_state.argtypes = [vp, P(HgpuState)]
    L.hgpu_set_state.argtypes = [vp, P(HgpuState)]
    L.hgpu_checkpoint.argtypes = [vp, C.c_char_p]
    L.hgpu_restore.argtypes = [vp, C.c_char_p]
    L.hgpu_eval_excitations.argtypes = [vp, P(C.c_int64), P(C.c_int64), C.c_int64, C.c_int64, P(C.c_int32),
                                        P(C.c_double), P(C.c_double), P(C.c_int32), P(C.c_int64)]
    L.hgpu_annihilate_fixed.argtypes = [vp, P(C.c_int64), C.c_int64, C.c_int64]
    L.hgpu_eval_diagonal.argtypes = [vp, P(C.c_int64), C.c_int64, P(C.c_double)]
    L.hgpu_profile_cycle.argtypes = [vp, P(C.c_double), C.c_int32, P(C.c_int64)]
    L.hgpu_snapshot.argtypes = [vp, C.c_int32]
    L.hgpu_get_launch.argtypes = [vp, P(HgpuLaunch)]
    L.hgpu_set_launch.argtypes = [vp, P(HgpuLaunch)]
    L.hgpu_self_annihilate_noalloc.argtypes = [vp, C.c_int64, C.c_int32, C.c_int32, vp, P(C.c_int64), vp]
    for name in EXPORTS:
        if name != "hgpu_error_string":
            getattr(L, name).restype = C.c_int32
    _lib = L
    return L


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Engine:
    """One FCIQMC calculation resident on the GPU (an hgpu_handle)."""

    def __init__(self, system, cfg: HgpuConfig = None, **kw):
        self.L = load_library()
        self.system = system
        self.packed = PackedSystem(system)
        self.cfg = cfg if cfg is not None else make_config(system, **kw)
        self.R = max(1, self.cfg.nspaces)
        h = C.c_void_p()
        self._check(self.L.hgpu_create(C.byref(self.cfg), C.byref(self.packed.struct), C.byref(h)), "hgpu_create")
        self.h = h

    def _check(self, rc, where, allow=()):
        if rc != 0 and rc not in allow:
            raise HgpuError(rc, where, self.L.hgpu_error_string(rc).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.hgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_distribution(self):
        self._check(self.L.hgpu_initial_distribution(self.h), "hgpu_initial_distribution")

    def set_walkers(self, states, pops, dat=None):
        st = np.ascontiguousarray(states, dtype=np.int64)
        po = np.ascontiguousarray(pops, dtype=np.int64)
        da = None if dat is None else np.ascontiguousarray(dat, dtype=np.float64)
        self._check(self.L.hgpu_upload_walkers(self.h, _p(st, C.c_int64), _p(po, C.c_int64),
                                               None if da is None else _p(da, C.c_double), po.shape[0]),
                    "hgpu_upload_walkers")

    def rdm(self):
        """The replica 2-RDM of the current report, [pair][pair] (None without density_matrices)."""
        n = C.c_int64()
        self._check(self.L.hgpu_rdm_download(self.h, None, 0, C.byref(n)), "hgpu_rdm_download")
        if n.value == 0:
            return None
        out = np.zeros(n.value)
        m = C.c_int64()
        self._check(self.L.hgpu_rdm_download(self.h, _p(out, C.c_double), n.value, C.byref(m)), "hgpu_rdm_download")
        k = int(round(np.sqrt(n.value)))
        return out.reshape(k, k)

    def walkers(self):
        n = C.c_int64()
        self.L.hgpu_download_walkers(self.h, None, None, None, 0, C.byref(n))
        n = n.value
        W = self.system.nwords
        st = np.zeros((n, W), dtype=np.int64)
        po = np.zeros((n, self.R), dtype=np.int64)
        da = np.zeros(n, dtype=np.float64)
        m = C.c_int64()
        self._check(self.L.hgpu_download_walkers(self.h, _p(st, C.c_int64), _p(po, C.c_int64),
                                                 _p(da, C.c_double), n, C.byref(m)), "hgpu_download_walkers")
        return st, po, da

    def run_cycles(self, n):
        return self._check(self.L.hgpu_run_cycles(self.h, n), "hgpu_run_cycles", allow=(3, 4))

    def end_report(self) -> HgpuReport:
        r = HgpuReport()
        self._check(self.L.hgpu_end_report(self.h, C.byref(r)), "hgpu_end_report", allow=(3, 4))
        return r

    def run_report(self) -> HgpuReport:
        r = HgpuReport()
        self._check(self.L.hgpu_run_report(self.h, C.byref(r)), "hgpu_run_report", allow=(3, 4))
        return r

    def state(self) -> HgpuState:
        s = HgpuState()
        self._check(self.L.hgpu_get_state(self.h, C.byref(s)), "hgpu_get_state")
        return s

    def get_state(self) -> HgpuState:
        s = HgpuState()
        self._check(self.L.hgpu_get_state(self.h, C.byref(s)), "hgpu_get_state")
        return s

    def set_state(self, s: HgpuState):
        self._check(self.L.hgpu_set_state(self.h, C.byref(s)), "hgpu_set_state")

    def checkpoint(self, path: str):
        self._check(self.L.hgpu_checkpoint(self.h, path.encode()), "hgpu_checkpoint")

    def restore(self, path: str):
        return self.L.hgpu_restore(self.h, path.encode())

    def eval_excitations(self, parents, parent_pops, iteration):
        pa = np.ascontiguousarray(parents, dtype=np.int64)
        pp = np.ascontiguousarray(parent_pops, dtype=np.int64)
        n = pp.shape[0]
        orbs = np.zeros((n, 4), dtype=np.int32)
        pgen = np.zeros(n)
        hm = np.zeros(n)
        al = np.zeros(n, dtype=np.int32)
        ns = np.zeros(n, dtype=np.int64)
        self._check(self.L.hgpu_eval_excitations(self.h, _p(pa, C.c_int64), _p(pp, C.c_int64), n, iteration,
                                                 _p(orbs, C.c_int32), _p(pgen, C.c_double), _p(hm, C.c_double),
                                                 _p(al, C.c_int32), _p(ns, C.c_int64)), "hgpu_eval_excitations")
        return orbs, pgen, hm, al, ns

    def annihilate_fixed(self, sdata, iteration):
        sd = np.ascontiguousarray(sdata, dtype=np.int64)
        return self._check(self.L.hgpu_annihilate_fixed(self.h, _p(sd, C.c_int64), sd.shape[0], iteration),
                           "hgpu_annihilate_fixed", allow=(4,))

    def snapshot(self, restore: bool = False):
        self._check(self.L.hgpu_snapshot(self.h, 1 if restore else 0), "hgpu_snapshot")

    def launch(self) -> HgpuLaunch:
        """The launch shape of the handle's kernels (spawn chunk and block counts)."""
        x = HgpuLaunch()
        self._check(self.L.hgpu_get_launch(self.h, C.byref(x)), "hgpu_get_launch")
        return x

    def set_launch(self, spawn_chunk, spawn_blocks, stream_blocks, sort_blocks):
        x = HgpuLaunch(int(spawn_chunk), int(spawn_blocks), int(stream_blocks), int(sort_blocks))
        self._check(self.L.hgpu_set_launch(self.h, C.byref(x)), "hgpu_set_launch")

    PHASES = ["prep", "attempt_scan", "spawn", "sort", "splits", "annihilate", "end"]

    def profile_cycle(self):
        """One cycle with per-phase device times (ms) and list sizes."""
        ms = np.zeros(7)
        cnt = np.zeros(8, dtype=np.int64)
        self._check(self.L.hgpu_profile_cycle(self.h, _p(ms, C.c_double), 7, _p(cnt, C.c_int64)),
                    "hgpu_profile_cycle")
        keys = ["N", "attempts", "spawned", "unique", "N_after", "launches_per_cycle", "sort_passes",
                "sort_bytes_per_entry"]
        return dict(zip(self.PHASES, ms.tolist())), dict(zip(keys, cnt.tolist()))

    def eval_diagonal(self, dets):
        d = np.ascontiguousarray(dets, dtype=np.int64)
        n = d.shape[0]
        out = np.zeros(n)
        self._check(self.L.hgpu_eval_diagonal(self.h, _p(d, C.c_int64), n, _p(out, C.c_double)),
                    "hgpu_eval_diagonal")
        return out


class Batch:
    """Independent calculations (Engines) advanced together: one CUDA graph launch
    per cycle for all of them (hgpu_batch_*).  The engines stay usable on their
    own between batch calls (reports, downloads, snapshots)."""

    def __init__(self, engines):
        self.L = load_library()
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        b = C.c_void_p()
        rc = self.L.hgpu_batch_create(arr, len(self.engines), C.byref(b))
        if rc != 0:
            raise HgpuError(rc, "hgpu_batch_create", self.L.hgpu_error_string(rc).decode())
        self.b = b

    def run_cycles(self, n):
        rc = self.L.hgpu_batch_run_cycles(self.b, n)
        if rc not in (0, 3, 4):
            raise HgpuError(rc, "hgpu_batch_run_cycles", self.L.hgpu_error_string(rc).decode())
        return rc

    def run_report(self):
        """ncycles of every engine (each engine's own ncycles must agree), then
        each engine's report."""
        nc = {e.cfg.ncycles for e in self.engines}
        if len(nc) != 1:
            raise ValueError("engines of a batch report must share ncycles")
        self.run_cycles(nc.pop())
        return [e.end_report() for e in self.engines]

    def close(self):
        if getattr(self, "b", None):
            self.L.hgpu_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
