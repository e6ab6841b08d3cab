"""Benchmark: FCIQMC spawn attempts/s and iteration time on one GB300.

Headline workload (one "step" = one FCIQMC Monte Carlo cycle): the large
configuration -- the synthetic molecular Hamiltonian with 64 spatial orbitals
(two-word determinants) and 20 electrons (C1, ms=0), initiator FCIQMC
(threshold 3) with two replicas (quadrature initiator test) and the replica
2-RDM accumulating, real amplitudes (2^-31 fixed point), spawn cutoff 0.01,
uniform renorm generator with p_double 0.9, tau 2e-4, grown on the device to
about 5e8 walkers over both replicas (~157 GB of HBM held).  Each timed step
is one cycle (a report of one cycle) on that same walker list, restored device
to device (untimed) before it; every replay draws fresh random numbers.

  value      spawn attempts/s of the FP64 engine (the reference's precision)
             over the K timed cycles, CUDA events on the engine's stream
  e2e        the same through the C ABI with host-resident walker lists in
             pinned memory: upload, one cycle, download per step
  roofline   HBM roofline of the dominant kernel (spawning) and of the
             annihilation phases (sort + self-annihilation + merge)
  mixed_precision  the FP32 engine (FP32 H_ij, p_gen; FP64 K_ii, shift,
             estimators) on the same workload and its E_proj against FP64
  parity     one cycle of the GPU engine against the oracle from the same
             list, state and iteration: a slice of the benchmark's own list at
             the headline parameters, and the whole 26-orbital list
  cpu_baseline  the oracle (C restatement of HANDE's cycle), one core, on a
             bounded slice of the same walker list
  mol26      the 26-orbital molecule (FP64, ~1e7 walkers): attempts/s,
             phases and rooflines
  batched    128 Hubbard calculations advanced together

--impl reference times the CPU restatement of the reference algorithm as HANDE
runs it on many cores: one calculation hash-partitioned over all host cores
(threads) with an all-to-all of the spawned walkers every cycle, on the same
system and parameters at a bounded population (the reference itself, Fortran +
MPI + Lua, cannot be built here).
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "spawn attempts/s & iter time @1 GB300: FP32-batched vs FP64 plain at equal E_proj σ"
WORKLOAD = ("synthetic molecule M=26 nel=10 C1, real amplitudes, cutoff 0.01, uniform renorm p_double=0.9, "
            "tau=1e-3, ~1e7 walkers, FP64; each step = one full cycle on the same device-grown walker list")


def system_and_config(target=1e7, seed_ham=2024, seed_rng=7, cap_main=None, cap_spawn=None, ncycles=10):
    from hande_gb300 import systems
    from hande_gb300._abi import make_config
    s = systems.synthetic_molecule(26, 10, seed=seed_ham)
    cm = cap_main or int(4 * target) + 200000
    cs = cap_spawn or int(4 * target) + 200000
    cfg = make_config(s, tau=1e-3, init_pop=10, target_population=target, ncycles=ncycles, seed=seed_rng,
                      real_amplitudes=True, spawn_cutoff=0.01, excit_gen="renorm", pattempt_single=0.1,
                      pattempt_double=0.9, state_size=cm, spawned_state_size=cs)
    return s, cfg


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def pinned_array(rt, shape, dtype):
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = C.c_void_p()
    if rt is None or rt.cudaHostAlloc(C.byref(p), C.c_size_t(max(n, 8)), 0) != 0:
        return np.zeros(shape, dtype=dtype), None
    buf = (C.c_byte * max(n, 8)).from_address(p.value)
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape), p


def grow(eng, target, max_cycles=400, verbose=False):
    """Grow from the reference, one cycle at a time, until the population
    reaches half the target (the benchmark Hamiltonian grows about 3x per cycle
    at tau = 1e-3, so the list ends between 0.5x and 1.5x the target)."""
    rep = None
    for c in range(max_cycles):
        eng.run_cycles(1)
        rep = eng.end_report()
        if verbose:
            sys.stderr.write("grow %d Nw=%.4g states=%d shift=%.3f\n" % (c, rep.nparticles[0], rep.nstates,
                                                                         rep.shift[0]))
        if rep.error_flags:
            raise RuntimeError("walker list overflow while growing (flags %d)" % rep.error_flags)
        if rep.nparticles[0] >= 0.5 * target:
            break
    return rep


def cpu_sample_on_state(states, pops, dat, seconds=10.0, seed=7):
    """The oracle timed on whole cycles of the engine's own 26-orbital walker list."""
    from oracle.pyoracle import Oracle
    n = states.shape[0]
    s, cfg = system_and_config(target=1e7, seed_rng=seed, cap_main=int(3 * n) + 1000, cap_spawn=int(4 * n) + 1000)
    o = Oracle(s, cfg)
    o.set_walkers(states, pops, dat)
    a0 = o.total_attempts()
    t0 = time.perf_counter()
    ncyc = 0
    while ncyc == 0 or time.perf_counter() - t0 < seconds:
        o.run_cycles(1)
        ncyc += 1
    dt = time.perf_counter() - t0
    return {"attempts": o.total_attempts() - a0, "seconds": dt, "cycles": ncyc, "walkers": float(np.abs(pops).sum()) / 2 ** 31,
            "states": n}


def parity_cycle(s, cfg, st, po, da, state, sample):
    """One cycle of the GPU engine and of the oracle from the same walker list,
    state (iteration, shift, vary_shift) and hence the same random streams:
    the resulting lists must be equal bit for bit."""
    from hande_gb300.engine import Engine
    from oracle.pyoracle import Oracle
    g = Engine(s, cfg)
    o = Oracle(s, cfg)
    for x in (g, o):
        x.set_walkers(st, po, da)
        x.set_state(state)
    t0 = time.perf_counter()
    ro = o.run_report()
    t_oracle = time.perf_counter() - t0
    rg = g.run_report()
    sg, pg, kg = g.walkers()
    so, pq, ko = o.walkers()
    g.close()
    o.close()
    same_shape = sg.shape == so.shape
    out = {"sample": sample, "states_in": int(st.shape[0]), "states_out": int(so.shape[0]),
           "states_equal": bool(same_shape and np.array_equal(sg, so)),
           "pops_equal": bool(same_shape and np.array_equal(pg, pq)),
           "kii_max_rel_err": float(np.max(np.abs(kg - ko) / np.maximum(np.abs(ko), 1e-300))) if same_shape and
           ko.size else None,
           "attempts_equal": rg.nattempts == ro.nattempts, "spawned_equal": rg.nspawned == ro.nspawned,
           "blooms_equal": (rg.nblooms, rg.tot_bloom) == (ro.nblooms, ro.tot_bloom),
           "attempts": int(ro.nattempts), "oracle_seconds": t_oracle}
    if ro.rdm_trace:
        out["rdm_energy_rel_err"] = abs(rg.rdm_energy - ro.rdm_energy) / abs(ro.rdm_energy)
    return out


LARGE_WORKLOAD = ("synthetic molecule M=64 nel=20 ms=0 C1 (two-word determinants, 75-bit rank keys), "
                  "initiator FCIQMC (threshold 3) with 2 replicas (quadrature initiator) and the replica 2-RDM, real "
                  "amplitudes, spawn cutoff 0.01, uniform renorm generator (p_double 0.9), tau 2e-4, grown on the "
                  "device to ~5e8 walkers over both replicas; each step = one cycle on that same walker list")


def large_system():
    from hande_gb300 import systems
    return systems.synthetic_molecule(64, 20, seed=2024)


def large_config(s, precision, main_cap, spawn_cap, init_pop=1e6, seed=5):
    """The large configuration; the shift is held (target 1e300) while the
    population grows."""
    from hande_gb300._abi import make_config
    return make_config(s, tau=2e-4, init_pop=init_pop, target_population=1e300, ncycles=1, seed=seed,
                       real_amplitudes=True, spawn_cutoff=0.01, excit_gen="renorm", pattempt_single=0.1,
                       pattempt_double=0.9, initiator=True, initiator_threshold=3.0, nspaces=2,
                       precision=precision, density_matrices=True, density_matrix_report=0,
                       state_size=main_cap, spawned_state_size=spawn_cap)


def grow_replicas(e, target_total, max_grow=60, label="grow"):
    """Report by report (one cycle each) until both replicas together hold
    about target_total walkers: stop at 0.9 of it, or before a cycle that would
    overshoot it by 20 %."""
    last = None
    for r in range(max_grow):
        rep = e.run_report()
        tot = rep.nparticles[0] + rep.nparticles[1]
        if os.environ.get("HGPU_BENCH_VERBOSE"):
            sys.stderr.write("%s %d Nw=%.4g+%.4g states=%d flags=%d\n" % (
                label, r, rep.nparticles[0], rep.nparticles[1], rep.nstates, rep.error_flags))
        if rep.error_flags:
            raise RuntimeError("walker list overflow while growing (flags %d)" % rep.error_flags)
        g = tot / last if last else 1.0
        if tot >= 0.9 * target_total or tot * g > 1.2 * target_total:
            return rep, r + 1
        last = tot
    return rep, max_grow


def hold_and_save(e):
    """Every shift varying (so the replica RDM accumulates, as after
    equilibration), the walker list saved on the device as the step input."""
    st = e.get_state()
    st.vary_shift[0] = st.vary_shift[1] = 1
    e.set_state(st)
    e.snapshot()


def replay_steps(e, steps, warmup, clocks=None, barrier=None):
    """W untimed and K timed steps, each one report of one cycle started from
    the saved list (restored device to device, untimed)."""
    R = e.cfg.nspaces
    for _ in range(warmup):
        e.snapshot(restore=True)
        e.run_report()
    if barrier:
        barrier()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    dev_ms, att, flags = 0.0, 0, 0
    eproj, rdm = [], []
    for _ in range(steps):
        e.snapshot(restore=True)
        r = e.run_report()  # CUDA events on the engine stream around the cycle; synchronises
        dev_ms += r.device_ms
        att += r.nattempts
        flags |= r.error_flags
        eproj.append([r.proj_energy[q] / r.D0_population[q] if r.D0_population[q] else float("nan")
                      for q in range(R)])
        if r.rdm_trace:
            rdm.append(r.rdm_energy / r.rdm_trace)
    clk = clocks.stop() if clocks else None
    if flags:
        raise RuntimeError("walker list overflow during the timed cycles (flags %d)" % flags)
    return {"dev_ms": dev_ms, "attempts": att, "eproj": np.array(eproj), "rdm": rdm, "clocks": clk}


def e2e_measure(e, W, R, steps, main_cap):
    """The metric through the C ABI with host-resident walker lists: per step,
    hgpu_upload_walkers from pinned host memory, one cycle, hgpu_end_report and
    hgpu_download_walkers into pinned host memory; one untimed step first."""
    from hande_gb300.engine import _p
    rt = cudart()
    e.snapshot(restore=True)
    e.end_report()  # close the report that a cycle run before (e.g. hgpu_profile_cycle) left open
    st, po, da = e.walkers()
    n0 = st.shape[0]
    bufs = []
    hst, p1 = pinned_array(rt, (n0, W), np.int64)
    hpo, p2 = pinned_array(rt, (n0, R), np.int64)
    hda, p3 = pinned_array(rt, (n0,), np.float64)
    ost, p4 = pinned_array(rt, (main_cap, W), np.int64)
    opo, p5 = pinned_array(rt, (main_cap, R), np.int64)
    oda, p6 = pinned_array(rt, (main_cap,), np.float64)
    bufs = [p1, p2, p3, p4, p5, p6]
    pinned = [p is not None for p in bufs]
    hst[:] = st
    hpo[:] = po
    hda[:] = da
    del st, po, da
    L = e.L
    # one untimed step first, as the device-timed steps have their warm-up
    for _ in range(1):
        e._check(L.hgpu_upload_walkers(e.h, _p(hst, C.c_int64), _p(hpo, C.c_int64), _p(hda, C.c_double), n0),
                 "upload")
        e.run_report()
        m = C.c_int64()
        e._check(L.hgpu_download_walkers(e.h, _p(ost, C.c_int64), _p(opo, C.c_int64), _p(oda, C.c_double),
                                         main_cap, C.byref(m)), "download")
    h2d = d2h = att = 0
    t_up = t_cyc = t_down = 0.0
    up_ms = []
    rep_ms = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        ta = time.perf_counter()
        e._check(L.hgpu_upload_walkers(e.h, _p(hst, C.c_int64), _p(hpo, C.c_int64), _p(hda, C.c_double), n0),
                 "upload")
        h2d += n0 * (8 * W + 8 * R + 8)
        tb = time.perf_counter()
        r = e.run_report()
        att += r.nattempts
        rep_ms += r.device_ms
        tc = time.perf_counter()
        m = C.c_int64()
        e._check(L.hgpu_download_walkers(e.h, _p(ost, C.c_int64), _p(opo, C.c_int64), _p(oda, C.c_double),
                                         main_cap, C.byref(m)), "download")
        d2h += m.value * (8 * W + 8 * R + 8)
        t_up += tb - ta
        up_ms.append(1e3 * (tb - ta))
        t_cyc += tc - tb
        t_down += time.perf_counter() - tc
    e2e_s = time.perf_counter() - t0
    del hst, hpo, hda, ost, opo, oda
    for p in bufs:
        if p is not None and rt is not None:
            rt.cudaFreeHost(p)
    return {"value": att / e2e_s, "unit": "attempts/s", "h2d_bytes_per_step": h2d // steps,
            "d2h_bytes_per_step": d2h // steps,
            "note": "per step: hgpu_upload_walkers from pinned host memory, one cycle (hgpu_run_report), "
                    "hgpu_download_walkers into pinned host memory; host wall clock",
            "host_ms_per_step": {"upload": 1e3 * t_up / steps, "cycle": 1e3 * t_cyc / steps,
                                 "download": 1e3 * t_down / steps},
            "upload_ms_each": up_ms, "pinned": pinned, "steps": steps, "warmup": 1}


def cpu_slice(s, cfg, st, po, da, state, n, seconds):
    """The oracle (one core) on whole cycles of a slice of the benchmark's own
    walker list, with the benchmark's state (every shift varying, the RDM
    accumulating)."""
    from oracle.pyoracle import Oracle
    i0 = max(0, (st.shape[0] - n) // 2)
    sl = slice(i0, i0 + n)
    c = type(cfg).from_buffer_copy(cfg)
    c.walker_length = int(4 * n) + 1000
    c.spawned_walker_length = int(20 * n) + 1000
    o = Oracle(s, c)
    att = 0
    dt = 0.0
    ncyc = 0
    while ncyc == 0 or dt < seconds:
        o.set_walkers(st[sl], po[sl], da[sl])
        o.set_state(state)
        a0 = o.total_attempts()
        t0 = time.perf_counter()
        o.run_cycles(1)
        dt += time.perf_counter() - t0
        o.end_report()
        att += o.total_attempts() - a0
        ncyc += 1
    o.close()
    return {"value": att / dt, "unit": "attempts/s", "cores": 1, "kind": "port",
            "sample": "CPU oracle, 1 core, %d whole cycle(s) of a %d-state slice of the benchmark's own list "
                      "(%.3g attempts per cycle) in %.1f s" % (ncyc, n, att / ncyc, dt)}


REF_TARGET = 4e6  # total walkers of the reference arm's calculation (both replicas)


def cpu_reference_rate(s, cfg, ncores, target, steps, warmup, replicas):
    """The CPU restatement run as HANDE runs: one calculation hash-partitioned
    over `ncores` host threads (threads as ranks: owner =
    modulo(MurmurHash2(det), ranks), spawned walkers and RDM spawns exchanged
    every cycle, estimators summed per report), grown from the reference
    determinant with the shift held until it holds about `target` walkers (the
    bounded sample); then every shift varies, the list is saved, and each of
    `warmup` and `steps` steps is one cycle from that list (restored, untimed),
    the cycle timed on the host.  Returns (attempts/s, seconds per cycle,
    walkers, states, growth reports, attempts per step)."""
    from oracle.pyoracle import OraclePar
    o = OraclePar(s, cfg, ncores)
    o.initial_distribution()
    last = None
    grown = 0
    for r in range(80):
        rep = o.run_report()
        grown = r + 1
        if rep.error_flags:
            raise RuntimeError("CPU restatement: list overflow while growing (flags %d)" % rep.error_flags)
        tot = sum(rep.nparticles[q] for q in range(replicas))
        g = tot / last if last else 1.0
        if tot >= 0.9 * target or tot * g > 1.2 * target:
            break
        last = tot
    st = o.state()
    for q in range(replicas):
        st.vary_shift[q] = 1
    o.set_state(st)
    o.snapshot()
    for _ in range(warmup):
        o.snapshot(restore=True)
        o.run_report()
    secs, att = [], 0
    for _ in range(steps):
        o.snapshot(restore=True)
        o.begin_report()
        a0 = o.total_attempts()
        t0 = time.perf_counter()
        o.run_cycles(1)
        secs.append(time.perf_counter() - t0)
        att += o.total_attempts() - a0
        o.end_report()
    o.close()
    walkers = sum(rep.nparticles[q] for q in range(replicas))
    return att / sum(secs), float(np.mean(secs)), walkers, int(rep.nstates), grown, att / steps


def reference_arm(args):
    """The reference algorithm as HANDE runs it on many cores
    (cpu_reference_rate) on the headline system and parameters, with the
    population bounded (REF_TARGET walkers over both replicas, grown from the
    reference determinant) so that the run ends in a few minutes; like the GPU
    arm, every shift then varies (the RDM accumulates), the list is saved, and
    each of W warm-up and K timed steps is one cycle from that list."""
    from hande_gb300._abi import PREC_FP64
    ncores = os.cpu_count() or 1
    target = float(os.environ.get("HGPU_REF_TARGET", REF_TARGET))
    s = large_system()
    cfg = large_config(s, PREC_FP64, main_cap=int(2 * target / ncores) + 100000,
                       spawn_cap=int(3 * target / ncores) + 100000, init_pop=target / 500.0)
    t_start = time.perf_counter()
    rate, sec, walkers, states, grown, att_step = cpu_reference_rate(s, cfg, ncores, target, args.steps, args.warmup,
                                                                     2)
    sample = ("one calculation over %d host cores (threads as hash-partitioned ranks), grown to %.3g walkers "
              "(%d states) in %d cycles; each step one cycle from that list" % (ncores, walkers, states, grown))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "attempts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": LARGE_WORKLOAD, "sample": sample,
                   "parallelism": "one calculation hash-partitioned over all host cores"},
        "cpu_baseline": {"value": rate, "unit": "attempts/s", "cores": ncores, "kind": "port",
                         "sample": sample + " (CPU restatement of HANDE's cycle and MPI decomposition)"},
        "e2e": {"value": rate, "unit": "attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "attempts_per_step": att_step,
        "wall_s": time.perf_counter() - t_start,
    }
    print(json.dumps(line))


BATCH_WORKLOAD = ("128 independent Hubbard k-space calculations (2D periodic LxL, L in 3..6, "
                  "U in {2,4,8}, electrons = sites - 2, ms = 0 or 1 for odd counts, integer walkers, targets "
                  "log-uniform in [1e4, 1e6], seeded draw) advanced together, one graph launch per cycle")


def batched_instances(n=128, seed=4):
    """The batched configuration: systems and configurations of n instances."""
    from hande_gb300 import systems
    from hande_gb300._abi import make_config
    rng = np.random.default_rng(seed)
    out = []
    cache = {}
    for k in range(n):
        L = int(rng.choice([3, 4, 5, 6]))
        U = float(rng.choice([2.0, 4.0, 8.0]))
        target = float(10 ** rng.uniform(4, 6))
        nel = L * L - 2
        ms = nel % 2
        key = (L, U)
        if key not in cache:
            cache[key] = systems.hubbard_k([[L, 0], [0, L]], nel, U=U, ms=ms)
        s = cache[key]
        na, nb = (nel + ms) // 2, (nel - ms) // 2
        nvirt = L * L - na
        # tau: at most 0.2 expected spawned walkers per attempt, so that the
        # population grows by at most ~20 % per cycle
        tau = min(0.005, 0.2 / ((U / (L * L)) * na * nb * nvirt))
        cap = int(16 * target) + 20000
        # the calculation starts with the target population on the reference
        # determinant and reports (updates the shift) every cycle, so the shift
        # acts from the first cycle on
        cfg = make_config(s, tau=tau, init_pop=target, target_population=target, ncycles=1, seed=1000 + k,
                          state_size=cap, spawned_state_size=cap)
        out.append((s, cfg, dict(L=L, U=U, target=target, tau=tau)))
    return out


def batched_measure(steps, equil_cycles=150, tune=True):
    """The batch: every instance starts with its target population on the
    reference determinant; `equil_cycles` untimed cycles (a report after each,
    so that the shift acts every cycle) spread it out; the launch shapes are
    tuned on those lists (hande_gb300.autotune, untimed); then `steps` batch
    cycles are timed (one graph launch each for all instances), device time
    from the CUDA events around the batch's graph launches."""
    from hande_gb300.autotune import BatchTuner
    from hande_gb300.engine import Batch, Engine
    inst = batched_instances()
    engines = [Engine(s, cfg) for s, cfg, _ in inst]
    for e in engines:
        e.initial_distribution()
    batch = Batch(engines)
    reps = None
    for c in range(equil_cycles):
        batch.run_cycles(1)
        reps = [e.end_report() for e in engines]
    varying = sum(1 for rp in reps if rp.vary_shift[0])
    targets = sum(m["target"] for _, _, m in inst)
    walkers = sum(rp.nparticles[0] for rp in reps)
    states = sum(rp.nstates for rp in reps)
    tuned = None
    if tune:
        t0 = time.perf_counter()
        tuner = BatchTuner(batch, engines, trial_cycles=3)
        choice, base_ms, best_ms = tuner.tune()
        tuned = {"default_ms_per_cycle": base_ms, "tuned_ms_per_cycle": best_ms, "trials": len(tuner.table),
                 "classes": tuner.summary(), "search_s": time.perf_counter() - t0}
    batch.run_cycles(3)  # warm-up
    for e in engines:
        e.end_report()
    t0 = time.perf_counter()
    batch.run_cycles(steps)  # synchronises at the end
    dt = time.perf_counter() - t0
    reps = [e.end_report() for e in engines]
    dev_s = reps[0].device_ms * 1e-3  # every handle of the batch carries the batch's device time
    att = sum(rp.nattempts for rp in reps)
    flags = 0
    for rp in reps:
        flags |= rp.error_flags
    batch.close()
    for e in engines:
        e.close()
    return {"workload": BATCH_WORKLOAD, "instances": len(inst), "value": att / dev_s, "unit": "attempts/s",
            "ms_per_step": 1e3 * dev_s / steps, "steps": steps, "walkers": walkers, "states": int(states),
            "target_walkers": targets, "instances_shift_varying": varying, "equilibration_cycles": equil_cycles,
            "error_flags": flags, "dtype": "int64 walkers, f64", "launch_tuning": tuned,
            "host_wall_value": att / dt,
            "timing": "device: CUDA events around the batch's graph launches (hgpu_batch_run_cycles); "
                      "host_wall_value: host clock around the call"}


PRECISION_WORKLOAD = ("synthetic molecule M=48 nel=16 C1 (96 spin orbitals, 2-word determinants), heat-bath "
                      "excitation generator, initiator (threshold 3), real amplitudes, cutoff 0.01; FP32 spawning "
                      "(integrals, heat-bath weights, p_gen) against FP64 with the same seed")


def precision_study(target=1e8, tau=1e-4, ncycles=1, equil=100, reports=500, nsample=1 << 20, seed=2024,
                    max_grow=2000, cpu=True):
    """The mixed-precision engine against the FP64 engine (48 orbitals, 1e8 walkers).  The FP64
    engine grows the population from the reference determinant until the shift
    varies (target walkers) and equilibrates for `equil` reports; its list and
    state then seed both runs, so that the FP64 and FP32 engines start from the
    same list at the same iteration and draw the same random numbers.  Each runs
    `reports` reports of `ncycles` cycles.  One cycle per report: the shift
    is updated every cycle, so that once it varies the population overshoots
    the target by less than a factor of two (with five cycles per report and
    shift damping 0.05 it reached four times the target before the shift
    caught up); the lists are sized for four times the target.  Reported: the reblocked E_proj and
    shift of each run, their difference in units of the combined standard error,
    the reblocked per-report difference of the two runs' E_proj (paired: the
    shared random numbers cancel most of the noise until the runs drift apart),
    attempts/s of each, and the largest error of FP32 H_ij and p_gen over
    nsample excitations generated from list parents with the same streams.
    With cpu, the CPU restatement of the same calculation (FP64) on every host
    core, hash-partitioned as HANDE runs it (cpu_reference_rate), on a bounded
    sample grown from the reference determinant."""
    from hande_gb300 import analysis, systems
    from hande_gb300._abi import PREC_FP64, PREC_MIXED, make_config
    from hande_gb300.engine import Engine
    s = systems.synthetic_molecule(48, 16, seed=seed)
    out = {"workload": PRECISION_WORKLOAD, "target": target, "tau": tau, "ncycles": ncycles, "reports": reports}

    def config(prec):
        return make_config(s, tau=tau, init_pop=max(target / 1000.0, 100.0), target_population=target,
                           ncycles=ncycles, seed=77, real_amplitudes=True, spawn_cutoff=0.01, excit_gen="heat_bath",
                           initiator=True, initiator_threshold=3.0, precision=prec,
                           state_size=int(4 * target) + 100000, spawned_state_size=int(4 * target) + 100000)

    t0 = time.perf_counter()
    e = Engine(s, config(PREC_FP64))
    out["table_build_s"] = time.perf_counter() - t0
    e.initial_distribution()
    flags = 0
    t0 = time.perf_counter()
    for r in range(max_grow):  # until the shift varies
        rep = e.run_report()
        flags |= rep.error_flags
        if rep.vary_shift[0]:
            break
    out["growth_reports"] = r + 1
    for r in range(equil):
        rep = e.run_report()
        flags |= rep.error_flags
    out["growth_and_equilibration_s"] = time.perf_counter() - t0
    st, po, da = e.walkers()
    state = e.get_state()
    rng = np.random.default_rng(5)
    pick = rng.integers(0, st.shape[0], nsample)
    xs = (st[pick], np.ones(nsample, np.int64), int(state.iteration) + 1000)
    series = {}
    xres = {}
    for name, prec in (("fp64", PREC_FP64), ("fp32", PREC_MIXED)):
        if name == "fp32":
            e = Engine(s, config(prec))
            e.set_walkers(st, po, da)
            e.set_state(state)
        xres[name] = e.eval_excitations(*xs)
        num, d0, shift = [], [], []
        att, dev_ms = 0, 0.0
        for r in range(reports):
            rep = e.run_report()
            flags |= rep.error_flags
            if r % 100 == 0:
                sys.stderr.write("%s report %d Nw=%.4g states=%d shift=%.4f flags=%d\n" % (
                    name, r, rep.nparticles[0], rep.nstates, rep.shift[0], rep.error_flags))
            num.append(rep.proj_energy[0])
            d0.append(rep.D0_population[0])
            shift.append(rep.shift[0])
            att += rep.nattempts
            dev_ms += rep.device_ms
        E, err, opt = analysis.projected_energy(num, d0)
        S, serr, sopt = analysis.mean_error(shift)
        series[name] = (np.array(num), np.array(d0))
        out[name] = {"E_proj": E, "sigma": err, "opt_block": opt, "shift": S, "shift_sigma": serr,
                     "shift_opt_block": sopt, "attempts_per_s": att / (dev_ms * 1e-3),
                     "ms_per_cycle": dev_ms / (reports * ncycles), "walkers": rep.nparticles[0],
                     "states": int(rep.nstates)}
        e.close()
    r64, r32 = xres["fp64"], xres["fp32"]
    same = np.all(r32[0] == r64[0], axis=1) & (r32[3] == r64[3]) & (r64[3] == 1)
    dh = np.abs(r32[2][same] - r64[2][same])
    rel_h = dh / np.abs(r64[2][same])
    rel_p = np.abs(r32[1][same] - r64[1][same]) / np.abs(r64[1][same])
    big = np.abs(r64[2][same]) > 1e-3 * np.max(np.abs(r64[2][same]))
    out["excitations"] = {"sampled": nsample, "same_excitation": float(same.sum()) / max(int((r64[3] == 1).sum()), 1),
                          "max_rel_err_hij": float(rel_h.max()), "max_rel_err_hij_above_1e-3_of_max":
                          float(rel_h[big].max()), "max_abs_err_hij_over_max_hij":
                          float(dh.max() / np.max(np.abs(r64[2][same]))), "max_rel_err_pgen": float(rel_p.max())}
    d = out["fp32"]["E_proj"] - out["fp64"]["E_proj"]
    sig = float(np.hypot(out["fp32"]["sigma"], out["fp64"]["sigma"]))
    out["dE_proj"] = d
    out["dE_proj_over_sigma"] = d / sig if sig > 0 else None
    # Paired comparison: the runs share their start and random streams, so the
    # difference of E_proj = sum(num) / sum(D0) over the same block of reports
    # cancels much of the common noise.  Per-report ratios are not averaged (a
    # report with a small D0 gives an outlier); the reports are cut into
    # nblk consecutive blocks, each block's E_proj difference is formed from
    # its sums, and the blocks' mean and standard error are reported.
    nblk = 10
    m = (reports // nblk) * nblk
    if m >= nblk:
        def bsum(x):
            return x[:m].reshape(nblk, -1).sum(axis=1)
        (n64, z64), (n32, z32) = series["fp64"], series["fp32"]
        dd = bsum(n32) / bsum(z32) - bsum(n64) / bsum(z64)
        pm, perr = float(dd.mean()), float(dd.std(ddof=1) / np.sqrt(nblk))
        out["dE_proj_paired"] = {"blocks": nblk, "reports_per_block": m // nblk, "mean": pm, "sigma": perr,
                                 "over_sigma": pm / perr if perr > 0 else None}
    out["D0_mean"] = {k: float(np.mean(v[1])) for k, v in series.items()}
    out["fp32_speedup"] = out["fp32"]["attempts_per_s"] / out["fp64"]["attempts_per_s"]
    out["error_flags"] = flags
    if cpu:
        ncores = os.cpu_count() or 1
        tgt = float(os.environ.get("HGPU_REF_TARGET", REF_TARGET))
        ccfg = make_config(s, tau=tau, init_pop=tgt / 50.0, target_population=1e300, ncycles=5, seed=77,
                           real_amplitudes=True, spawn_cutoff=0.01, excit_gen="heat_bath", initiator=True,
                           initiator_threshold=3.0, precision=PREC_FP64, state_size=int(2 * tgt / ncores) + 100000,
                           spawned_state_size=int(3 * tgt / ncores) + 100000)
        t0 = time.perf_counter()
        rate, sec, walkers, states, grown, att = cpu_reference_rate(s, ccfg, ncores, tgt, 3, 1, 1)
        out["cpu_reference"] = {
            "value": rate, "unit": "attempts/s", "cores": ncores, "kind": "port", "ms_per_cycle": 1e3 * sec,
            "sample": "one FP64 calculation of the same system over %d host cores (threads as hash-partitioned "
                      "ranks), grown to %.3g walkers (%d states) in %d reports of 5 cycles; 3 cycles from that "
                      "list timed" % (ncores, walkers, states, grown),
            "wall_s": time.perf_counter() - t0}
    return out


HUBBARD_WORKLOAD = ("Hubbard model in momentum space, 2D 4x4 periodic, t=1, U=4, 10 electrons (ms=0), "
                    "integer walkers, 10 on the reference at the start, target 5e4, tau=0.005, shift damping 0.05, "
                    "mc_cycles 10 x 2000 reports (20000 iterations), FP64")


def hubbard_run(excit_gen="renorm", nreports=2000, seed=7):
    """The Hubbard 4x4 run as specified: the whole 20000-iteration run on the device,
    one report per host call; attempts/s and time per iteration over the
    reports after the shift starts varying (device time of the cycles), and
    the reblocked shift and E_proj of that part."""
    from hande_gb300 import analysis, systems
    from hande_gb300._abi import make_config
    from hande_gb300.engine import Engine
    s = systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0, t=1.0)
    cfg = make_config(s, tau=0.005, init_pop=10, target_population=5e4, ncycles=10, seed=seed, shift_damping=0.05,
                      excit_gen=excit_gen, state_size=2000000, spawned_state_size=2000000)
    e = Engine(s, cfg)
    e.initial_distribution()
    t0 = time.perf_counter()
    att = 0
    dev_ms = 0.0
    cycles = 0
    shift, num, d0 = [], [], []
    flags = 0
    for r in range(nreports):
        rep = e.run_report()
        flags |= rep.error_flags
        if rep.vary_shift[0]:
            att += rep.nattempts
            dev_ms += rep.device_ms
            cycles += 10
            shift.append(rep.shift[0])
            num.append(rep.proj_energy[0])
            d0.append(rep.D0_population[0])
    wall = time.perf_counter() - t0
    E, err, _ = analysis.projected_energy(num, d0) if len(num) > 32 else (None, None, None)
    S, serr, _ = analysis.mean_error(shift) if len(shift) > 32 else (None, None, None)
    e.close()
    return {"excit_gen": excit_gen, "iterations": 10 * nreports, "wall_s": wall, "error_flags": flags,
            "cycles_measured": cycles, "attempts_per_s": att / (dev_ms * 1e-3) if dev_ms > 0 else None,
            "ms_per_iteration": dev_ms / cycles if cycles else None,
            "wall_ms_per_iteration_whole_run": 1e3 * wall / (10 * nreports),
            "walkers": rep.nparticles[0], "states": int(rep.nstates),
            "E_proj": E, "E_proj_error": err, "shift": S, "shift_error": serr}


def semi_stoch_run(size, steps=10, warmup=3, target=1e7):
    """The 26-orbital cycle with a semi-stochastic 'high' space of `size`
    determinants (src/semi_stoch.F90): the walker list is grown as for the
    26-orbital line, moved into a second calculation whose space is built at its
    first cycle from that list, then whole cycles are timed from a snapshot
    taken after the build.  Returns the per-cycle device time, the phase split
    and the one-time cost of building the space."""
    from hande_gb300.engine import Engine
    s, cfg = system_and_config(target=target)
    a = Engine(s, cfg)
    a.initial_distribution()
    grow(a, target)
    st, po, da = a.walkers()
    a.close()
    cfg2 = type(cfg).from_buffer_copy(cfg)
    cfg2.semi_stoch_space = 1
    cfg2.semi_stoch_size = int(size)
    cfg2.semi_stoch_start_iter = 1
    b = Engine(s, cfg2)
    b.set_walkers(st, po, da)
    t0 = time.time()
    b.run_cycles(1)  # builds the space at the start of iteration 1, then one cycle
    r0 = b.end_report()
    build_s = time.time() - t0
    b.snapshot()
    for _ in range(max(warmup, 3)):
        b.snapshot(restore=True)
        b.run_cycles(1)
        b.end_report()
    dev_ms, attempts, flags = 0.0, 0, r0.error_flags
    for _ in range(steps):
        b.snapshot(restore=True)
        b.run_cycles(1)
        r = b.end_report()
        dev_ms += r.device_ms
        attempts += r.nattempts
        flags |= r.error_flags
    b.snapshot(restore=True)
    phases, counts = b.profile_cycle()
    b.close()
    if flags:
        raise RuntimeError("semi-stochastic run flagged errors (%d)" % flags)
    return {"workload": "26-orbital molecule cycle with a semi-stochastic 'high' space of %d determinants, built from the "
                        "grown %d-state list" % (size, st.shape[0]),
            "space_size": int(size), "steps": steps, "ms_per_step": dev_ms / steps,
            "attempts_per_s": attempts / (dev_ms / 1e3),
            "first_cycle_with_build_s": build_s, "phase_ms": phases, "cycle_counts": counts,
            "note": "the projection kernel runs inside the spawn phase (after k_spawn)"}


def device_free_bytes():
    rt = cudart()
    if rt is None:
        return None
    free, total = C.c_size_t(), C.c_size_t()
    if rt.cudaMemGetInfo(C.byref(free), C.byref(total)) != 0:
        return None
    return int(free.value)


def mol26_measure(steps, warmup, rank=0, cpu_seconds=10.0, parity=True):
    """The 26-orbital molecule (M = 26, 10 electrons, tau 1e-3, real amplitudes,
    FP64, ~1e7 walkers): attempts/s and iteration time over K replayed cycles,
    per-phase times, the rooflines, one cycle of the oracle on the same list
    (bit-exact comparison) and the one-core oracle's rate on it."""
    from hande_gb300.engine import Engine
    from hande_gb300.measure import roofline_figures
    s, cfg = system_and_config(target=1e7, seed_rng=7 + rank, ncycles=1)  # a step is one cycle
    eng = Engine(s, cfg)
    eng.initial_distribution()
    grown = grow(eng, 1e7)
    eng.snapshot()
    r = replay_steps(eng, steps, warmup)
    eng.snapshot(restore=True)
    phases, counts = eng.profile_cycle()
    roof, annih = roofline_figures(phases, counts, W=s.nwords, R=1, initiator=False, peaks=load_peaks())
    out = {"workload": WORKLOAD, "value": r["attempts"] / (r["dev_ms"] * 1e-3), "unit": "attempts/s",
           "ms_per_step": r["dev_ms"] / steps, "walkers": grown.nparticles[0], "states": int(grown.nstates),
           "attempts_per_step": r["attempts"] / steps, "phase_ms": phases, "cycle_counts": counts,
           "roofline": roof, "annihilation_roofline": annih}
    if parity:
        eng.snapshot(restore=True)
        st, po, da = eng.walkers()
        state = eng.get_state()
        out["parity"] = parity_cycle(s, cfg, st, po, da, state,
                                     "one cycle of the whole %d-state 26-orbital list" % st.shape[0])
        c = cpu_sample_on_state(st, po, da, cpu_seconds)
        out["cpu_baseline"] = {"value": c["attempts"] / c["seconds"], "unit": "attempts/s", "cores": 1,
                               "kind": "port", "sample": "CPU oracle, 1 core, %d whole cycle(s) of the %.3g-walker "
                                                         "list in %.1f s" % (c["cycles"], c["walkers"], c["seconds"])}
    eng.close()
    return out


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def eproj_stats(e):
    """Mean and standard error over the replayed cycles of each replica's
    one-cycle E_proj (the replays are independent draws from one list)."""
    return [(float(np.mean(e[:, q])), float(np.std(e[:, q], ddof=1) / np.sqrt(e.shape[0])))
            for q in range(e.shape[1])]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--large-total", type=float, default=5e8, help="walkers of both replicas in the headline list")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle legs (parity and cpu_baseline)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched measurement (128 Hubbard calculations)")
    ap.add_argument("--no-extra", action="store_true", help="skip the FP32 run and the 26-orbital line")
    ap.add_argument("--workload", default="large", choices=["large", "mol26", "hubbard", "precision"],
                    help="large: the headline line (default); mol26: the 26-orbital measurement alone; hubbard: "
                         "the Hubbard 4x4 run; precision: the mixed-precision study (one JSON line each)")
    ap.add_argument("--precision-target", type=float, default=1e8, help="precision study: target population")
    ap.add_argument("--precision-reports", type=int, default=500,
                    help="precision study: measured reports of each precision")
    ap.add_argument("--semi-stoch", type=int, default=0,
                    help="time the 26-orbital cycle with a semi-stochastic 'high' space of this size (one JSON line)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return
    if args.workload == "precision":
        if rank == 0:
            print(json.dumps(precision_study(target=args.precision_target, reports=args.precision_reports,
                                             cpu=not args.no_cpu)))
        return
    if args.workload == "hubbard":
        if rank == 0:
            print(json.dumps({"workload": HUBBARD_WORKLOAD, "renorm": hubbard_run("renorm"),
                              "no_renorm": hubbard_run("no_renorm")}))
        return
    if args.workload == "mol26":
        if rank == 0:
            print(json.dumps(mol26_measure(args.steps, args.warmup, cpu_seconds=args.cpu_seconds,
                                           parity=not args.no_cpu)))
        return
    if args.semi_stoch > 0:
        if rank == 0:
            print(json.dumps(semi_stoch_run(args.semi_stoch, steps=args.steps, warmup=args.warmup)))
        return

    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        td.init_process_group("nccl")
        dist = td

    from hande_gb300._abi import PREC_FP64, PREC_MIXED
    from hande_gb300.engine import Engine
    from hande_gb300.measure import roofline_figures
    s = large_system()
    main_cap, spawn_cap = int(0.6 * args.large_total), int(1.6 * args.large_total)
    cfg = large_config(s, PREC_FP64, main_cap, spawn_cap, init_pop=args.large_total / 500.0, seed=5 + rank)
    free0 = device_free_bytes()
    t0 = time.perf_counter()
    eng = Engine(s, cfg)
    eng.initial_distribution()
    grown, ngrow = grow_replicas(eng, args.large_total, label="fp64")
    grow_s = time.perf_counter() - t0
    hold_and_save(eng)
    held = None if free0 is None or device_free_bytes() is None else free0 - device_free_bytes()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    r64 = replay_steps(eng, args.steps, args.warmup, clocks=clocks, barrier=dist.barrier if dist else None)
    dev_ms, attempts = r64["dev_ms"], float(r64["attempts"])
    if dist:
        import torch
        t = torch.tensor([dev_ms, attempts], dtype=torch.float64, device="cuda")
        mx = t.clone()
        dist.all_reduce(mx[:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
        dev_ms, attempts = float(mx[0]), float(t[1])
    value = attempts / (dev_ms * 1e-3)

    # per-phase times of one cycle from the same list and the rooflines
    eng.snapshot(restore=True)
    phases, counts = eng.profile_cycle()
    roof, annih = roofline_figures(phases, counts, W=s.nwords, R=2, initiator=True, peaks=load_peaks())
    # end to end through the C ABI with host walker lists
    e2e = e2e_measure(eng, s.nwords, 2, args.e2e_steps, main_cap)
    parity = cpu = None
    # the step input on the host: the FP32 engine replays the same list
    eng.snapshot(restore=True)
    st, po, da = eng.walkers()
    state = eng.get_state()
    xs = x64 = None
    if rank == 0 and not args.no_extra:
        # FP64 excitations of 2^20 parents drawn from the list, for the FP32 comparison
        rng = np.random.default_rng(5)
        pick = rng.integers(0, st.shape[0], 1 << 20)
        xs = (st[pick], np.ones(1 << 20, np.int64), int(state.iteration) + 1000)
        x64 = eng.eval_excitations(*xs)
    if rank == 0 and not args.no_cpu:
        n = 50000
        i0 = max(0, (st.shape[0] - n) // 2)
        sl = slice(i0, i0 + n)
        pc = type(cfg).from_buffer_copy(cfg)
        pc.walker_length, pc.spawned_walker_length = 40 * n, 80 * n
        parity = parity_cycle(s, pc, st[sl], po[sl], da[sl], state,
                              "one cycle of a %d-state slice (from state %d) of the benchmark's own %d-state list, "
                              "the benchmark's iteration, shift and parameters (FP64)" % (n, i0, st.shape[0]))
        cpu = cpu_slice(s, cfg, st, po, da, state, 100000, args.cpu_seconds)
    eng.close()

    extra = {}
    if rank == 0 and not args.no_extra:
        # the FP32 engine on the same list: attempts/s, the replica (RDM)
        # energy of each replayed cycle against FP64's, and the FP32 matrix
        # elements and p_gen of the same 2^20 generated excitations
        cfg32 = large_config(s, PREC_MIXED, main_cap, spawn_cap, seed=5 + rank)
        e32 = Engine(s, cfg32)
        e32.set_walkers(st, po, da)
        e32.set_state(state)
        e32.snapshot()
        r32 = replay_steps(e32, args.steps, args.warmup)
        x32 = e32.eval_excitations(*xs)
        e32.close()
        same = np.all(x32[0] == x64[0], axis=1) & (x32[3] == x64[3]) & (x64[3] == 1)
        rel_h = np.abs(x32[2][same] - x64[2][same]) / np.abs(x64[2][same])
        rel_p = np.abs(x32[1][same] - x64[1][same]) / np.abs(x64[1][same])
        e64 = np.array(r64["rdm"])
        e32r = np.array(r32["rdm"])
        ok = len(e64) > 1 and len(e32r) == len(e64)

        def mse(x):
            return [float(np.mean(x)), float(np.std(x, ddof=1) / np.sqrt(len(x)))]

        extra["mixed_precision"] = {
            "value": r32["attempts"] / (r32["dev_ms"] * 1e-3), "unit": "attempts/s",
            "ms_per_step": r32["dev_ms"] / args.steps, "speedup_over_fp64": (r32["attempts"] / r32["dev_ms"]) / (
                r64["attempts"] / r64["dev_ms"]),
            "rdm_energy_one_cycle": {"fp64": mse(e64) if ok else None, "fp32": mse(e32r) if ok else None},
            # both engines replay the same iterations, hence the same random
            # streams: the paired difference isolates the FP32 arithmetic
            "dE_rdm_paired": mse(e32r - e64) if ok else None,
            "dE_rdm_over_sigma": (float(np.mean(e32r) - np.mean(e64)) /
                                  float(np.hypot(mse(e64)[1], mse(e32r)[1]))) if ok else None,
            "excitations": {"sampled": len(xs[0]), "same_excitation": float(same.mean()),
                            "max_rel_err_hij": float(rel_h.max()) if rel_h.size else None,
                            # relative errors of near-cancelling |H_ij| (a difference of two
                            # similar integrals) are large; against the largest |H_ij|:
                            "max_abs_err_hij_over_max_hij": float(np.max(np.abs(x32[2][same] - x64[2][same])) /
                                                                  np.max(np.abs(x64[2][same]))) if rel_h.size else None,
                            "max_rel_err_hij_above_1e-3_of_max": float(rel_h[np.abs(x64[2][same]) > 1e-3 * np.max(
                                np.abs(x64[2][same]))].max()) if rel_h.size else None,
                            "max_rel_err_pgen": float(rel_p.max()) if rel_p.size else None},
            "note": "FP32 H_ij and p_gen, FP64 K_ii, shift and estimators; both engines replay one-cycle reports "
                    "from the same walker list: the replica (variational, RDM) energy of each replayed cycle, "
                    "relative to H_00, mean and standard error over the K replays (dE_rdm_over_sigma treats the "
                    "two sets as independent, which overstates sigma); the FP32 H_ij and p_gen of 2^20 "
                    "excitations generated from list parents with the same random streams as FP64's"}
    del st, po, da
    if rank == 0 and not args.no_extra:
        extra["mol26"] = mol26_measure(args.steps, args.warmup, cpu_seconds=args.cpu_seconds,
                                           parity=not args.no_cpu)
    batched = None
    if rank == 0 and not args.no_batched:
        try:
            batched = batched_measure(args.steps)
        except Exception as exc:  # reported in the line; the headline numbers stand
            batched = {"workload": BATCH_WORKLOAD, "error": "%s: %s" % (type(exc).__name__, exc)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": LARGE_WORKLOAD, "walkers": grown.nparticles[0] + grown.nparticles[1],
                       "states": int(grown.nstates), "attempts_per_step": attempts / args.steps / world,
                       "growth_cycles": ngrow, "growth_s": grow_s, "device_bytes_held": held,
                       "main_capacity": main_cap, "spawn_capacity": spawn_cap, "l2": "inputs larger than L2",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": e2e,
            "gpu_launches": int(counts["launches_per_cycle"]) * args.steps,
            "roofline": roof,
            "annihilation_roofline": annih,
            "phase_ms": phases,
            "cycle_counts": counts,
            "clocks": r64["clocks"],
            "E_proj": [x[0] for x in eproj_stats(r64["eproj"])],
            "rdm_energy_one_cycle": [float(np.mean(r64["rdm"])), float(np.std(r64["rdm"], ddof=1) /
                                                                      np.sqrt(len(r64["rdm"])))]
            if len(r64["rdm"]) > 1 else None,
            "parity": parity,
            "cpu_baseline": cpu,
            "batched": batched,
        }
        line.update(extra)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
