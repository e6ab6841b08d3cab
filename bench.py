"""Benchmark: FCIQMC spawn attempts/s and iteration time on one GB300.

Workload (one "step" = one FCIQMC Monte Carlo cycle): the synthetic molecular
Hamiltonian with 26 spatial orbitals and 10 electrons (C1, ms=0), real
amplitudes (2^-31 fixed point), spawn cutoff 0.01, uniform excitation
generator with p_double = 0.9, tau = 1e-3, FP64, target population 1e7.  The
population is grown from the reference determinant until the shift varies
(untimed), then W warm-up and K timed cycles run on the device.

  value      spawn attempts/s over the K timed cycles, device-timed with CUDA
             events on the engine's stream (the main and spawned lists,
             >= 200 MB each, exceed the 129 MB L2 between cycles)
  e2e        the same metric through the C ABI with host-resident walker
             lists: upload (pinned host -> device), one cycle, download
  roofline   HBM roofline of the dominant kernel (spawning) and of the
             annihilation phases (sort + self-annihilation + merge)
  cpu_baseline  the CPU oracle (C restatement of HANDE's cycle) on a bounded
             sample of the same workload

--impl reference times the CPU restatement of the reference algorithm on all
host cores (the reference itself, Fortran + MPI + Lua, cannot be built here).
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
WORKLOAD = ("config2: synthetic molecule M=26 nel=10 C1, real amplitudes, cutoff 0.01, uniform renorm p_double=0.9, "
            "tau=1e-3, ~1e7 walkers, FP64; each step = one full cycle on the same device-grown walker list")


def system_and_config(target=1e7, seed_ham=2024, seed_rng=7, cap_main=None, cap_spawn=None):
    from hande_gb300 import systems
    from hande_gb300._abi import make_config
    s = systems.synthetic_molecule(26, 10, seed=seed_ham)
    cm = cap_main or int(4 * target) + 200000
    cs = cap_spawn or int(4 * target) + 200000
    cfg = make_config(s, tau=1e-3, init_pop=10, target_population=target, ncycles=10, seed=seed_rng,
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


def cpu_sample(seconds=15.0, target=2e5, seed=7):
    """The oracle on a bounded sample of the same workload: grow to `target`
    walkers, then time whole cycles for about `seconds` s."""
    from oracle.pyoracle import Oracle
    s, cfg = system_and_config(target=target, seed_rng=seed, cap_main=int(20 * target), cap_spawn=int(40 * target))
    o = Oracle(s, cfg)
    o.initial_distribution()
    for _ in range(300):  # grow cycle by cycle up to the sample size
        o.run_cycles(1)
        if o.end_report().nparticles[0] >= target:
            break
    a0 = o.total_attempts()
    t0 = time.perf_counter()
    ncyc = 0
    while time.perf_counter() - t0 < seconds:
        o.run_cycles(1)
        ncyc += 1
    dt = time.perf_counter() - t0
    att = o.total_attempts() - a0
    rep = o.end_report()
    return {"attempts": att, "seconds": dt, "cycles": ncyc, "walkers": rep.nparticles[0],
            "states": rep.nstates}


def cpu_sample_on_state(states, pops, dat, seconds=10.0, seed=7):
    """The oracle timed on whole cycles of the engine's own walker list."""
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


def _cpu_worker(args):
    seconds, target, seed = args
    return cpu_sample(seconds, target, seed)


def reference_arm(args):
    """CPU restatement of HANDE's FCIQMC cycle on every host core: one
    independent calculation per core (HANDE runs one MPI rank per core)."""
    import multiprocessing as mp
    ncores = os.cpu_count() or 1
    seconds = float(os.environ.get("HGPU_REF_SECONDS", "20"))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(ncores) as pool:
        res = pool.map(_cpu_worker, [(seconds, 2e5, 7 + k) for k in range(ncores)])
    wall = time.perf_counter() - t0
    att = sum(r["attempts"] for r in res)
    rate = att / max(r["seconds"] for r in res)
    ms_per_cycle = 1e3 * np.mean([r["seconds"] / max(r["cycles"], 1) for r in res])
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "attempts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_cycle, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": "per core: grow to 2e5 walkers, time whole cycles %.0f s" % seconds,
                   "parallelism": "one independent calculation per host core"},
        "cpu_baseline": {"value": rate, "unit": "attempts/s", "cores": ncores, "kind": "port",
                         "sample": "%d cores x %.0f s of cycles at ~2e5 walkers (CPU restatement of HANDE's cycle)"
                                   % (ncores, seconds)},
        "e2e": {"value": rate, "unit": "attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line))


BATCH_WORKLOAD = ("config4: 128 independent Hubbard k-space calculations (2D periodic LxL, L in 3..6, "
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


def batched_measure(steps, equil_cycles=150):
    """config 4: every instance starts with its target population on the
    reference determinant; `equil_cycles` untimed cycles (a report after each,
    so that the shift acts every cycle) spread it out, then `steps` batch
    cycles are timed (one graph launch each for all instances)."""
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
    batch.run_cycles(3)  # warm-up
    for e in engines:
        e.end_report()
    t0 = time.perf_counter()
    batch.run_cycles(steps)  # synchronises at the end
    dt = time.perf_counter() - t0
    reps = [e.end_report() for e in engines]
    att = sum(rp.nattempts for rp in reps)
    flags = 0
    for rp in reps:
        flags |= rp.error_flags
    batch.close()
    for e in engines:
        e.close()
    return {"workload": BATCH_WORKLOAD, "instances": len(inst), "value": att / dt, "unit": "attempts/s",
            "ms_per_step": 1e3 * dt / steps, "steps": steps, "walkers": walkers, "states": int(states),
            "target_walkers": targets, "instances_shift_varying": varying, "equilibration_cycles": equil_cycles,
            "error_flags": flags, "dtype": "int64 walkers, f64",
            "timing": "host wall clock around hgpu_batch_run_cycles (graph launches and the final synchronisation)"}


PRECISION_WORKLOAD = ("config3: synthetic molecule M=48 nel=16 C1 (96 spin orbitals, 2-word determinants), heat-bath "
                      "excitation generator, initiator (threshold 3), real amplitudes, cutoff 0.01; FP32 spawning "
                      "(integrals, heat-bath weights, p_gen) against FP64 with the same seed")


def precision_study(target=2e5, tau=5e-5, equil=100, reports=600, nsample=1 << 20, seed=2024, max_grow=600):
    """config 3: the mixed-precision engine against the FP64 engine on the same
    seed -- the largest relative error of FP32 H_ij and p_gen over nsample
    generated excitations, the reblocked E_proj of both runs and their
    difference in units of the combined standard error, and the attempts/s of
    each."""
    from hande_gb300 import analysis, systems
    from hande_gb300._abi import PREC_FP64, PREC_MIXED, make_config
    from hande_gb300.engine import Engine
    s = systems.synthetic_molecule(48, 16, seed=seed)
    out = {"workload": PRECISION_WORKLOAD, "target": target, "tau": tau}
    res = {}
    for name, prec in (("fp64", PREC_FP64), ("fp32", PREC_MIXED)):
        cfg = make_config(s, tau=tau, init_pop=2000, target_population=target, ncycles=10, seed=77,
                          real_amplitudes=True, spawn_cutoff=0.01, excit_gen="heat_bath", initiator=True,
                          initiator_threshold=3.0, precision=prec, state_size=int(20 * target) + 100000,
                          spawned_state_size=int(20 * target) + 100000)
        t0 = time.perf_counter()
        e = Engine(s, cfg)
        build_s = time.perf_counter() - t0
        e.initial_distribution()
        num, d0 = [], []
        att = 0
        dev_ms = 0.0
        flags = 0
        grown = 0
        for r in range(max_grow):  # until the shift varies
            rep = e.run_report()
            flags |= rep.error_flags
            grown = r + 1
            if rep.vary_shift[0]:
                break
        for r in range(equil + reports):
            rep = e.run_report()
            flags |= rep.error_flags
            if r % 50 == 0:
                sys.stderr.write("%s report %d Nw=%.4g states=%d shift=%.4f flags=%d\n" % (
                    name, r, rep.nparticles[0], rep.nstates, rep.shift[0], rep.error_flags))
            if r >= equil:
                num.append(rep.proj_energy[0])
                d0.append(rep.D0_population[0])
                att += rep.nattempts
                dev_ms += rep.device_ms
        E, err, opt = analysis.projected_energy(num, d0)
        res[name] = {"E_proj": E, "sigma": err, "opt_block": opt, "attempts_per_s": att / (dev_ms * 1e-3),
                     "growth_reports": grown, "reports": reports,
                     "walkers": rep.nparticles[0], "states": int(rep.nstates), "error_flags": flags,
                     "table_build_s": build_s}
        res[name + "_engine"] = e
    # generated excitations of the same parents, FP32 against FP64
    e64, e32 = res.pop("fp64_engine"), res.pop("fp32_engine")
    st, po, _ = e64.walkers()
    rng = np.random.default_rng(5)
    pick = rng.integers(0, st.shape[0], nsample)
    parents, pp = st[pick], np.ones(nsample, np.int64)
    r64 = e64.eval_excitations(parents, pp, 3)
    r32 = e32.eval_excitations(parents, pp, 3)
    same = np.all(r32[0] == r64[0], axis=1) & (r32[3] == r64[3]) & (r64[3] == 1)
    rel_h = np.abs(r32[2][same] - r64[2][same]) / np.abs(r64[2][same])
    rel_p = np.abs(r32[1][same] - r64[1][same]) / np.abs(r64[1][same])
    big = np.abs(r64[2][same]) > 1e-3 * np.max(np.abs(r64[2][same]))
    out.update(res)
    out["excitations"] = {"sampled": nsample, "same_excitation": float(same.sum()) / max(int((r64[3] == 1).sum()), 1),
                          "max_rel_err_hij": float(rel_h.max()), "max_rel_err_hij_above_1e-3_of_max":
                          float(rel_h[big].max()), "max_rel_err_pgen": float(rel_p.max())}
    d = res["fp32"]["E_proj"] - res["fp64"]["E_proj"]
    sig = float(np.hypot(res["fp32"]["sigma"], res["fp64"]["sigma"]))
    out["dE_proj"] = d
    out["dE_proj_over_sigma"] = d / sig if sig > 0 else None
    e64.close()
    e32.close()
    return out


HUBBARD_WORKLOAD = ("config1: Hubbard model in momentum space, 2D 4x4 periodic, t=1, U=4, 10 electrons (ms=0), "
                    "integer walkers, 10 on the reference at the start, target 5e4, tau=0.005, shift damping 0.05, "
                    "mc_cycles 10 x 2000 reports (20000 iterations), FP64")


def hubbard_run(excit_gen="renorm", nreports=2000, seed=7):
    """config 1 as specified: the whole 20000-iteration run on the device,
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


LARGE_WORKLOAD = ("config5: synthetic molecule M=64 nel=20 ms=0 C1 (two-word determinants, 128-bit rank keys), "
                  "initiator FCIQMC (threshold 3) with 2 replicas and the replica 2-RDM (variational energy), real "
                  "amplitudes, spawn cutoff 0.01, uniform renorm generator (p_double 0.9), FP32 matrix elements and "
                  "p_gen, FP64 estimators, grown on the device to ~5e8 walkers in total, shift from E_proj")


def semi_stoch_run(size, steps=10, warmup=3, target=1e7):
    """The config-2 cycle with a semi-stochastic 'high' space of `size`
    determinants (src/semi_stoch.F90): the walker list is grown as for the
    headline line, moved into a second calculation whose space is built at its
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
    return {"workload": "config2 cycle with a semi-stochastic 'high' space of %d determinants, built from the "
                        "grown %d-state list" % (size, st.shape[0]),
            "space_size": int(size), "steps": steps, "ms_per_step": dev_ms / steps,
            "attempts_per_s": attempts / (dev_ms / 1e3),
            "first_cycle_with_build_s": build_s, "phase_ms": phases, "cycle_counts": counts,
            "note": "the projection kernel runs inside the spawn phase (after k_spawn)"}


def large_replica_run(target_total=5e8, tau=2e-4, cycles=5, seed=2024, max_grow=60):
    """config 5: one large replica calculation, measured like the headline
    step -- grown on the device (shift held at 0) until the two replicas hold
    about target_total walkers together; then the shifts are set varying (the
    condition for accumulating the replica 2-RDM), the walker list is saved on
    the device, and each of `cycles` reports of one cycle starts from it
    (restored device to device, untimed) with the RDM accumulating:
    attempts/s, time per cycle, memory held, E_proj and the RDM (variational)
    energy of each cycle."""
    from hande_gb300 import systems
    from hande_gb300._abi import PREC_MIXED, make_config
    from hande_gb300.engine import Engine
    s = systems.synthetic_molecule(64, 20, seed=seed)
    main_cap, spawn_cap = int(0.6 * target_total), int(1.6 * target_total)
    cfg = make_config(s, tau=tau, init_pop=1e6, target_population=1e300, ncycles=1, seed=5,
                      real_amplitudes=True, spawn_cutoff=0.01, excit_gen="renorm",
                      pattempt_single=0.1, pattempt_double=0.9, initiator=True, initiator_threshold=3.0,
                      nspaces=2, precision=PREC_MIXED, density_matrices=True, density_matrix_report=0,
                      state_size=main_cap, spawned_state_size=spawn_cap)
    free0 = device_free_bytes()
    t0 = time.perf_counter()
    e = Engine(s, cfg)
    e.initial_distribution()
    setup_s = time.perf_counter() - t0
    flags = 0
    grown = 0
    last = None
    for r in range(max_grow):
        rep = e.run_report()
        flags |= rep.error_flags
        grown = r + 1
        tot = rep.nparticles[0] + rep.nparticles[1]
        sys.stderr.write("config5 grow %d Nw=%.4g+%.4g states=%d flags=%d\n" % (
            r, rep.nparticles[0], rep.nparticles[1], rep.nstates, rep.error_flags))
        # stop at the target, or before a cycle that would overshoot it by 20 %
        g = tot / last if last else 1.0
        if flags or tot >= 0.9 * target_total or tot * g > 1.2 * target_total:
            break
        last = tot
    st = e.get_state()
    st.vary_shift[0] = st.vary_shift[1] = 1
    e.set_state(st)
    e.snapshot()
    held = None if free0 is None or device_free_bytes() is None else free0 - device_free_bytes()
    att = 0
    dev_ms = 0.0
    rdm = []
    walkers = None
    for c in range(cycles):
        e.snapshot(restore=True)
        rep = e.run_report()
        flags |= rep.error_flags
        att += rep.nattempts
        dev_ms += rep.device_ms
        if rep.rdm_trace:
            rdm.append(rep.rdm_energy / rep.rdm_trace)
        sys.stderr.write("config5 cycle %d attempts=%d ms=%.1f flags=%d\n" % (
            c, rep.nattempts, rep.device_ms, rep.error_flags))
    # one more cycle from the same list with per-phase device times and list sizes
    e.snapshot(restore=True)
    phases, counts = e.profile_cycle()
    out = {"workload": LARGE_WORKLOAD, "tau": tau, "main_capacity": main_cap, "spawn_capacity": spawn_cap,
           "device_bytes_held": held, "setup_s": setup_s, "growth_cycles": grown, "cycles": cycles,
           "error_flags": flags, "input_walkers_total": tot, "input_states": int(counts["N"]),
           "phase_ms": phases, "cycle_counts": counts,
           "attempts_per_cycle": att / cycles,
           "value": att / (dev_ms * 1e-3) if dev_ms > 0 else None, "unit": "attempts/s",
           "ms_per_cycle": dev_ms / cycles,
           "E_proj": [rep.proj_energy[q] / rep.D0_population[q] for q in range(2)],
           "rdm_energy_per_cycle": rdm,
           "note": "each timed cycle starts from the same device-grown ~%.2g-walker list (saved and restored on "
                   "the device, untimed) as one report whose RDM gives one replica (variational) energy; "
                   "energies relative to the reference determinant's H_00" % tot}
    e.close()
    return out


def device_free_bytes():
    rt = cudart()
    if rt is None:
        return None
    free, total = C.c_size_t(), C.c_size_t()
    if rt.cudaMemGetInfo(C.byref(free), C.byref(total)) != 0:
        return None
    return int(free.value)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--target", type=float, default=1e7)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (config 4) measurement")
    ap.add_argument("--config", type=int, default=2,
                    help="2: the headline line (default); 1: the Hubbard 4x4 run of config 1; 3: the "
                         "mixed-precision study of config 3; 5: the large replica run of config 5 (one JSON line each)")
    ap.add_argument("--large-total", type=float, default=5e8, help="config 5: total walkers of both replicas")
    ap.add_argument("--semi-stoch", type=int, default=0,
                    help="time the config-2 cycle with a semi-stochastic 'high' space of this size (one JSON line)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return
    args.warmup = max(args.warmup, 3)
    if args.config == 3:
        if rank == 0:
            print(json.dumps(precision_study()))
        return
    if args.config == 1:
        if rank == 0:
            print(json.dumps({"workload": HUBBARD_WORKLOAD, "renorm": hubbard_run("renorm"),
                              "no_renorm": hubbard_run("no_renorm")}))
        return
    if args.config == 5:
        if rank == 0:
            print(json.dumps(large_replica_run(target_total=args.large_total, cycles=args.steps)))
        return
    if args.semi_stoch > 0:
        if rank == 0:
            print(json.dumps(semi_stoch_run(args.semi_stoch, steps=args.steps, warmup=args.warmup,
                                            target=args.target)))
        return

    cpu = None
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        td.init_process_group("nccl")
        dist = td

    from hande_gb300.engine import Engine
    s, cfg = system_and_config(target=args.target, seed_rng=7 + rank)
    eng = Engine(s, cfg)
    eng.initial_distribution()
    grown = grow(eng, args.target, verbose=bool(os.environ.get("HGPU_BENCH_VERBOSE")))
    # the step input: this walker list, restored (device to device, untimed)
    # before every cycle
    eng.snapshot()
    for _ in range(args.warmup):
        eng.snapshot(restore=True)
        eng.run_cycles(1)
    eng.end_report()

    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    if dist:
        dist.barrier()
    clocks.start()
    time.sleep(0.3)
    dev_ms = 0.0
    attempts = 0
    flags = 0
    for _ in range(args.steps):
        eng.snapshot(restore=True)
        eng.run_cycles(1)  # device-timed with events on the engine stream; synchronises
        r1 = eng.end_report()
        dev_ms += r1.device_ms
        attempts += r1.nattempts
        flags |= r1.error_flags
    clk = clocks.stop()
    rep = grown
    if flags:
        raise RuntimeError("walker list overflow during the timed cycles (flags %d)" % flags)
    if dist:
        import torch
        t = torch.tensor([dev_ms, float(attempts)], dtype=torch.float64, device="cuda")
        mx = t.clone()
        dist.all_reduce(mx[:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
        dev_ms, attempts = float(mx[0]), float(t[1])
    value = attempts / (dev_ms * 1e-3)
    ms_per_step = dev_ms / args.steps

    # per-phase times of one cycle and the HBM roofline figures
    eng.snapshot(restore=True)
    phases, counts = eng.profile_cycle()
    from hande_gb300.measure import roofline_figures
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    roof, annih = roofline_figures(phases, counts, W=s.nwords, R=1, initiator=False, peaks=peaks)

    # end to end through the C ABI with host-resident walker lists
    rt = cudart()
    eng.snapshot(restore=True)
    st, po, da = eng.walkers()
    n0 = st.shape[0]
    cap = int(n0 * 4) + 1000
    hst, _ = pinned_array(rt, (cap, s.nwords), np.int64)
    hpo, _ = pinned_array(rt, (cap, 1), np.int64)
    hda, _ = pinned_array(rt, (cap,), np.float64)
    ost, _ = pinned_array(rt, (cap, s.nwords), np.int64)
    opo, _ = pinned_array(rt, (cap, 1), np.int64)
    oda, _ = pinned_array(rt, (cap,), np.float64)
    hst[:n0] = st
    hpo[:n0] = po
    hda[:n0] = da
    n = n0
    from hande_gb300.engine import _p
    L = eng.L
    h2d = d2h = 0
    e_att = 0
    eng.end_report()
    t_up = t_cyc = t_down = 0.0
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        n = n0  # every step starts from the same host walker list
        ta = time.perf_counter()
        eng._check(L.hgpu_upload_walkers(eng.h, _p(hst, C.c_int64), _p(hpo, C.c_int64), _p(hda, C.c_double), n),
                   "upload")
        h2d += n * (8 * s.nwords + 8 + 8)
        tb = time.perf_counter()
        eng.run_cycles(1)
        tc = time.perf_counter()
        m = C.c_int64()
        eng._check(L.hgpu_download_walkers(eng.h, _p(ost, C.c_int64), _p(opo, C.c_int64), _p(oda, C.c_double),
                                           cap, C.byref(m)), "download")
        d2h += m.value * (8 * s.nwords + 8 + 8)
        t_up += tb - ta
        t_cyc += tc - tb
        t_down += time.perf_counter() - tc
    e2e_s = time.perf_counter() - t0
    e_rep = eng.end_report()
    e_att = e_rep.nattempts
    e2e = {"value": e_att / e2e_s, "unit": "attempts/s", "h2d_bytes_per_step": h2d // args.e2e_steps,
           "d2h_bytes_per_step": d2h // args.e2e_steps,
           "note": "per step: hgpu_upload_walkers from pinned host memory, one cycle, hgpu_download_walkers",
           "host_ms_per_step": {"upload": 1e3 * t_up / args.e2e_steps, "cycle": 1e3 * t_cyc / args.e2e_steps,
                                "download": 1e3 * t_down / args.e2e_steps}}

    batched = None
    if rank == 0 and not args.no_batched:
        eng.close()
        try:
            batched = batched_measure(args.steps)
        except Exception as exc:  # reported in the line; the config-2 numbers stand
            batched = {"workload": BATCH_WORKLOAD, "error": "%s: %s" % (type(exc).__name__, exc)}

    if rank == 0 and not args.no_cpu:
        # the oracle on whole cycles of the same (device-grown) walker list, 1 core
        r = cpu_sample_on_state(st, po, da, args.cpu_seconds)
        cpu = {"value": r["attempts"] / r["seconds"], "unit": "attempts/s", "cores": 1, "kind": "port",
               "sample": "CPU oracle, 1 core, %d whole cycle(s) in %.1f s on the benchmark's own %.3g-walker list"
                         % (r["cycles"], r["seconds"], r["walkers"])}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "walkers": rep.nparticles[0], "states": int(rep.nstates),
                       "attempts_per_step": attempts / args.steps / world, "l2": "inputs larger than L2",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": e2e,
            "gpu_launches": int(counts["launches_per_cycle"]) * args.steps,
            "roofline": roof,
            "annihilation_roofline": annih,
            "phase_ms": phases,
            "cycle_counts": counts,
            "clocks": clk,
            "cpu_baseline": cpu,
            "batched": batched,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
