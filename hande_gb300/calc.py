"""The fciqmc calculation driver: the report loop of do_fciqmc
(src/fciqmc.f90:276-470) around the GPU engine, with the option names of
HANDE's Lua interface (``qmc``/``fciqmc`` tables, src/lua_hande_calc.f90:304,
:1318-1331, :1549).

Per report the engine runs mc_cycles cycles on the device, then the host closes
the report (estimators, shift update) and prints a line with the columns of
write_qmc_report (src/qmc_io.f90:23-136)."""

from __future__ import annotations

import os
import sys
import time
from typing import Optional

from . import restart as restart_files
from ._abi import PREC_FP64, PREC_MIXED, make_config
from .engine import Engine
from .systems import System

QMC_KEYS = {
    "tau", "init_pop", "mc_cycles", "nreports", "state_size", "spawned_state_size", "rng_seed",
    "target_population", "real_amplitudes", "spawn_cutoff", "excit_gen", "pattempt_single",
    "pattempt_double", "pattempt_parallel", "power_pitzer_min_weight", "initiator", "initiator_threshold",
    "shift_damping", "vary_shift_from", "initial_shift", "precision",
    "shift_harmonic_forcing", "shift_harmonic_crit_damp", "shift_harmonic_forcing_two_stage",
    "reference_target", "vary_shift",
}
FCIQMC_KEYS = {"replica_tricks", "density_matrices", "density_matrix_report", "density_matrix_file",
               "quadrature_initiator"}
SEMI_STOCH_KEYS = {"space", "size", "start_iteration", "shift_start_iteration", "separate_annihilation", "ci_space"}
RESTART_KEYS = {"read", "write", "write_frequency"}


def _restart_id(v) -> Optional[int]:
    """read / write of the restart table: an id, or true for id 0 (the file
    names HANDE.RS.<id>.p<rank>.H5 of restart_info_t)."""
    if v is None or v is False:
        return None
    return 0 if v is True else int(v)


def semi_stoch_options(ss: Optional[dict]) -> dict:
    """The semi_stoch table of read_semi_stoch_in (src/lua_hande_calc.f90:1640-1721):
    space = 'high' with its size, or 'ci' with ci_space = {ex_level = n} (the
    calculation's reference); start_iteration (default 1); with
    shift_start_iteration the start waits for the shift (start_iteration =
    huge); separate_annihilation = false puts the projected amplitudes into
    the spawned list (combined annihilation).  'read' needs a HANDE HDF5 file;
    a ci_space with its own determinant is not provided."""
    if not ss:
        return {}
    unknown = set(ss) - SEMI_STOCH_KEYS
    if unknown:
        raise ValueError("unknown semi_stoch option(s): %s" % ", ".join(sorted(unknown)))
    if "space" not in ss:
        raise ValueError("Deterministic space not specified.")
    if ss["space"] not in ("high", "ci"):
        raise ValueError("semi_stoch space %r is not provided ('high', 'ci')" % ss["space"])
    out = dict(semi_stoch_start_iter=int(ss.get("start_iteration", 1)), semi_stoch_shift_iter=-1,
               semi_stoch_combined=0 if ss.get("separate_annihilation", True) else 1)
    if ss["space"] == "high":
        if "size" not in ss:
            raise ValueError("Target space size not given.")
        out.update(semi_stoch_space=1, semi_stoch_size=int(ss["size"]))
    else:
        ci = ss.get("ci_space") or {}
        if set(ci) - {"ex_level"} or int(ci.get("ex_level", -1)) < 0:
            raise ValueError("ci_space needs ex_level >= 0 (and no other key)")
        out.update(semi_stoch_space=4, semi_stoch_ci_level=int(ci["ex_level"]))
    if "shift_start_iteration" in ss:
        out["semi_stoch_start_iter"] = 2 ** 62
        out["semi_stoch_shift_iter"] = int(ss["shift_start_iteration"])
    return out


def _opts(qmc: dict, fciqmc_opts: Optional[dict]):
    unknown = set(qmc) - QMC_KEYS
    if unknown:
        raise ValueError("unknown qmc option(s): %s" % ", ".join(sorted(unknown)))
    fo = fciqmc_opts or {}
    unknown = set(fo) - FCIQMC_KEYS
    if unknown:
        raise ValueError("unknown fciqmc option(s): %s" % ", ".join(sorted(unknown)))
    for key in ("tau", "init_pop", "mc_cycles", "nreports"):
        if key not in qmc:
            raise ValueError("qmc.%s is required" % key)
    return fo


def harmonic_forcing(qmc: dict) -> float:
    """qs%shift_harmonic_forcing as init_qmc sets it (src/qmc.F90:193-208):
    shift_damping^2 / 4 (critical damping) with shift_harmonic_crit_damp.
    Otherwise it stays 0: init_qmc copies the input's shift_harmonic_forcing
    only when the state's value is already non-zero, which it never is there,
    so the option alone leaves the dynamics unchanged; the same here."""
    if qmc.get("shift_harmonic_crit_damp", False):
        return float(qmc.get("shift_damping", 0.05)) ** 2 / 4.0
    return 0.0


def config_from_options(system: System, qmc: dict, fciqmc_opts: Optional[dict] = None, reference=None,
                        semi_stoch: Optional[dict] = None):
    fo = _opts(qmc, fciqmc_opts)
    # reference_target: the target is the reference population (src/lua_hande_calc.f90:1412-1417)
    if "reference_target" in qmc and "target_population" in qmc:
        raise ValueError("Cannot provide both target_population and reference_target")
    target = float(qmc["reference_target"]) if "reference_target" in qmc else \
        float(qmc.get("target_population", 1e300))
    vsf = qmc.get("vary_shift_from", 0.0)
    prec = qmc.get("precision", "fp64")
    return make_config(
        system, tau=qmc["tau"], ncycles=int(qmc["mc_cycles"]), seed=int(qmc.get("rng_seed", 7)),
        init_pop=float(qmc["init_pop"]), target_population=target, target_reference="reference_target" in qmc,
        shift_damping=float(qmc.get("shift_damping", 0.05)), initial_shift=float(qmc.get("initial_shift", 0.0)),
        shift_harmonic_forcing=harmonic_forcing(qmc),
        vary_shift_from=0.0 if vsf == "proje" else float(vsf), vary_shift_from_proje=(vsf == "proje"),
        real_amplitudes=bool(qmc.get("real_amplitudes", False)), spawn_cutoff=float(qmc.get("spawn_cutoff", 0.01)),
        excit_gen=qmc.get("excit_gen", "renorm"), pattempt_single=float(qmc.get("pattempt_single", -1.0)),
        pattempt_double=float(qmc.get("pattempt_double", -1.0)),
        pattempt_parallel=float(qmc.get("pattempt_parallel", -1.0)),
        power_pitzer_min_weight=float(qmc.get("power_pitzer_min_weight", 0.01)),
        initiator=bool(qmc.get("initiator", False)),
        initiator_threshold=float(qmc.get("initiator_threshold", 3.0)),
        # density_matrices turns replica_tricks on (src/lua_hande_calc.f90:1569-1573)
        nspaces=2 if (fo.get("replica_tricks") or fo.get("density_matrices")) else 1,
        density_matrices=bool(fo.get("density_matrices", False)),
        quadrature_initiator=bool(fo.get("quadrature_initiator", True)),
        density_matrix_report=int(fo.get("density_matrix_report", 0)),
        precision=PREC_MIXED if prec in ("mixed", "fp32", PREC_MIXED) else PREC_FP64,
        state_size=int(qmc.get("state_size", -1000)), spawned_state_size=int(qmc.get("spawned_state_size", -500)),
        reference=reference, **semi_stoch_options(semi_stoch))


HEADER = (" iterations      Shift        \\sum H_0j N_j       N_0          # H psips    # states  "
          "# spawn_events  R_spawn   time")


def fciqmc(sys: System, qmc: dict, fciqmc: Optional[dict] = None, reference=None, out=None,
           comm_file: str = "HANDE.COMM", verbose: bool = True, semi_stoch: Optional[dict] = None,
           restart: Optional[dict] = None, directory: str = ".") -> dict:
    """Run FCIQMC on the GPU.  Returns {'reports': [...], 'engine': Engine}.

    A file named ``comm_file`` containing ``softexit = true`` in the working
    directory ends the calculation after the current report (calc_interact,
    src/interact.F90:11-188).

    ``restart`` takes the keys of HANDE's restart table
    (src/lua_hande_calc.f90, restart_info_t): ``read`` starts from the walker
    list and state of HANDE restart files HANDE.RS.<read>.p*.H5 in
    ``directory`` (written by HANDE or by this driver) instead of the initial
    distribution; ``write`` writes HANDE.RS.<write>.p0.H5 at the end, and every
    ``write_frequency`` iterations when that is set."""
    rs = dict(restart or {})
    bad = set(rs) - RESTART_KEYS
    if bad:
        raise ValueError("unknown restart options %s" % sorted(bad))
    read_id, write_id = _restart_id(rs.get("read")), _restart_id(rs.get("write"))
    read_paths = restart_files.restart_paths(read_id, directory) if read_id is not None else None
    if read_paths and reference is None:
        reference = restart_files.reference_of(read_paths, sys)
    cfg = config_from_options(sys, qmc, fciqmc, reference, semi_stoch)
    eng = Engine(sys, cfg)
    write_freq = int(rs.get("write_frequency", 0) or 0)
    write_path = None if write_id is None else os.path.join(directory, "HANDE.RS.%d.p0.H5" % write_id)
    if read_paths:
        restart_files.load_into(eng, read_paths)
    else:
        eng.initial_distribution()
        if cfg.shift_harmonic_forcing != 0.0 and not qmc.get("shift_harmonic_forcing_two_stage", False):
            # with harmonic forcing the shift varies from the start unless the
            # forcing waits for the target population (src/qmc.F90:209-212)
            st = eng.get_state()
            for q in range(eng.R):
                st.vary_shift[q] = 1
            eng.set_state(st)
    if "vary_shift" in qmc:
        # the input's vary_shift overrides everything else, a restart included; a
        # shift that does not vary starts from initial_shift (src/qmc.F90:881-893)
        st = eng.get_state()
        for q in range(eng.R):
            st.vary_shift[q] = int(bool(qmc["vary_shift"]))
            if not qmc["vary_shift"]:
                st.shift[q] = float(qmc.get("initial_shift", 0.0))
        eng.set_state(st)
    stream = out if out is not None else sys_stdout()
    if verbose:
        stream.write(HEADER + "\n")
    reports = []
    t0 = time.time()
    for ireport in range(int(qmc["nreports"])):
        rep = eng.run_report()
        t1 = time.time()
        row = rep.as_dict(eng.R)
        row["time"] = t1 - t0
        t0 = t1
        reports.append(row)
        if write_path and write_freq > 0 and row["iterations"] % write_freq == 0:
            restart_files.save_from(eng, write_path, report=row)
        if verbose:
            stream.write(" %10d  %14.8f  %16.8f  %12.4f  %14.4f  %10d  %10d  %8.4f  %7.4f\n" % (
                row["iterations"], row["Shift"][0], row["\\sum H_0j N_j"][0], row["N_0"][0], row["# H psips"][0],
                row["# states"], row["# spawn_events"], row["R_spawn"], row["time"]))
        if row["error_flags"]:
            if verbose:
                stream.write("# Error: walker list full (flags %d); exiting at the end of this report.\n"
                             % row["error_flags"])
            break
        if _softexit(comm_file):
            if verbose:
                stream.write("# Soft exit requested through %s.\n" % comm_file)
            break
    if write_path:
        restart_files.save_from(eng, write_path, report=reports[-1] if reports else None)
    fo = fciqmc or {}
    if fo.get("density_matrices"):
        rdm = eng.rdm()
        if rdm is not None and reports and "RDM trace" in reports[-1]:
            write_final_rdm(rdm, sys.nel, sys.nbasis, fo.get("density_matrix_file", "RDM"), stream if verbose else None)
            if verbose:
                stream.write(" # Final energy from RDM  %17.10e\n" %
                             (reports[-1]["RDM energy num."] / reports[-1]["RDM trace"]))
    return {"reports": reports, "engine": eng}


def write_final_rdm(rdm, nel: int, nbasis: int, filename: str, comment=None):
    """write_final_rdm (src/replica_rdm.F90:266-328): normalise the trace to
    nel (nel - 1) / 2 (normalise_rdm), make the RDM Hermitian
    (check_hermiticity, reporting the deviation) and write the elements above
    depsilon as `i j k l value` with 1-based spin orbitals i < j, k < l."""
    import numpy as np
    r = np.array(rdm, dtype=float)
    r = r * nel * (nel - 1) * 0.5 / np.trace(r)
    iu = np.triu_indices(r.shape[0], 1)
    err = np.abs(r[iu] - r.T[iu])
    if comment is not None:
        comment.write(" # Maximum deviation from Hermiticity is: %17.10e\n" % (err.max() if err.size else 0.0))
        comment.write(" # Average deviation from Hermiticity is: %17.10e\n" % (err.mean() if err.size else 0.0))
    r = 0.5 * (r + r.T)
    with open(filename, "w") as fh:
        for i in range(nbasis):
            for j in range(i + 1, nbasis):
                row = j * (j - 1) // 2 + i
                for k in range(nbasis):
                    for l in range(k + 1, nbasis):
                        v = r[row, l * (l - 1) // 2 + k]
                        if abs(v) > 1e-12:
                            fh.write("%4d%4d%4d%4d  %24.12E\n" % (i + 1, j + 1, k + 1, l + 1, v))
    return r


def _softexit(path: str) -> bool:
    if not os.path.exists(path):
        return False
    try:
        txt = open(path).read().lower().replace(" ", "")
    except OSError:
        return False
    if "softexit=true" in txt:
        try:
            os.remove(path)
        except OSError:
            pass
        return True
    return False


def sys_stdout():
    return sys.stdout
