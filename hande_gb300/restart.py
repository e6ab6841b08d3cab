"""HANDE restart files for the device engine: read the walker list and the
calculation state of a HANDE FCIQMC restart (HANDE.RS.<id>.p<rank>.H5, one
file per MPI rank) into an engine, and write an engine's list and state as a
restart file that HANDE reads back (src/restart_hdf5.F90).

Reading follows read_restart_hdf5 (src/restart_hdf5.F90:554-933):
- determinants: 32-bit words are joined pairwise into the engine's 64-bit
  words, low word first, the high half cleared when their number is odd
  (bit_string_32_to_64, src/restart_utils.F90:480-505); the words of the
  information string, if any, are dropped;
- populations: int32 or int64, rescaled from the file's 'population scale
  factor' to the engine's fixed-point factor by an integer multiply or divide
  (change_pop_scaling_64, src/restart_utils.F90:454-478); a file without the
  factor keeps the engine's;
- the ranks' lists are merged and sorted in HANDE's order (the last word most
  significant), as a restart onto another number of processors re-sorts;
- data(1, :) is K_ii = H_ii - H_00;
- qmc/state: ncycles, shift, vary shift (false when absent); qmc/psips/total
  population is the population the next shift update compares against.

Writing follows dump_restart_hdf5 (src/restart_hdf5.F90:307-552) with restart
version 3, one rank, 64-bit determinant words and the datasets that
read_restart_hdf5 requires or reads when present.  The engine draws from
counter-based Philox streams, not dSFMT, so the rng group is written empty: a
HANDE calculation restarted from the file seeds its generator afresh, as it
does for any restart file without an rng state.  The calc type is
fciqmc_calc, which HANDE sets for every FCIQMC calculation
(src/lua_hande_calc.f90:399); nprocs is 1, and HANDE restarts on a different
number of processes only from files its redistribute step rewrote
(src/restart_hdf5.F90:663-666): `redistribute {nprocs = N, read = id, write = id2}`.
"""

import glob
import os
import re
import time
import uuid as uuidlib

import numpy as np

from . import hdf5lite

RESTART_VERSION = 3
FCIQMC_CALC = 4  # fciqmc_calc (src/calc.F90:35)


def restart_paths(read_id, directory="."):
    """HANDE.RS.<id>.p<rank>.H5 for every rank, rank order (restart_info_t's
    file names, src/restart_hdf5.F90:112-130)."""
    pat = os.path.join(directory, "HANDE.RS.%d.p*.H5" % read_id)
    paths = glob.glob(pat)
    if not paths:
        raise FileNotFoundError("no restart files %s" % pat)
    rank = lambda p: int(re.search(r"\.p(\d+)\.H5$", p).group(1))
    return sorted(paths, key=rank)


def _words64(dets, i0_length, nbasis, info_len):
    """Determinant words of a restart (n, words) as the engine's 64-bit words (n, W)."""
    dets = np.asarray(dets)
    n = dets.shape[0]
    W = (nbasis + 63) // 64
    if i0_length == 64:
        return dets[:, :W].astype(np.int64)
    if i0_length != 32:
        raise ValueError("i0_length %d" % i0_length)
    nb = (nbasis + 31) // 32 if nbasis else dets.shape[1] - info_len
    w32 = dets[:, :nb].astype(np.int64) & 0xFFFFFFFF
    if nb % 2:
        w32 = np.concatenate([w32, np.zeros((n, 1), np.int64)], axis=1)
    out = (w32[:, 0::2] | (w32[:, 1::2] << 32)).astype(np.int64)
    return out[:, :W] if nbasis else out


def _rescale(pops, old, new):
    pops = np.asarray(pops, dtype=np.int64)
    if old < new:
        return pops * (new // old)
    if old > new:
        # Fortran integer division truncates toward zero
        q = old // new
        return np.sign(pops) * (np.abs(pops) // q)
    return pops


def _sort_order(states):
    """Indices that sort (n, W) 64-bit words ascending, the last word most
    significant, compared unsigned (src/bit_utils.F90:452-478)."""
    u = states.view(np.uint64)
    return np.lexsort(tuple(u[:, w] for w in range(u.shape[1])))


def read(paths, nbasis, nspaces, real_factor):
    """Merge the restart files of every rank.  Returns a dict: states (n, W)
    int64, pops (n, nspaces) int64 in the engine's fixed point, kii (n,),
    iteration, shift, vary_shift, nparticles_old (per space), reference
    (W words), proj_energy and D0_population (per space, when present),
    restart_version."""
    if isinstance(paths, (str, os.PathLike)):
        paths = [paths]
    files = [hdf5lite.read(p) for p in paths]
    f0 = files[0]
    i0 = int(f0["/metadata/i0_length"])
    version = int(f0["/metadata/restart version"])
    nbasis_file = int(f0["/basis/nbasis"]) if "/basis/nbasis" in f0 else nbasis
    info_len = int(f0["/basis/info string len"]) if "/basis/info string len" in f0 else 0
    if nbasis_file != nbasis:
        raise ValueError("restart basis has %d spin orbitals, the calculation %d" % (nbasis_file, nbasis))
    st, po, kii = [], [], []
    for f in files:
        dets = f["/qmc/psips/determinants"]
        pops = f["/qmc/psips/populations"]
        if pops.shape[1] < nspaces:
            raise ValueError("restart has %d spaces, the calculation %d" % (pops.shape[1], nspaces))
        scale = int(f["/qmc/psips/population scale factor"][0]) if "/qmc/psips/population scale factor" in f \
            else real_factor
        st.append(_words64(dets, i0, nbasis, info_len))
        po.append(_rescale(pops[:, :nspaces], scale, real_factor))
        kii.append(np.asarray(f["/qmc/psips/data"], dtype=np.float64)[:, 0])
    states = np.concatenate(st) if st else np.zeros((0, (nbasis + 63) // 64), np.int64)
    pops = np.concatenate(po)
    kii = np.concatenate(kii)
    order = _sort_order(states)
    states, pops, kii = states[order], pops[order], kii[order]
    if len(states) > 1:
        same = np.all(states[1:] == states[:-1], axis=1)
        if same.any():
            raise ValueError("a determinant appears twice in the restart files")
    s = "/qmc/state/"
    ref = f0["/qmc/reference/reference determinant"]
    out = {
        "states": states, "pops": pops, "kii": kii,
        "iteration": int(f0[s + "ncycles"]),
        "shift": [float(x) for x in np.ravel(f0[s + "shift"])[:nspaces]],
        "vary_shift": [bool(x) for x in np.ravel(f0[s + "vary shift"])[:nspaces]] if s + "vary shift" in f0
        else [False] * nspaces,
        "nparticles_old": [float(x) for x in np.ravel(f0["/qmc/psips/total population"])[:nspaces]],
        "reference": _words64(np.asarray(ref).reshape(1, -1), i0, nbasis, info_len)[0],
        "restart_version": version,
    }
    if s + "projected energy" in f0:
        out["proj_energy"] = [float(x) for x in np.ravel(f0[s + "projected energy"])[:nspaces]]
    ref_pop = "/qmc/reference/reference population @ t-1"
    if ref_pop in f0:
        out["D0_population"] = [float(x) for x in np.ravel(f0[ref_pop])[:nspaces]]
    return out


def write(path, states, pops, kii, *, nbasis, real_factor, iteration, shift, vary_shift, nparticles_old,
          reference, proj_energy=None, D0_population=None, hash_seed=7, shift_damping=0.05, mtime=None):
    """One restart file (one rank) in restart version 3 with 64-bit words."""
    states = np.ascontiguousarray(states, dtype=np.int64)
    pops = np.ascontiguousarray(pops, dtype=np.int64)
    n, R = pops.shape
    kii = np.asarray(kii, dtype=np.float64).reshape(n)
    data = np.zeros((n, R), np.float64)
    data[:, 0] = kii
    zeros = np.zeros(R, np.float64)
    pe = np.asarray(proj_energy if proj_energy is not None else zeros, np.float64)[:R]
    d0 = np.asarray(D0_population if D0_population is not None else zeros, np.float64)[:R]
    ref = np.asarray(reference, dtype=np.int64).reshape(-1)[:states.shape[1] if n else len(reference)]
    now = time.localtime(time.time() if mtime is None else mtime)
    ds = {
        "/metadata/restart version": np.int32(RESTART_VERSION),
        "/metadata/hande version": b"hande_gb300".ljust(40),
        "/metadata/date": time.strftime("%H:%M:%S %d/%m/%Y", now).encode(),
        "/metadata/uuid": str(uuidlib.uuid4()).encode(),
        "/metadata/calc type": np.int32(FCIQMC_CALC),
        "/metadata/nprocs": np.int32(1),
        "/metadata/i0_length": np.int32(64),
        "/basis/nbasis": np.int32(nbasis),
        "/basis/info string len": np.int32(0),
        "/qmc/psips/determinants": states,
        "/qmc/psips/populations": pops,
        "/qmc/psips/data": data,
        "/qmc/psips/total population": np.asarray(nparticles_old, np.float64)[:R],
        "/qmc/psips/population scale factor": np.array([real_factor], np.int64),
        "/qmc/psips/processor map": np.array([0], np.int32),
        "/qmc/state/ncycles": np.int32(iteration),
        "/qmc/state/shift": np.asarray(shift, np.float64)[:R],
        "/qmc/state/projected energy": pe,
        "/qmc/state/projected energy real": pe,
        "/qmc/state/projected energy imag": zeros,
        "/qmc/state/hash_seed": np.int32(hash_seed),
        "/qmc/state/move_freq": np.int32(0),
        "/qmc/state/vary shift": np.asarray(vary_shift, np.int32)[:R],
        "/qmc/state/shift_damping": np.array([shift_damping], np.float64),
        "/qmc/state/shift_damping_status": np.int32(-2),
        "/qmc/reference/reference determinant": ref,
        "/qmc/reference/Hilbert space reference determinant": ref,
        "/qmc/reference/reference population @ t-1": d0,
        "/qmc/reference/reference population @ t-1 real": d0,
        "/qmc/reference/reference population @ t-1 imag": zeros,
    }
    hdf5lite.write(path, ds, groups=["/rng"], mtime=int(time.time() if mtime is None else mtime))


def _get_state(calc):
    return calc.get_state() if hasattr(calc, "get_state") else calc.state()


def reference_of(paths, system):
    """The reference determinant of a restart as occupied spin orbitals: a
    restarted HANDE calculation takes its reference from the file
    (get_reference_hdf5, src/restart_hdf5.F90:935-1030), and the stored K_ii
    are relative to it."""
    if isinstance(paths, (str, os.PathLike)):
        paths = [paths]
    f0 = hdf5lite.read(paths[0])
    i0 = int(f0["/metadata/i0_length"])
    info_len = int(f0["/basis/info string len"]) if "/basis/info string len" in f0 else 0
    ref = np.asarray(f0["/qmc/reference/reference determinant"]).reshape(1, -1)
    return system.decode(_words64(ref, i0, system.nbasis, info_len)[0])


def load_into(engine, paths):
    """Replace a calculation's walker list and state (the device engine's, or
    the oracle's) by those of HANDE restart files; returns what read()
    returned.  The calculation must have been created with the restart's
    reference determinant (reference_of)."""
    s = engine.system
    rf = (1 << 31) if engine.cfg.real_amplitudes else 1
    r = read(paths, s.nbasis, engine.R, rf)
    ours = [int(engine.cfg.ref_det[w]) & 0xFFFFFFFFFFFFFFFF for w in range(s.nwords)]
    if ours != [int(x) & 0xFFFFFFFFFFFFFFFF for x in r["reference"]]:
        raise ValueError("the calculation's reference determinant differs from the restart's")
    engine.set_walkers(r["states"], r["pops"], r["kii"])
    st = _get_state(engine)
    st.iteration = r["iteration"]
    for q in range(engine.R):
        st.shift[q] = r["shift"][q]
        st.vary_shift[q] = int(r["vary_shift"][q])
        st.nparticles_old[q] = r["nparticles_old"][q]
    engine.set_state(st)
    return r


def save_from(engine, path, report=None, mtime=None):
    """Write an engine's walker list and state as a HANDE restart file;
    `report` (the last report's dict) supplies the projected energy and the
    reference population."""
    s = engine.system
    states, pops, kii = engine.walkers()
    st = _get_state(engine)
    R = engine.R
    W = s.nwords
    write(path, states, pops, kii, nbasis=s.nbasis, real_factor=(1 << 31) if engine.cfg.real_amplitudes else 1,
          iteration=int(st.iteration), shift=[st.shift[q] for q in range(R)],
          vary_shift=[bool(st.vary_shift[q]) for q in range(R)],
          nparticles_old=[st.nparticles_old[q] for q in range(R)],
          reference=[int(engine.cfg.ref_det[w]) for w in range(W)],
          proj_energy=None if report is None else report["\\sum H_0j N_j"],
          D0_population=None if report is None else report["N_0"], hash_seed=int(engine.cfg.seed), mtime=mtime)
