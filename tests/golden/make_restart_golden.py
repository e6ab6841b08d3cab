"""Regenerate the restart-file fixtures of this directory from HANDE restart
files in the reference's test suite:

    python tests/golden/make_restart_golden.py /path/to/hande

The files are read with hande_gb300.hdf5lite (no HDF5 library is needed) and
reduced to what the tests check:
- restart_hubbard_k_2d.npz: the walker list of test_suite/fciqmc/np2/
  hubbard_k_2d_restart (18-site Hubbard model in a Bloch basis, 32-bit
  determinant words, int64 populations) -- the raw 32-bit words, the list in
  64-bit words sorted in HANDE's order, the populations, K_ii (data(1,:)) and
  the scalars of qmc/state and qmc/psips;
- restart_he2.npz: the same for test_suite/fciqmc_real_64/np1/
  He2-aug-cc-pVDZ_real_64_restart (He2 aug-cc-pVDZ, whose integral file is
  He2-aug-cc-pVDZ.fcidump here; int32 integer populations, scale factor 1);
- restart_structure.json: the header-message signature (type, flags,
  version) of every object of a restart-version-2 FCIQMC file and of a
  restart-version-3 file, which the writer's files are compared against;
- restart_continuation.json: HANDE's own continuation of the Hubbard restart
  (the report table of the test's benchmark output), reblocked after a
  10-report window with hande_gb300.analysis, with the run's parameters.
The tests never need the reference tree."""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from hande_gb300 import hdf5lite, restart  # noqa: E402
from tests.golden.make_reference_runs import json_echo, report_table, summarise  # noqa: E402

CASES = [
    # fixture, test directory, restart id, nbasis, nspaces, real factor of the calculation reading it
    ("restart_hubbard_k_2d", "fciqmc/np2/hubbard_k_2d_restart", 0, 36, 1, 1),
    ("restart_he2", "fciqmc_real_64/np1/He2-aug-cc-pVDZ_real_64_restart", 0, 20, 1, 1 << 31),
]

STRUCTURES = [
    ("version2_fciqmc", "fciqmc/np2/hubbard_k_2d_restart/HANDE.RS.0.p0.H5"),
    ("version3", "ccmc_real_64/np1/H4-STO-3g_ccsd_multiref/HANDE.RS.3.p0.H5"),
]


def main(ref_root: str):
    suite = os.path.join(ref_root, "test_suite")
    for name, d, rid, nbasis, R, rf in CASES:
        paths = restart.restart_paths(rid, os.path.join(suite, d))
        raw = hdf5lite.read(paths[0])
        r = restart.read(paths, nbasis, R, rf)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            raw_determinants=raw["/qmc/psips/determinants"], raw_populations=raw["/qmc/psips/populations"],
            raw_scale=np.array([int(raw["/qmc/psips/population scale factor"][0])]),
            states=r["states"], pops=r["pops"], kii=r["kii"], reference=r["reference"],
            iteration=np.array([r["iteration"]]), shift=np.array(r["shift"]),
            vary_shift=np.array(r["vary_shift"]), nparticles_old=np.array(r["nparticles_old"]),
            real_factor=np.array([rf]))
    out = {}
    for name, rel in STRUCTURES:
        out[name] = {k: [list(m) for m in v] for k, v in hdf5lite.structure(os.path.join(suite, rel)).items()}
    with open(os.path.join(HERE, "restart_structure.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    import glob
    d = os.path.join(suite, "fciqmc/np2/hubbard_k_2d_restart")
    bench = glob.glob(os.path.join(d, "benchmark.out.*inp=hubbard.in"))[0]
    text = open(bench).read()
    q = json_echo(text)["qmc"]
    table = report_table(text[text.index("-- End JSON block --"):])
    cont = {"source": "test_suite/fciqmc/np2/hubbard_k_2d_restart/%s" % os.path.basename(bench),
            "qmc": {k: q[k] for k in ("tau", "rng_seed", "ncycles", "nreport", "target_particles", "shift_damping")
                    if k in q},
            "first_iteration": int(table[0, 0]), "reports_in_output": int(table.shape[0] - 1),
            "reference_stats": summarise(table[1:], 0.0)}
    with open(os.path.join(HERE, "restart_continuation.json"), "w") as f:
        json.dump(cont, f, indent=1)
    print(cont)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
