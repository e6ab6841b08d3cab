"""Regenerate reference_fciqmc_runs.json from the FCIQMC outputs of the
reference's own test suite (HANDE test_suite/, benchmark.out.* files):

    python tests/golden/make_reference_runs.py /path/to/hande

For each case it reads the report table that HANDE printed (columns
iterations, Shift, \\sum H_0j N_j, N_0, # H psips of the first space), finds the
report at which the shift starts to vary, and reblocks the reports after an
equilibration window with hande_gb300.analysis (the same code that reblocks the
GPU engine's runs in tests/test_gpu_reference_runs.py).  It stores, per case,
the calculation's inputs (from the JSON echo of the input in the output), the
reference determinant HANDE used, and the reblocked shift and projected energy
with their standard errors.  Only these summaries are committed; the tests
never read the reference tree."""

from __future__ import annotations

import glob
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from hande_gb300 import analysis  # noqa: E402

# name, test directory, input file, system kind, system parameters as the Lua input gives them
CASES = [
    ("hubbard_k_1d_14s_14e_renorm", "fciqmc/np1/hubbard_k_1d_no_renorm", "renorm.in", "hubbard_k",
     {"lattice": [[14]], "electrons": 14, "ms": 0, "U": 1.0}),
    ("hubbard_k_1d_14s_14e_no_renorm", "fciqmc/np1/hubbard_k_1d_no_renorm", "no_renorm.in", "hubbard_k",
     {"lattice": [[14]], "electrons": 14, "ms": 0, "U": 1.0}),
    ("hubbard_k_14s_10e_U2_initiator", "ifciqmc/np2/hubbard_k_14s_14e_U2", "hubbard.in", "hubbard_k",
     {"lattice": [[14]], "electrons": 10, "ms": 0, "U": 2.0}),
    ("hubbard_k_2x2_2e", "fciqmc/np1/hubbard_k_nontilted_2d_fciqmc", "hubbard.in", "hubbard_k",
     {"lattice": [[2, 0], [0, 2]], "electrons": 2, "ms": 0, "U": 1.0}),
    ("H2-sto-3g-replica", "fciqmc/np1/H2-sto-3g-replica", "h2.in", "read_in",
     {"int_file": "H2-sto-3g.fcidump", "nel": 2, "ms": 0}),
]

QMC_KEYS = ["tau", "rng_seed", "D0_population", "ncycles", "nreport", "target_particles", "initial_shift",
            "shift_damping", "initiator_approx", "initiator_pop", "excit_gen", "real_amplitudes",
            "vary_shift_from", "vary_shift_from_proje", "spawn_cutoff", "shift_harmonic_forcing",
            "shift_harmonic_forcing_two_stage"]


def json_echo(text: str) -> dict:
    """The JSON block in which HANDE echoes its input ("-- Start JSON block --")."""
    m = re.search(r"-- Start JSON block --\s*\n(.*?)\n\s*-- End JSON block --", text, re.S)
    body = m.group(1)
    body = re.sub(r",\s*([}\]])", r"\1", body)  # HANDE leaves a comma before some closing brackets
    return json.loads(body)


def report_table(text: str):
    """Rows of the first report table after the input echo: iterations and the
    first space's Shift, sum H_0j N_j, N_0, # H psips."""
    lines = text.splitlines()
    start = None
    for k, ln in enumerate(lines):
        if ln.lstrip().startswith("#") and "iterations" in ln and "Shift" in ln:
            start = k
            break
    rows = []
    for ln in lines[start + 1:]:
        f = ln.split()
        if not f:
            break
        if f[0] == "#":
            f = f[1:]
        try:
            vals = [float(x) for x in f[:5]]
        except ValueError:
            break
        rows.append(vals)
    return np.array(rows)


def window(shift: np.ndarray, initial_shift: float):
    """First report used for the statistics: the first report at which the
    shift has moved off its initial value, plus 10 reports of equilibration."""
    moved = np.nonzero(shift != initial_shift)[0]
    first = int(moved[0]) if moved.size else len(shift)
    return first + 10


def summarise(table: np.ndarray, initial_shift: float) -> dict:
    it, shift, num, d0, nw = table.T
    k0 = window(shift, initial_shift)
    S, Serr, Sopt = analysis.mean_error(shift[k0:])
    E, Eerr, Eopt = analysis.projected_energy(num[k0:], d0[k0:])
    return {"first_report": int(k0), "reports": int(len(shift) - k0), "shift": S, "shift_error": Serr,
            "shift_opt_block": Sopt, "proj_energy": E, "proj_energy_error": Eerr, "proj_energy_opt_block": Eopt,
            "mean_walkers": float(nw[k0:].mean())}


def main(ref_root: str) -> None:
    ts = os.path.join(ref_root, "test_suite")
    out = []
    for name, tdir, inp, kind, sysp in CASES:
        path = os.path.join(ts, tdir)
        bench = glob.glob(os.path.join(path, "benchmark.out.*inp=%s" % inp))[0]
        text = open(bench).read()
        js = json_echo(text)
        q = js["qmc"]
        fo = js.get("fciqmc", {})
        qmc = {k: q[k] for k in QMC_KEYS if k in q}
        entry = {"name": name, "source": "test_suite/%s/%s" % (tdir, os.path.basename(bench)), "system": kind,
                 "system_params": sysp, "qmc": qmc,
                 "replica_tricks": bool(fo.get("replica_tricks", False)),
                 "density_matrices": bool(fo.get("density_matrices", False)),
                 "quadrature_initiator": bool(fo.get("quadrature_initiator", True)),
                 "reference_det": js["reference"]["det"]}
        table = report_table(text[text.index("-- End JSON block --"):])
        entry["nreports_in_output"] = int(table.shape[0] - 1)
        entry["reference_stats"] = summarise(table[1:], float(q.get("initial_shift", 0.0)))
        out.append(entry)
        print(name, entry["reference_stats"])
    with open(os.path.join(HERE, "reference_fciqmc_runs.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote %d cases" % len(out))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
