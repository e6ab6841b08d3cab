"""Regenerate the golden fixtures of this directory from the reference's own
test suite (HANDE test_suite/).  Run in a checkout where the reference tree is
available:

    python tests/golden/make_golden.py /path/to/hande

It copies the small integral files the FCI tests use and extracts, from each
test's benchmark output, the exact-diagonalisation energies ("State  Energy"
table) and the system definition from the Lua input.  From a second set of
QMC tests it takes the integral file, the reference determinant and the
pattempt_single / pattempt_double that HANDE printed in its input echo
(find_single_double_prob's default when the input sets neither).  The fixtures are
committed so that the tests never need the reference tree at run time."""

from __future__ import annotations

import glob
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, test directory, input file, integral file (or None)
    ("hubbard_k_1d", "fci/hubbard_k_1d", "hubbard.in", None),
    ("hubbard_k_nontilted_2d_fci", "fci/hubbard_k_nontilted_2d_fci", "hubbard.in", None),
    ("hubbard_k_tilted_2d_fci", "fci/hubbard_k_tilted_2d_fci", "hubbard.in", None),
    ("H2O-RHF-sto-2g", "fci/H2O-RHF-sto-2g", "h2o_fci.in", "INTDUMP"),
    ("H2O-RHF-sto-2g-no-sp-eigv", "fci/H2O-RHF-sto-2g-no-sp-eigv", "h2o_fci.in", "INTDUMP"),
    ("h6_sto3g", "fci/h6_sto3g", "fci_hamiltonian_diag.in", "FCIDUMP"),
]

PATTEMPT_CASES = [
    # name, test directory, integral file
    ("N2-RHF-STO-3G", "fciqmc/np4/N2-RHF-STO-3G-harmonic_pop_control_two_stage", "n2_sto3g.fcidump"),
    ("H4-STO-3g", "fciqmc_real_64/np1/H4-STO-3g_cheby", "INTDUMP"),
    ("H2-sto-3g", "fciqmc/np1/H2-sto-3g-replica", "FCIDUMP"),
    ("O2_sto3g_triplet", "fciqmc_real_64/np4/O2_sto3g_triplet_state_histogram", "FCIDUMP"),
    ("He2-aug-cc-pVDZ", "fciqmc_real_64/np4/He2-aug-cc-pVDZ_real_64_SS", "INTDUMP"),
]


def pattempt_entry(out_text: str) -> dict:
    """The first input echo that prints pattempt_single: its excitation
    generator, both probabilities and the reference determinant after it."""
    pos = out_text.index('"pattempt_single"')
    ps = float(re.match(r'"pattempt_single":\s*(-?[\d.]+)', out_text[pos:]).group(1))
    pd = float(re.search(r'"pattempt_double":\s*(-?[\d.]+)', out_text[pos:]).group(1))
    eg = re.findall(r'"excit_gen":\s*"(\w+)"', out_text[:pos])[-1]
    ref = out_text.index('"reference"', pos)
    det = re.search(r'"det":\s*\[([^\]]*)\]', out_text[ref:]).group(1)
    ms = int(re.search(r'"det_ms":\s*(-?\d+)', out_text[ref:]).group(1))
    nel = int(re.search(r'"nel":\s*(\d+)', out_text).group(1))
    return {"excit_gen": eg, "pattempt_single": ps, "pattempt_double": pd,
            "det": [int(x) for x in det.split(",")], "ms": ms, "nel": nel}


def energies(out_text: str, nmax: int = 4):
    m = re.search(r"State\s+Energy\s*\n((?:\s+\d+\s+-?\d+\.\d+\s*\n)+)", out_text)
    vals = []
    for line in m.group(1).strip().splitlines()[:nmax]:
        vals.append(float(line.split()[1]))
    return vals


def lua_table(text: str, key: str):
    m = re.search(key + r"\s*=\s*(\{.*?\}\s*\})", text, re.S)
    if not m:
        m = re.search(key + r"\s*=\s*(\{[^}]*\})", text, re.S)
    return m.group(1) if m else None


def parse_hubbard(text: str) -> dict:
    d = {}
    d["electrons"] = int(re.search(r"electrons\s*=\s*(\d+)", text).group(1))
    lat = re.search(r"lattice\s*=\s*(\{\s*\{.*?\}\s*\})", text, re.S).group(1)
    vecs = re.findall(r"\{([^{}]*)\}", lat)
    d["lattice"] = [[int(x) for x in v.split(",") if x.strip()] for v in vecs]
    for key in ("ms", "sym"):
        m = re.search(r"\b%s\s*=\s*(-?\d+)" % key, text)
        if m:
            d[key] = int(m.group(1))
    m = re.search(r"twist\s*=\s*\{([^}]*)\}", text)
    if m:
        d["twist"] = [float(x) for x in m.group(1).split(",")]
    for key in ("U", "t"):
        m = re.search(r"\b%s\s*=\s*(-?[\d.]+)" % key, text)
        if m:
            d[key] = float(m.group(1))
    return d


def parse_read_in(text: str) -> dict:
    d = {}
    for key in ("nel", "ms", "sym"):
        m = re.search(r"\b%s\s*=\s*(-?\d+)" % key, text)
        if m:
            d[key] = int(m.group(1))
    d["diagonal_only"] = "hamiltonian_diagonal_only = true" in text
    return d


def main(ref_root: str) -> None:
    ts = os.path.join(ref_root, "test_suite")
    fixtures = []
    for name, tdir, inp, ints in CASES:
        path = os.path.join(ts, tdir)
        text = open(os.path.join(path, inp)).read()
        outs = glob.glob(os.path.join(path, "benchmark.out.*"))
        e = energies(open(outs[0]).read())
        entry = {"name": name, "source": "test_suite/%s/%s" % (tdir, os.path.basename(outs[0])),
                 "energies": e}
        if ints is None:
            entry["system"] = "hubbard_k"
            entry["params"] = parse_hubbard(text)
        else:
            entry["system"] = "read_in"
            entry["params"] = parse_read_in(text)
            dst = "%s.fcidump" % name
            shutil.copyfile(os.path.join(path, ints), os.path.join(HERE, dst))
            entry["int_file"] = dst
        fixtures.append(entry)
    with open(os.path.join(HERE, "fci_energies.json"), "w") as fh:
        json.dump(fixtures, fh, indent=1)
    print("wrote %d cases" % len(fixtures))
    cases = []
    for name, tdir, ints in PATTEMPT_CASES:
        path = os.path.join(ts, tdir)
        outs = sorted(glob.glob(os.path.join(path, "benchmark.out.*")))
        entry = {"name": name, "source": "test_suite/%s/%s" % (tdir, os.path.basename(outs[0]))}
        entry.update(pattempt_entry(open(outs[0]).read()))
        dst = "%s.fcidump" % name
        shutil.copyfile(os.path.join(path, ints), os.path.join(HERE, dst))
        entry["int_file"] = dst
        cases.append(entry)
    with open(os.path.join(HERE, "pattempt.json"), "w") as fh:
        json.dump(cases, fh, indent=1)
    print("wrote %d pattempt cases" % len(cases))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
