"""Regenerate the golden fixtures of this directory from the reference's own
test suite (HANDE test_suite/).  Run in a checkout where the reference tree is
available:

    python tests/golden/make_golden.py /path/to/hande

It copies the small integral files the FCI tests use and extracts, from each
test's benchmark output, the exact-diagonalisation energies ("State  Energy"
table) and the system definition from the Lua input.  The fixtures are
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
