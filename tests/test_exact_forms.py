"""The integer forms of FP64 expressions used by the spawning kernels
(hande_gb300/csrc/hgpu_exact.h) against the FP64 expressions themselves, on the
host: random and boundary inputs, compiled with the same header the device
code includes."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact_forms_match_fp64(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "exact_forms_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-o", exe,
                    os.path.join(HERE, "exact_forms_check.cpp")], check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
