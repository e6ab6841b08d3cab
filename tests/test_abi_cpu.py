"""CPU-side checks of the C-ABI library: it builds, loads, exports every entry
point that include/hande_gpu.h declares, and fails loudly without a GPU."""

import ctypes as C
import os
import re
import subprocess

import pytest

from hande_gb300 import build as hbuild
from hande_gb300 import systems
from hande_gb300._abi import HgpuConfig, HgpuReport, HgpuState, HgpuSystem, PackedSystem, make_config
from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "hande_gpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char \*)\s*(hgpu_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    path = hbuild.build()
    return path


def test_header_matches_binding():
    from hande_gb300.engine import EXPORTS
    assert declared() == sorted(EXPORTS)


def test_library_exports_every_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    syms = set(re.findall(r"\bT (hgpu_\w+)", out))
    missing = set(declared()) - syms
    assert not missing, missing


def test_library_loads_and_reports_version(lib):
    from hande_gb300.engine import load_library
    L = load_library()
    assert L.hgpu_version() >= 100
    assert L.hgpu_error_string(0) == b"ok"


def test_struct_sizes_match_header():
    """ctypes layouts equal the C compiler's layout of the ABI structs."""
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "hande_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(hgpu_system), sizeof(hgpu_config), sizeof(hgpu_report),
         sizeof(hgpu_state), offsetof(hgpu_config, ref_det), offsetof(hgpu_report, device_ms));
  return 0;
}
'''
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    exp = [C.sizeof(HgpuSystem), C.sizeof(HgpuConfig), C.sizeof(HgpuReport), C.sizeof(HgpuState),
           HgpuConfig.ref_det.offset, HgpuReport.device_ms.offset]
    assert got == exp


def test_no_device_fails_loudly(lib):
    """Without a GPU the engine refuses to run (no CPU fallback)."""
    from hande_gb300.engine import Engine, HgpuError, load_library
    L = load_library()
    if L.hgpu_device_count() > 0:
        pytest.skip("a GPU is visible")
    s = systems.hubbard_k([[2, 0], [0, 2]], 2)
    with pytest.raises(HgpuError) as e:
        Engine(s, make_config(s, tau=0.01))
    assert e.value.status == 7


def test_invalid_config_rejected(lib):
    from hande_gb300.engine import load_library
    L = load_library()
    s = systems.hubbard_k([[2, 0], [0, 2]], 2)
    cfg = make_config(s, tau=-1.0)
    ps = PackedSystem(s)
    h = C.c_void_p()
    rc = L.hgpu_create(C.byref(cfg), C.byref(ps.struct), C.byref(h))
    assert rc in (1, 7) and not h.value
