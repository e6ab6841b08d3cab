"""The allocation-free self-annihilation entry point (hgpu_self_annihilate_noalloc).

It exists for callers that cannot let the library allocate device memory: a
host program whose own pool allocator owns all of it, or a caller that must not
allocate on its critical path.  It works in the caller's input/output buffers
and a fixed scratch array inside the library.  Here it is called through the C
ABI on device buffers this test allocates itself, twice in a row, and its output
is compared with the existing entry point hgpu_annihilate_fixed run on an empty
main list (which then holds exactly the self-annihilated spawned list)."""

import ctypes as C

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from tests.helpers import main_and_spawns

pytestmark = pytest.mark.gpu

MAX_ENTRIES = 65536  # HGPU_NOALLOC_MAX_ENTRIES


def cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.skip("CUDA runtime library not found")


class DevBuf:
    def __init__(self, rt, nbytes):
        self.rt = rt
        self.p = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.p), C.c_size_t(max(nbytes, 8))) == 0
        self.nbytes = nbytes

    def upload(self, a):
        a = np.ascontiguousarray(a)
        assert self.rt.cudaMemcpy(self.p, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes), 1) == 0

    def download(self, shape, dtype):
        out = np.zeros(shape, dtype=dtype)
        if out.nbytes:
            assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), self.p, C.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.p)


def reference_result(s, R, sdata):
    """Existing entry point: hgpu_annihilate_fixed into an empty main list."""
    from hande_gb300.engine import Engine
    cfg = make_config(s, tau=0.01, nspaces=R, seed=5, state_size=4 * sdata.shape[0] + 16,
                      spawned_state_size=2 * sdata.shape[0] + 16)
    g = Engine(s, cfg)
    g.set_walkers(np.zeros((0, s.nwords), np.int64), np.zeros((0, R), np.int64))
    g.annihilate_fixed(sdata, 1)
    st, po, _ = g.walkers()
    g.close()
    return st, po


def call_noalloc(L, rt, sdata, W, R):
    n = sdata.shape[0]
    din = DevBuf(rt, sdata.nbytes)
    din.upload(sdata)
    dout = DevBuf(rt, 8 * (W + R) * max(n, 1))
    nout = C.c_int64(-1)
    rc = L.hgpu_self_annihilate_noalloc(din.p, n, W, R, dout.p, C.byref(nout), None)
    assert rc == 0, rc
    res = dout.download((nout.value, W + R), np.int64)
    din.free()
    dout.free()
    return res


@pytest.mark.parametrize("name,R", [("hub_k_4x4", 1), ("mol40_w2", 2)])
def test_noalloc_matches_annihilate_fixed(name, R):
    from hande_gb300.engine import load_library
    L = load_library()
    rt = cudart()
    s = {"hub_k_4x4": systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0),
         "mol40_w2": systems.synthetic_molecule(40, 12, seed=6)}[name]
    W = s.nwords
    rng = np.random.default_rng(17)
    for call in range(2):  # two calls in a row share the library's scratch array
        _, _, sdata = main_and_spawns(s, rng, 1500, 5000 + 2000 * call, R, False, False, hit_frac=0.0)
        got = call_noalloc(L, rt, sdata, W, R)
        st, po = reference_result(s, R, sdata)
        assert got.shape[0] == st.shape[0] > 0
        np.testing.assert_array_equal(got[:, :W], st)
        np.testing.assert_array_equal(got[:, W:], po)


def test_noalloc_rejects_oversized_list():
    from hande_gb300.engine import load_library
    L = load_library()
    nout = C.c_int64(0)
    rc = L.hgpu_self_annihilate_noalloc(C.c_void_p(16), MAX_ENTRIES + 1, 1, 1, C.c_void_p(16), C.byref(nout), None)
    assert rc == 1
    assert nout.value == -MAX_ENTRIES
