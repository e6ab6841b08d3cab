"""HANDE restart files on the device engine: a calculation restarted from
HANDE's own restart file (the 18-site Hubbard list of tests/golden/
restart_hubbard_k_2d.npz, written as an HDF5 restart) evolves bit-identically
to the oracle restarted from the same file, writes a restart that reads back
as its walker list, and the fciqmc driver reads and writes restart files."""

import os

import numpy as np
import pytest

from hande_gb300 import restart, systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.test_gpu_parity import engine

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _hande_restart(directory, rid=0):
    g = dict(np.load(os.path.join(GOLDEN, "restart_hubbard_k_2d.npz")))
    restart.write(os.path.join(directory, "HANDE.RS.%d.p0.H5" % rid), g["states"], g["pops"], g["kii"], nbasis=36,
                  real_factor=1, iteration=int(g["iteration"][0]), shift=g["shift"], vary_shift=g["vary_shift"],
                  nparticles_old=g["nparticles_old"], reference=g["reference"], mtime=1_700_000_000)
    return g


def _hubbard():
    return systems.hubbard_k([[3, 3], [3, -3]], 18, U=0.5)


def test_restart_from_hande_file_bit_exact(tmp_path):
    _hande_restart(str(tmp_path))
    s = _hubbard()
    cfg = make_config(s, tau=0.01, ncycles=25, seed=7, target_population=5500, state_size=40000,
                      spawned_state_size=40000)
    paths = restart.restart_paths(0, str(tmp_path))
    g = engine(s, cfg)
    o = Oracle(s, cfg)
    rg = restart.load_into(g, paths)
    restart.load_into(o, paths)
    for r in range(3):
        a, b = g.run_report(), o.run_report()
        assert a.error_flags == 0 and b.error_flags == 0
        assert a.iteration == b.iteration == rg["iteration"] + 25 * (r + 1)
        sg, pg, _ = g.walkers()
        so, po, _ = o.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po, err_msg="report %d pops" % r)
        assert a.shift[0] == b.shift[0]
    out = str(tmp_path / "HANDE.RS.1.p0.H5")
    restart.save_from(g, out, report=a.as_dict(1))
    back = restart.read([out], s.nbasis, 1, 1)
    sg, pg, dg = g.walkers()
    np.testing.assert_array_equal(back["states"], sg)
    np.testing.assert_array_equal(back["pops"], pg)
    np.testing.assert_array_equal(back["kii"], dg)
    assert back["iteration"] == a.iteration and back["shift"][0] == a.shift[0]
    g.close()
    o.close()


def test_fciqmc_driver_reads_and_writes_restarts(tmp_path):
    from hande_gb300.calc import fciqmc
    g = _hande_restart(str(tmp_path), rid=2)
    qmc = dict(tau=0.01, rng_seed=7, init_pop=10, mc_cycles=25, nreports=2, target_population=5500,
               state_size=40000, spawned_state_size=40000)
    res = fciqmc(_hubbard(), qmc, restart={"read": 2, "write": 3}, directory=str(tmp_path), verbose=False)
    reps = res["reports"]
    assert reps[-1]["iterations"] == int(g["iteration"][0]) + 50
    back = restart.read(restart.restart_paths(3, str(tmp_path)), 36, 1, 1)
    st, po, _ = res["engine"].walkers()
    np.testing.assert_array_equal(back["states"], st)
    np.testing.assert_array_equal(back["pops"], po)
    res["engine"].close()


def test_engine_continues_hande_restart_like_hande(tmp_path):
    from tests.test_restart_hdf5 import continue_and_compare
    continue_and_compare(engine, tmp_path, 1000)
