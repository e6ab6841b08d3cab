"""Replica 2-RDM (density_matrices, src/replica_rdm.F90) on the GPU against
the oracle.  The walker lists stay bit-exact (the RDM draw comes after the
spawn's own draws in each attempt's stream); the RDM itself is summed with
FP64 atomics in an order of its own, so it is compared to rounding: every
element within 1e-12 of the largest plus 1e-10 relative, the RDM energy and
trace within 1e-9 relative."""

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.test_gpu_parity import SYS, engine

pytestmark = pytest.mark.gpu


def _mol12():
    return systems.synthetic_molecule(12, 6, seed=9)


CASES = [
    ("h2o_sto2g", lambda: SYS["h2o_sto2g"], dict(tau=0.01, init_pop=200, target_population=3000, initial_shift=1.0,
                                                   density_matrix_report=2), 30),
    ("mol12", _mol12, dict(tau=5e-4, init_pop=1000, target_population=1500, density_matrix_report=1,
                           excit_gen="no_renorm"), 4),
    ("mol40_w2", lambda: SYS["mol40_w2"], dict(tau=5e-5, init_pop=2000, target_population=2500,
                                                 density_matrix_report=0), 3),
]


def _close(g, o, what):
    g = np.asarray(g, float)
    o = np.asarray(o, float)
    scale = max(np.abs(o).max(), 1e-300)
    bad = np.abs(g - o) > 1e-12 * scale + 1e-10 * np.abs(o)
    assert not bad.any(), "%s: max abs err %g (scale %g)" % (what, np.abs(g - o).max(), scale)


@pytest.mark.parametrize("name,make,opts,nrep", CASES, ids=[c[0] for c in CASES])
def test_rdm_run_matches_oracle(name, make, opts, nrep):
    s = make()
    cfg = make_config(s, ncycles=10, seed=23, real_amplitudes=True, nspaces=2, density_matrices=True,
                      state_size=400000, spawned_state_size=400000, **opts)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    accumulated = 0
    for r in range(nrep):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0
        so, po, _ = o.walkers()
        sg, pg, _ = g.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po, err_msg="report %d pops" % r)
        assert (ro.rdm_trace != 0.0) == (rg.rdm_trace != 0.0)
        if ro.rdm_trace != 0.0:
            accumulated += 1
            _close(g.rdm(), o.rdm(), "report %d rdm" % r)
            assert abs(rg.rdm_trace - ro.rdm_trace) <= 1e-9 * abs(ro.rdm_trace)
            assert abs(rg.rdm_energy - ro.rdm_energy) <= 1e-9 * abs(ro.rdm_energy) + 1e-12 * abs(ro.rdm_trace)
    assert accumulated >= 1


def test_rdm_requires_replicas():
    from hande_gb300.engine import HgpuError
    s = SYS["mol26"]
    with pytest.raises(HgpuError):
        engine(s, make_config(s, tau=0.01, nspaces=1, density_matrices=True, state_size=100,
                              spawned_state_size=100))
    h = SYS["hub_k_4x4"]
    with pytest.raises(HgpuError):
        engine(h, make_config(h, tau=0.01, nspaces=2, density_matrices=True, state_size=100,
                              spawned_state_size=100))
