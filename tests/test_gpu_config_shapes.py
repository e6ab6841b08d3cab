"""Whole runs with the parameters of the benchmark configurations, at
populations the oracle finishes in seconds: the GPU engine against the oracle,
walker lists bit-exact after every report, counters and bloom statistics equal.

- the 26-orbital synthetic molecule of the benchmark (10 electrons, C1,
  Hamiltonian seed 2024), tau 1e-3, real amplitudes, spawn cutoff 0.01, uniform
  renorm generator with pattempt_single 0.1 / pattempt_double 0.9; plain and
  initiator (threshold 3).  This Hamiltonian grows about threefold per cycle at
  tau 1e-3, so the reports are one cycle long.
- the headline's synthetic molecule with M = 64 (two-word determinants, 75-bit
  rank keys) and 20 electrons, initiator, two replicas with the quadrature
  initiator test, the replica 2-RDM accumulating; FP64 (the FP32 mode is
  checked against the oracle with tolerances in test_gpu_heat_bath.py).
The 26-orbital runs spawn many events of 3 or more particles, so the bloom
counters (accumulate_bloom_stats) are compared on non-zero values."""

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.test_gpu_parity import assert_close, engine

pytestmark = pytest.mark.gpu

MOL26 = dict(tau=1e-3, real_amplitudes=True, spawn_cutoff=0.01, excit_gen="renorm", pattempt_single=0.1,
             pattempt_double=0.9, init_pop=10, target_population=5000, ncycles=1)


def compare_reports(o, g, nrep, rdm=False):
    blooms = 0
    for r in range(nrep):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0, "list capacity too small for a parity run"
        so, po, ko = o.walkers()
        sg, pg, kg = g.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po, err_msg="report %d pops" % r)
        assert_close(kg, ko)
        assert rg.nattempts == ro.nattempts
        assert rg.nspawned == ro.nspawned
        assert list(rg.nparticles) == list(ro.nparticles)
        assert list(rg.shift) == list(ro.shift)
        assert list(rg.vary_shift) == list(ro.vary_shift)
        assert (rg.nblooms, rg.tot_bloom, rg.max_bloom) == (ro.nblooms, ro.tot_bloom, ro.max_bloom)
        for q in range(2 if rdm else 1):
            assert_close(rg.proj_energy[q], ro.proj_energy[q], 1e-10)
        if rdm and ro.rdm_trace != 0.0:
            assert_close(rg.rdm_energy, ro.rdm_energy, 1e-9)
            assert_close(rg.rdm_trace, ro.rdm_trace, 1e-9)
        blooms += ro.nblooms
    return blooms


@pytest.mark.parametrize("initiator", [False, True])
def test_mol26_benchmark_parameters_bit_exact(initiator):
    s = systems.synthetic_molecule(26, 10, seed=2024)
    cfg = make_config(s, seed=7, initiator=initiator, initiator_threshold=3.0, state_size=400000,
                      spawned_state_size=600000, **MOL26)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    blooms = compare_reports(o, g, 9)
    if not initiator:
        assert blooms > 0, "this case produces blooms (events of 3 or more particles)"
    o.close()


@pytest.mark.parametrize("quadrature", [True, False])
def test_mol64_replica_shape_bit_exact(quadrature):
    s = systems.synthetic_molecule(64, 20, seed=2024)
    cfg = make_config(s, tau=2e-4, init_pop=300, target_population=500, ncycles=2, seed=5, real_amplitudes=True,
                      spawn_cutoff=0.01, excit_gen="renorm", pattempt_single=0.1, pattempt_double=0.9,
                      initiator=True, initiator_threshold=3.0, quadrature_initiator=quadrature, nspaces=2,
                      density_matrices=True, density_matrix_report=0, state_size=300000,
                      spawned_state_size=600000)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    compare_reports(o, g, 4, rdm=True)
    o.close()
