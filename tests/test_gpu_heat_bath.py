"""Heat-bath excitation generators on the GPU (src/excit_gen_heat_bath_mol.F90)
against the CPU oracle, through the C ABI.

FP64 mode: excitations, p_gen, H_ij and whole runs are bit-exact (the host
table builder and the device generator follow the reference's operation
order).  Mixed precision (FP32 tables, integrals and p_gen) is compared with
the FP64 oracle by its relative error, with the bound written in the test."""

import os

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import PREC_MIXED, make_config
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN
from tests.helpers import random_dets
from tests.test_gpu_parity import assert_close, engine

pytestmark = pytest.mark.gpu

HB_SYS = {
    "h2o_sto2g": lambda: systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump")),
    "mol12": lambda: systems.synthetic_molecule(12, 6, seed=4),
    "mol34_w2": lambda: systems.synthetic_molecule(34, 8, seed=4),
}
_cache = {}


def hb_sys(name):
    if name not in _cache:
        _cache[name] = HB_SYS[name]()
    return _cache[name]


@pytest.mark.parametrize("name", list(HB_SYS))
@pytest.mark.parametrize("gen", ["heat_bath", "heat_bath_uniform", "heat_bath_single"])
def test_eval_heat_bath(name, gen):
    s = hb_sys(name)
    rng = np.random.default_rng(21)
    cfg = make_config(s, tau=0.01, excit_gen=gen, real_amplitudes=True, seed=4321, state_size=1000,
                      spawned_state_size=1000)
    parents = random_dets(s, 3000, rng, include=[s.aufbau_occ()])
    pp = rng.integers(1, 5, parents.shape[0]) * np.where(rng.random(parents.shape[0]) < 0.5, -1, 1)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    for it in (1, 52):
        ro = o.eval_excitations(parents, pp, it)
        rg = g.eval_excitations(parents, pp, it)
        np.testing.assert_array_equal(rg[0], ro[0])  # orbitals
        np.testing.assert_array_equal(rg[3], ro[3])  # allowed
        assert_close(rg[1], ro[1])                   # p_gen
        assert_close(rg[2], ro[2])                   # H_ij
        np.testing.assert_array_equal(rg[4], ro[4])  # spawned population
        assert ro[3].mean() > 0.1


HB_RUNS = [
    ("mol12", dict(tau=2e-3, init_pop=500, target_population=5000, real_amplitudes=True, excit_gen="heat_bath"), 5),
    ("mol12", dict(tau=2e-3, init_pop=500, target_population=5000, real_amplitudes=True,
                   excit_gen="heat_bath_uniform", pattempt_single=0.2, pattempt_double=0.8), 6),
    ("mol12", dict(tau=2e-3, init_pop=500, target_population=5000, real_amplitudes=True, excit_gen="heat_bath",
                   initiator=True), 6),
    ("mol12", dict(tau=2e-3, init_pop=500, target_population=5000, real_amplitudes=True,
                   excit_gen="heat_bath_single", pattempt_single=0.2, pattempt_double=0.8), 5),
    ("h2o_sto2g", dict(tau=0.01, init_pop=100, target_population=300, excit_gen="heat_bath", initial_shift=3.0), 8),
    ("mol34_w2", dict(tau=5e-4, init_pop=1000, target_population=20000, real_amplitudes=True,
                      excit_gen="heat_bath", initiator=True), 3),
]


@pytest.mark.parametrize("name,opts,nrep", HB_RUNS, ids=["%s-%d" % (r[0], i) for i, r in enumerate(HB_RUNS)])
def test_whole_run_heat_bath(name, opts, nrep):
    s = hb_sys(name)
    cfg = make_config(s, ncycles=10, seed=17, state_size=1000000, spawned_state_size=1000000, **opts)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    for r in range(nrep):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0
        so, po, ko = o.walkers()
        sg, pg, kg = g.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po, err_msg="report %d pops" % r)
        assert_close(kg, ko)
        assert rg.nattempts == ro.nattempts
        assert rg.nspawn_events == ro.nspawn_events
        assert list(rg.shift) == list(ro.shift)
        assert_close(rg.proj_energy[0], ro.proj_energy[0], 1e-10)
    assert rg.nstates > 10


# FP32 tables and integrals: p_gen is a product of a few ratios (a few float
# ulps); a single's H_ij is a sum of 2 nel integrals that can cancel, so its
# bound is relative plus an absolute floor.
MIXED_RTOL_PGEN = 2e-5
MIXED_RTOL_H, MIXED_ATOL_H = 1e-4, 1e-6


@pytest.mark.parametrize("gen", ["heat_bath", "heat_bath_uniform", "heat_bath_single"])
def test_mixed_precision_heat_bath(gen):
    """FP32 heat-bath path against the FP64 oracle: where the same excitation is
    drawn (a draw can fall on the other side of an alias threshold that moved by
    an FP32 rounding), H_ij and p_gen agree to the bounds above."""
    s = hb_sys("mol12")
    rng = np.random.default_rng(8)
    parents = random_dets(s, 20000, rng, include=[s.aufbau_occ()])
    pp = np.ones(parents.shape[0], np.int64)
    c64 = make_config(s, tau=0.01, excit_gen=gen, real_amplitudes=True, seed=99, state_size=1000,
                      spawned_state_size=1000)
    c32 = make_config(s, tau=0.01, excit_gen=gen, real_amplitudes=True, seed=99, state_size=1000,
                      spawned_state_size=1000, precision=PREC_MIXED)
    ro = Oracle(s, c64).eval_excitations(parents, pp, 5)
    rg = engine(s, c32).eval_excitations(parents, pp, 5)
    same = np.all(rg[0] == ro[0], axis=1) & (rg[3] == ro[3])
    assert same.mean() > 0.999
    ok = same & (ro[3] == 1)
    err_h = np.abs(rg[2][ok] - ro[2][ok])
    rel_p = np.abs(rg[1][ok] - ro[1][ok]) / np.abs(ro[1][ok])
    assert np.all(err_h <= MIXED_RTOL_H * np.abs(ro[2][ok]) + MIXED_ATOL_H), err_h.max()
    assert rel_p.max() < MIXED_RTOL_PGEN, rel_p.max()


def test_heat_bath_bias_refused():
    """The original heat bath refuses a system where a valid single has no j
    (src/excit_gen_heat_bath_mol.F90:185-197): status HGPU_ERR_INVALID."""
    from hande_gb300.engine import HgpuError
    M = 5
    h = np.diag(-1.0 + 0.2 * np.arange(M)) + 0.01 * (np.ones((M, M)) - np.eye(M))
    v = np.zeros(systems.tri0(systems.tri0(M - 1, M - 1), systems.tri0(M - 1, M - 1)) + 1)
    for p in range(M):
        for q in range(M):
            v[systems.v2_index(p, p, q, q)] = 0.5 / (1 + abs(p - q))
    s = systems.molecular_from_arrays(h, v, 4)
    cfg = make_config(s, tau=0.01, excit_gen="heat_bath", seed=1, state_size=100, spawned_state_size=100)
    with pytest.raises(HgpuError):
        engine(s, cfg)
    cfg = make_config(s, tau=0.01, excit_gen="heat_bath_uniform", seed=1, state_size=100, spawned_state_size=100)
    engine(s, cfg).close()
