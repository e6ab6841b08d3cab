"""uniform_power_pitzer, uniform_cauchy_schwarz, heat_bath_power_pitzer,
heat_bath_cauchy_schwarz (gen_excit_mol_power_pitzer_occ,
src/excit_gen_power_pitzer_mol.F90:1260-1547) and heat_bath_power_pitzer_ref
(gen_excit_mol_power_pitzer_orderN, :941-1258) on the GPU
against the oracle: excitations, allowed flags and spawned amounts bit-exact,
p_gen and H_ij to 1e-12 relative, whole runs bit-exact after every report."""

import numpy as np
import pytest

from hande_gb300._abi import PREC_MIXED, make_config
from oracle.pyoracle import Oracle
from tests.helpers import random_dets
from tests.test_gpu_parity import SYS, assert_close, engine

pytestmark = pytest.mark.gpu

GENS = ["uniform_power_pitzer", "uniform_cauchy_schwarz", "heat_bath_power_pitzer", "heat_bath_cauchy_schwarz",
        "heat_bath_power_pitzer_ref"]


@pytest.mark.parametrize("name", ["h2o_sto2g", "mol26", "mol40_w2"])
@pytest.mark.parametrize("gen", GENS)
def test_eval_excitations_pp(name, gen):
    s = SYS[name]
    rng = np.random.default_rng(33)
    cfg = make_config(s, tau=0.01, excit_gen=gen, real_amplitudes=True, seed=2468, state_size=1000,
                      spawned_state_size=1000)
    parents = random_dets(s, 3000, rng, include=[s.aufbau_occ()])
    pops = rng.integers(1, 5, parents.shape[0]) * np.where(rng.random(parents.shape[0]) < 0.5, -1, 1)
    pops = pops * (1 << 31)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    for it in (1, 4):
        ro = o.eval_excitations(parents, pops, it)
        rg = g.eval_excitations(parents, pops, it)
        np.testing.assert_array_equal(rg[0], ro[0])  # orbitals
        np.testing.assert_array_equal(rg[3], ro[3])  # allowed
        assert_close(rg[1], ro[1])                   # p_gen
        assert_close(rg[2], ro[2])                   # H_ij
        np.testing.assert_array_equal(rg[4], ro[4])  # spawned population
    al = ro[3].astype(bool) & (ro[0][:, 1] >= 0)
    ms = s.orb_ms
    par = ms[ro[0][al, 0]] == ms[ro[0][al, 1]]
    assert par.any() and (~par).any()


RUNS = [
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                   excit_gen="uniform_power_pitzer"), 3),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      excit_gen="uniform_cauchy_schwarz", initiator=True), 2),
    ("h2o_sto2g", dict(tau=0.01, init_pop=100, target_population=200, real_amplitudes=True, initial_shift=3.0,
                       excit_gen="uniform_power_pitzer"), 6),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                   excit_gen="heat_bath_power_pitzer", initiator=True), 3),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      excit_gen="heat_bath_cauchy_schwarz"), 2),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                   excit_gen="heat_bath_power_pitzer_ref"), 3),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      excit_gen="heat_bath_power_pitzer_ref", power_pitzer_min_weight=0.0, initiator=True), 2),
    ("h2o_sto2g", dict(tau=0.01, init_pop=100, target_population=200, real_amplitudes=True, initial_shift=3.0,
                       excit_gen="heat_bath_power_pitzer_ref"), 6),
]


@pytest.mark.parametrize("name,opts,nrep", RUNS, ids=["%s-%d" % (r[0], i) for i, r in enumerate(RUNS)])
def test_whole_run_pp_bit_exact(name, opts, nrep):
    s = SYS[name]
    cfg = make_config(s, ncycles=10, seed=19, state_size=1500000, spawned_state_size=1500000, **opts)
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
        assert list(rg.shift) == list(ro.shift)
        assert_close(rg.proj_energy[0], ro.proj_energy[0], 1e-10)
    assert so.shape[0] > 10


def test_pp_fp64_only_and_min_weight_range():
    from hande_gb300.engine import HgpuError
    s = SYS["mol26"]
    for gen in ("uniform_power_pitzer", "heat_bath_power_pitzer_ref"):
        with pytest.raises(HgpuError):
            engine(s, make_config(s, tau=0.01, excit_gen=gen, precision=PREC_MIXED, state_size=100,
                                  spawned_state_size=100))
    # src/check_input.F90:182-184
    with pytest.raises(HgpuError):
        engine(s, make_config(s, tau=0.01, excit_gen="heat_bath_power_pitzer_ref", power_pitzer_min_weight=1.5,
                              state_size=100, spawned_state_size=100))
