"""GPU engine (through the C ABI) against the CPU oracle on the same inputs.

Integer data (determinants, populations, excitations, spawned amounts) must be
bit-exact.  Floating-point data (p_gen, H_ij, K_ii, E_proj) is compared with a
relative tolerance of 1e-12; the engine is built with -fmad=false and follows
the reference's operation order, so it is normally exact."""

import os

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN
from tests.helpers import main_and_spawns, random_dets

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def engine(s, cfg):
    from hande_gb300.engine import Engine
    return Engine(s, cfg)


def _systems():
    return {
        "hub_k_4x4": systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0),
        "hub_k_3x3_ms1": systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1),
        "h2o_sto2g": systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump")),
        "mol26": systems.synthetic_molecule(26, 10, seed=5),
        "mol40_w2": systems.synthetic_molecule(40, 12, seed=6),
        # C(48,10)^2 > 2^64: two-word (128-bit) rank keys
        "mol48_w2_r128": systems.synthetic_molecule(48, 20, seed=12),
    }


SYS = _systems()


def assert_close(a, b, rtol=RTOL):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    scale = np.maximum(np.abs(b), 1e-300)
    bad = np.abs(a - b) > rtol * scale + 1e-300
    bad &= ~((a == 0) & (b == 0))
    assert not bad.any(), "max rel err %g at %s" % (np.max(np.abs(a - b) / scale), np.where(bad)[0][:5])


@pytest.mark.parametrize("name", list(SYS))
@pytest.mark.parametrize("gen", ["renorm", "no_renorm"])
def test_eval_excitations(name, gen):
    s = SYS[name]
    rng = np.random.default_rng(11)
    real = s.kind == "read_in"
    cfg = make_config(s, tau=0.01, excit_gen=gen, real_amplitudes=real, seed=1234, state_size=1000,
                      spawned_state_size=1000)
    parents = random_dets(s, 3000, rng, include=[s.aufbau_occ()])
    pp = rng.integers(1, 5, parents.shape[0]) * np.where(rng.random(parents.shape[0]) < 0.5, -1, 1)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    for it in (1, 77):
        ro = o.eval_excitations(parents, pp, it)
        rg = g.eval_excitations(parents, pp, it)
        np.testing.assert_array_equal(rg[0], ro[0])  # orbitals
        np.testing.assert_array_equal(rg[3], ro[3])  # allowed
        assert_close(rg[1], ro[1])                   # p_gen
        assert_close(rg[2], ro[2])                   # H_ij
        np.testing.assert_array_equal(rg[4], ro[4])  # spawned population


@pytest.mark.parametrize("name", list(SYS))
def test_eval_diagonal(name):
    s = SYS[name]
    rng = np.random.default_rng(3)
    cfg = make_config(s, tau=0.01, state_size=100, spawned_state_size=100)
    dets = random_dets(s, 500, rng, include=[s.aufbau_occ()])
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    h00 = o.sc0(s.encode(s.aufbau_occ()).view(np.int64))
    ref = np.array([o.sc0(d) - h00 for d in dets])
    assert_close(g.eval_diagonal(dets), ref)


CASES = [(n, R, real, ini) for n in ("hub_k_4x4", "mol26", "mol40_w2") for R in (1, 2) for real in (False, True)
         for ini in (False, True)]


@pytest.mark.parametrize("name,R,real,ini", CASES)
def test_annihilate_fixed(name, R, real, ini):
    """direct_annihilation of a fixed spawned list: bit-exact main list."""
    s = SYS[name]
    rng = np.random.default_rng(hash((name, R, real, ini)) & 0xFFFF)
    cfg = make_config(s, tau=0.01, real_amplitudes=real, initiator=ini, nspaces=R, seed=99,
                      state_size=20000, spawned_state_size=20000)
    main, pops, sdata = main_and_spawns(s, rng, 2000, 4000, R, real, ini)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.set_walkers(main, pops)
    g.set_walkers(main, pops)
    for it in (5, 6):
        assert o.annihilate_fixed(sdata, it) == 0
        g.annihilate_fixed(sdata, it)
        so, po, ko = o.walkers()
        sg, pg, kg = g.walkers()
        np.testing.assert_array_equal(sg, so)
        np.testing.assert_array_equal(pg, po)
        assert_close(kg, ko)


def test_annihilate_empty_and_no_spawns():
    s = SYS["hub_k_4x4"]
    cfg = make_config(s, tau=0.01, state_size=1000, spawned_state_size=1000)
    g = engine(s, cfg)
    o = Oracle(s, cfg)
    g.set_walkers(np.zeros((0, 1), np.int64), np.zeros((0, 1), np.int64))
    empty = np.zeros((0, 3), np.int64)
    g.annihilate_fixed(empty, 1)
    assert g.walkers()[0].shape[0] == 0
    rng = np.random.default_rng(0)
    main, pops, _ = main_and_spawns(s, rng, 300, 10, 1, False, False)
    pops[::7] = 0  # emptied by death: removed
    g.set_walkers(main, pops)
    o.set_walkers(main, pops)
    g.annihilate_fixed(empty, 2)
    o.annihilate_fixed(empty, 2)
    np.testing.assert_array_equal(g.walkers()[0], o.walkers()[0])
    np.testing.assert_array_equal(g.walkers()[1], o.walkers()[1])


RUNS = [
    ("hub_k_4x4", dict(tau=0.005, init_pop=10, target_population=1000, excit_gen="renorm"), 6),
    ("hub_k_4x4", dict(tau=0.005, init_pop=10, target_population=1000, excit_gen="no_renorm"), 5),
    # harmonic population control (critical damping: zeta = shift_damping^2 / 4)
    ("hub_k_4x4", dict(tau=0.005, init_pop=10, target_population=60, shift_damping=0.04,
                       shift_harmonic_forcing=0.0004), 8),
    # the shift starts to vary on the reference population (reference_target)
    ("hub_k_4x4", dict(tau=0.005, init_pop=10, target_population=11, target_reference=True), 6),
    ("hub_k_3x3_ms1", dict(tau=0.02, init_pop=100, target_population=500, initiator=True), 8),
    ("h2o_sto2g", dict(tau=0.01, init_pop=100, target_population=200, real_amplitudes=True, initial_shift=3.0), 10),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                   pattempt_single=0.1, pattempt_double=0.9), 3),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True, initiator=True), 5),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      excit_gen="no_renorm"), 2),
    ("mol48_w2_r128", dict(tau=5e-5, init_pop=2000, target_population=20000, real_amplitudes=True,
                           initiator=True, nspaces=2), 2),
]


@pytest.mark.parametrize("name,opts,nrep", RUNS, ids=["%s-%d" % (r[0], i) for i, r in enumerate(RUNS)])
def test_whole_run_bit_exact(name, opts, nrep):
    """Whole FCIQMC runs: same counter-based streams, so the walker lists must
    agree exactly after every report; estimators agree to rounding."""
    s = SYS[name]
    cfg = make_config(s, ncycles=10, seed=7, state_size=1500000, spawned_state_size=1500000, **opts)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    for r in range(nrep):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0, "list capacity too small for a parity run"
        so, po, ko = o.walkers()
        sg, pg, kg = g.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po, err_msg="report %d pops" % r)
        assert_close(kg, ko)
        assert rg.nstates == ro.nstates
        assert rg.nattempts == ro.nattempts
        assert rg.nspawned == ro.nspawned
        assert rg.nspawn_events == ro.nspawn_events
        assert list(rg.nparticles) == list(ro.nparticles)
        assert list(rg.shift) == list(ro.shift)
        assert list(rg.vary_shift) == list(ro.vary_shift)
        assert_close(rg.proj_energy[0], ro.proj_energy[0], 1e-10)
        assert_close(rg.D0_population[0], ro.D0_population[0], 1e-12)
        assert_close(rg.rspawn, ro.rspawn, 1e-12)


def test_singles_queue_overflow_bit_exact():
    """The spawning kernel queues singles for the singles kernel in a queue of
    a quarter of the spawned list's capacity (at least 65536 entries) and runs
    the ones past it itself: with p_single = 0.8 and 2e5 attempts per cycle
    about 1.6e5 singles meet a queue of 125000, so every cycle takes both
    paths.  The walker lists stay those of the oracle."""
    s = SYS["mol26"]
    cfg = make_config(s, tau=5e-5, init_pop=2e5, target_population=1e12, real_amplitudes=True,
                      pattempt_single=0.8, pattempt_double=0.2, ncycles=2, seed=11, state_size=1500000,
                      spawned_state_size=500000)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    for r in range(2):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0
        assert rg.nattempts > 2 * 150000  # two cycles of > 1.5e5 attempts: > 1.2e5 singles each
        np.testing.assert_array_equal(g.walkers()[0], o.walkers()[0], err_msg="report %d states" % r)
        np.testing.assert_array_equal(g.walkers()[1], o.walkers()[1], err_msg="report %d pops" % r)
        assert rg.nspawned == ro.nspawned
        assert rg.nattempts == ro.nattempts


def test_checkpoint_restore_bit_exact(tmp_path):
    s = SYS["hub_k_4x4"]
    cfg = make_config(s, tau=0.005, init_pop=10, target_population=2000, ncycles=10, seed=3, state_size=100000,
                      spawned_state_size=100000)
    a = engine(s, cfg)
    a.initial_distribution()
    for _ in range(5):
        a.run_report()
    path = str(tmp_path / "ck.bin")
    a.checkpoint(path)
    for _ in range(4):
        a.run_report()
    sa, pa, _ = a.walkers()
    b = engine(s, cfg)
    assert b.restore(path) == 0
    for _ in range(4):
        b.run_report()
    sb, pb, _ = b.walkers()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(pa, pb)
    # a truncated file is rejected
    data = open(path, "rb").read()
    open(path, "wb").write(data[:-5])
    c = engine(s, cfg)
    assert c.restore(path) != 0


def test_spawn_overflow_flag():
    """A tiny spawned list fills: the report carries the overflow flag (spawn%error)."""
    s = SYS["hub_k_4x4"]
    cfg = make_config(s, tau=0.005, init_pop=500, ncycles=10, seed=3, state_size=100000, spawned_state_size=5)
    g = engine(s, cfg)
    g.initial_distribution()
    rep = g.run_report()
    assert rep.error_flags & 1
