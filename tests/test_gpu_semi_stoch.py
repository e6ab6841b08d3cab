"""Semi-stochastic projection (src/semi_stoch.F90, 'high' and 'ci' spaces,
separate and combined annihilation) on the GPU against the oracle: the walker
lists, deterministic states included, bit-exact after every report, through the
building of the space (at a given iteration or after the shift starts varying),
the exact projection and its stochastic rounding; integer and real walkers,
Hubbard and molecular systems, one- and two-word determinants, initiator on and
off."""

import numpy as np
import pytest

from hande_gb300._abi import make_config
from oracle import fci
from oracle.pyoracle import Oracle
from tests.helpers import sort_dets
from tests.test_gpu_parity import SYS, assert_close, engine

pytestmark = pytest.mark.gpu

RUNS = [
    ("h2o_sto2g", dict(tau=0.01, init_pop=20, target_population=40, real_amplitudes=True, initial_shift=1.0,
                       semi_stoch_space=1, semi_stoch_size=12, semi_stoch_start_iter=2 ** 62,
                       semi_stoch_shift_iter=30), 14),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True, initiator=True,
                   semi_stoch_space=1, semi_stoch_size=300, semi_stoch_start_iter=15), 3),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      semi_stoch_space=1, semi_stoch_size=150, semi_stoch_start_iter=6), 3),
    ("hub_k_4x4", dict(tau=0.01, init_pop=50, target_population=5000, semi_stoch_space=1, semi_stoch_size=40,
                       semi_stoch_start_iter=8), 4),
    # 'ci' spaces: CISD of H2O/STO-2G, CIS of the M=26 molecule
    ("h2o_sto2g", dict(tau=0.01, init_pop=20, target_population=400, real_amplitudes=True, initial_shift=1.0,
                       semi_stoch_space=4, semi_stoch_ci_level=2, semi_stoch_start_iter=5), 6),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                   semi_stoch_space=4, semi_stoch_ci_level=1, semi_stoch_start_iter=12), 3),
    # a 'ci' space of the Hubbard model: CISD of the 4x4 lattice (momentum conserved)
    ("hub_k_4x4", dict(tau=0.01, init_pop=50, target_population=5000, semi_stoch_space=4, semi_stoch_ci_level=2,
                       semi_stoch_start_iter=6), 4),
    # two replicas (replica_tricks) sharing one space, initiator on
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True, nspaces=2,
                   initiator=True, semi_stoch_space=1, semi_stoch_size=250, semi_stoch_start_iter=9), 3),
    # combined annihilation (separate_annihilation = false): the projection as
    # spawns from initiators in the spawned list
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True, initiator=True,
                   semi_stoch_space=1, semi_stoch_size=300, semi_stoch_start_iter=15, semi_stoch_combined=1), 3),
    ("hub_k_4x4", dict(tau=0.01, init_pop=50, target_population=5000, semi_stoch_space=1, semi_stoch_size=40,
                       semi_stoch_start_iter=8, semi_stoch_combined=1), 4),
    ("mol40_w2", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True,
                      semi_stoch_space=4, semi_stoch_ci_level=1, semi_stoch_start_iter=6, semi_stoch_combined=1), 3),
    ("mol26", dict(tau=1e-4, init_pop=2000, target_population=20000, real_amplitudes=True, nspaces=2,
                   initiator=True, semi_stoch_space=1, semi_stoch_size=250, semi_stoch_start_iter=9,
                   semi_stoch_combined=1), 3),
]


@pytest.mark.parametrize("name,opts,nrep", RUNS, ids=["%s-%d" % (r[0], i) for i, r in enumerate(RUNS)])
def test_whole_run_semi_stoch_bit_exact(name, opts, nrep):
    s = SYS[name]
    cfg = make_config(s, ncycles=10, seed=29, state_size=1500000, spawned_state_size=1500000, **opts)
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
        assert rg.nblooms == ro.nblooms
        assert list(rg.shift) == list(ro.shift)
        assert_close(rg.proj_energy[0], ro.proj_energy[0], 1e-10)
    if opts["semi_stoch_space"] == 1:
        assert o.determ_space().shape[0] == opts["semi_stoch_size"]
    else:
        assert o.determ_space().shape[0] > 1
    o.close()


def test_full_space_power_iteration_bit_exact():
    s = SYS["h2o_sto2g"]
    sym = fci.det_symmetry(s, s.aufbau_occ())
    dets = np.array(fci.enumerate_dets(s, sym))
    dets = dets[sort_dets(dets)]
    n = len(dets)
    cfg = make_config(s, tau=0.01, ncycles=20, real_amplitudes=True, initial_shift=-0.3, target_population=1e12,
                      semi_stoch_space=1, semi_stoch_size=n, semi_stoch_start_iter=1, state_size=10000,
                      spawned_state_size=10000, seed=3)
    pops = np.zeros((n, 1), dtype=np.int64)
    pops[0, 0] = 100 << 31
    pops[n // 2, 0] = -(7 << 31)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.set_walkers(dets, pops)
    g.set_walkers(dets, pops)
    for r in range(2):
        o.run_report()
        g.run_report()
        so, po, _ = o.walkers()
        sg, pg, _ = g.walkers()
        np.testing.assert_array_equal(sg, so)
        np.testing.assert_array_equal(pg, po)
    assert sg.shape[0] == n
    o.close()


def test_semi_stoch_refusals():
    from hande_gb300.engine import HgpuError
    s = SYS["mol26"]
    with pytest.raises(HgpuError):  # the replica RDM with a deterministic space
        engine(s, make_config(s, tau=0.01, nspaces=2, density_matrices=True, real_amplitudes=True,
                              semi_stoch_space=1, semi_stoch_size=10, state_size=100, spawned_state_size=100))
    with pytest.raises(HgpuError):  # read_determ_space (an HDF5 file)
        engine(s, make_config(s, tau=0.01, semi_stoch_space=2, semi_stoch_size=10, state_size=100,
                              spawned_state_size=100))


def test_restart_rebuilds_space(tmp_path):
    """A restored calculation builds its deterministic space again at its first
    iteration (src/fciqmc.f90:229-235) and carries on without errors."""
    s = SYS["mol26"]
    cfg = make_config(s, ncycles=10, seed=31, tau=1e-4, init_pop=2000, target_population=20000,
                      real_amplitudes=True, semi_stoch_space=1, semi_stoch_size=200, semi_stoch_start_iter=5,
                      state_size=1500000, spawned_state_size=1500000)
    g = engine(s, cfg)
    g.initial_distribution()
    g.run_report()
    path = str(tmp_path / "ss.ckpt")
    g.checkpoint(path)
    h = engine(s, cfg)
    h.restore(path)
    r = h.run_report()
    assert r.error_flags == 0
    sg, pg, _ = h.walkers()
    assert sg.shape[0] >= 200


@pytest.mark.parametrize("via", ["upload", "snapshot"])
def test_new_list_after_build_rebuilds_space(via):
    """A list that lacks some deterministic states, put in place after the space
    was built (an upload, or the restore of a snapshot taken before the build),
    does not inherit the old space: the space is dropped and built again from
    the new list at the next iteration, bit-exactly as the oracle does."""
    s = SYS["mol26"]
    cfg = make_config(s, ncycles=10, seed=37, tau=1e-4, init_pop=2000, target_population=20000,
                      real_amplitudes=True, semi_stoch_space=1, semi_stoch_size=200, semi_stoch_start_iter=5,
                      state_size=1500000, spawned_state_size=1500000)
    o = Oracle(s, cfg)
    g = engine(s, cfg)
    o.initial_distribution()
    g.initial_distribution()
    if via == "snapshot":
        o.run_cycles(2)
        g.run_cycles(2)
        g.snapshot()
        saved = o.walkers()
    o.run_report()
    g.run_report()  # the space was built at iteration 5
    space = o.determ_space()
    assert space.shape[0] == 200
    if via == "upload":
        st, po, da = o.walkers()
        # drop every other deterministic state from the list
        drop = {tuple(x) for x in space[::2].tolist()}
        keep = np.array([tuple(x) not in drop for x in st.tolist()])
        st, po, da = st[keep], po[keep], da[keep]
        o.set_walkers(st, po, da)
        g.set_walkers(st, po, da)
    else:
        g.snapshot(restore=True)
        o.set_walkers(*saved)
        o.set_state(g.state())  # the snapshot keeps the report's N_w of the shift update
    for r in range(2):
        ro = o.run_report()
        rg = g.run_report()
        assert ro.error_flags == 0 and rg.error_flags == 0
        so, po_, ko = o.walkers()
        sg, pg, kg = g.walkers()
        np.testing.assert_array_equal(sg, so, err_msg="report %d states" % r)
        np.testing.assert_array_equal(pg, po_, err_msg="report %d pops" % r)
        assert_close(kg, ko)
        assert list(rg.shift) == list(ro.shift)
    rebuilt = o.determ_space()
    assert rebuilt.shape[0] == 200 and not np.array_equal(rebuilt, space)
    o.close()
