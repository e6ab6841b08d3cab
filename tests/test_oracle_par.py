"""The hash-partitioned oracle (the reference's MPI decomposition on threads,
oracle_par_* in oracle/hande_oracle.c) that times the reference algorithm on
all host cores: with one rank it is the plain oracle bit for bit; with several
ranks the merged walker list stays sorted and unique, every determinant lives
on its owner, and the statistics agree with the one-rank calculation."""

import numpy as np
import pytest

from hande_gb300 import analysis, systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle, OraclePar
from tests.helpers import sort_dets


def _run(o, nrep):
    reps = [o.run_report() for _ in range(nrep)]
    return reps, o.walkers()


@pytest.mark.parametrize("case", ["hub_k_4x4", "mol26_replicas_initiator_rdm"])
def test_one_rank_is_the_oracle(case):
    if case == "hub_k_4x4":
        s = systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0)
        cfg = make_config(s, tau=0.005, init_pop=10, target_population=2000, ncycles=10, seed=7,
                          state_size=200000, spawned_state_size=200000)
        nrep = 8
    else:
        s = systems.synthetic_molecule(26, 10, seed=5)
        cfg = make_config(s, tau=1e-4, init_pop=500, target_population=800, ncycles=5, seed=3, real_amplitudes=True,
                          initiator=True, nspaces=2, density_matrices=True, state_size=200000,
                          spawned_state_size=200000)
        nrep = 4
    a, b = Oracle(s, cfg), OraclePar(s, cfg, 1)
    a.initial_distribution()
    b.initial_distribution()
    for r in range(nrep):
        ra, rb = a.run_report(), b.run_report()
        sa, pa, ka = a.walkers()
        sb, pb, kb = b.walkers()
        np.testing.assert_array_equal(sa, sb)
        np.testing.assert_array_equal(pa, pb)
        np.testing.assert_array_equal(ka, kb)
        assert list(ra.shift) == list(rb.shift)
        assert ra.nattempts == rb.nattempts and ra.nspawned == rb.nspawned
        assert ra.proj_energy[0] == rb.proj_energy[0]
        assert ra.rdm_energy == rb.rdm_energy and ra.rdm_trace == rb.rdm_trace
    a.close()
    b.close()


def test_partitioned_list_and_statistics():
    s = systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0)
    nrep = 300
    cfg = make_config(s, tau=0.005, init_pop=100, target_population=3000, ncycles=10, seed=11, initiator=True,
                      state_size=200000, spawned_state_size=200000)
    res = {}
    for P in (1, 4):
        o = OraclePar(s, cfg, P)
        o.initial_distribution()
        num, d0 = [], []
        for r in range(nrep):
            rep = o.run_report()
            assert rep.error_flags == 0
            if r >= 100:
                num.append(rep.proj_energy[0])
                d0.append(rep.D0_population[0])
        st, po, _ = o.walkers()
        order = sort_dets(st)
        assert np.array_equal(order, np.arange(st.shape[0])), "merged list sorted"
        assert np.all(np.any(st[1:] != st[:-1], axis=1)), "merged list unique"
        assert np.all(np.any(po != 0, axis=1)), "no empty states"
        res[P] = analysis.projected_energy(num, d0)
        o.close()
    (e1, s1, _), (e4, s4, _) = res[1], res[4]
    assert abs(e1 - e4) < 3 * np.hypot(s1, s4), (res[1], res[4])
