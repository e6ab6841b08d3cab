"""The oracle's semi-stochastic projection (src/semi_stoch.F90, 'high' space,
separate annihilation) on the CPU.

Three checks.  The space is the find_most_populated_dets selection
(src/semi_stoch.F90:1318-1385), ties included, restated here in Python.  With
every determinant of the symmetry sector in the space no stochastic spawn
survives (deterministic parents do not spawn onto deterministic children) and
death is skipped, so a run is the power iteration c <- c - tau (K - S) c up to
the rounding of amplitudes to 2^-31: compared with dense numpy.  And with a
small space inside a stochastic run of H2O/STO-2G the reblocked projected
energy agrees with the reference's FCI energy (tests/golden)."""

import json
import os

import numpy as np

from hande_gb300 import analysis, systems
from hande_gb300._abi import make_config
from oracle import fci
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN
from tests.helpers import sort_dets


def _h2o():
    return systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))


def _most_populated(pops, k):
    """find_most_populated_dets: scan in order, replace the first smallest."""
    tot = np.abs(pops).sum(axis=1)
    sel = list(range(k))
    val = [int(tot[i]) for i in sel]
    mi = min(range(k), key=lambda q: (val[q], q))
    for i in range(k, len(tot)):
        if tot[i] > val[mi]:
            sel[mi] = i
            val[mi] = int(tot[i])
            mi = min(range(k), key=lambda q: (val[q], q))
    return sorted(sel)


def test_space_is_most_populated_with_ties():
    s = _h2o()
    sym = fci.det_symmetry(s, s.aufbau_occ())
    dets = np.array(fci.enumerate_dets(s, sym))
    dets = dets[sort_dets(dets)]
    rng = np.random.default_rng(4)
    pops = rng.integers(1, 6, size=(len(dets), 1)) * (1 << 31)  # many ties
    cfg = make_config(s, tau=0.01, real_amplitudes=True, semi_stoch_space=1, semi_stoch_size=17,
                      semi_stoch_start_iter=1, target_population=1e12, state_size=10000, spawned_state_size=10000)
    o = Oracle(s, cfg)
    o.set_walkers(dets, pops)
    o.run_report()
    got = o.determ_space()
    o.close()
    want = dets[_most_populated(pops, 17)]
    np.testing.assert_array_equal(got, want)


def test_full_space_is_power_iteration():
    s = _h2o()
    sym = fci.det_symmetry(s, s.aufbau_occ())
    dets = np.array(fci.enumerate_dets(s, sym))
    dets = dets[sort_dets(dets)]
    n = len(dets)
    tau, shift, ncyc = 0.01, -0.3, 20
    cfg = make_config(s, tau=tau, ncycles=ncyc, real_amplitudes=True, initial_shift=shift, target_population=1e12,
                      semi_stoch_space=1, semi_stoch_size=n, semi_stoch_start_iter=1, state_size=10000,
                      spawned_state_size=10000)
    o = Oracle(s, cfg)
    f0 = s.encode(s.aufbau_occ()).view(np.int64)
    i0 = int(np.nonzero((dets == f0).all(axis=1))[0][0])
    pops = np.zeros((n, 1), dtype=np.int64)
    pops[i0, 0] = 100 << 31
    pops[(i0 + 1) % n, 0] = 7 << 31
    o.set_walkers(dets, pops)
    H = fci.hamiltonian(o, list(dets))
    h00 = o.sc0(f0)
    o.run_report()
    st, po, _ = o.walkers()
    o.close()
    assert st.shape[0] == n  # deterministic states stay, even when empty
    np.testing.assert_array_equal(st, dets)
    K = H - h00 * np.eye(n)
    c = pops[:, 0] / 2.0 ** 31
    for _ in range(ncyc):
        c = c - tau * (K @ c - shift * c)
    got = po[:, 0] / 2.0 ** 31
    assert np.abs(got - c).max() < 1e-6 * np.abs(c).max()


def test_semi_stoch_energy_h2o_matches_fci():
    s = _h2o()
    e_fci = [e for e in json.load(open(os.path.join(GOLDEN, "fci_energies.json")))
             if e["name"] == "H2O-RHF-sto-2g"][0]["energies"][0]
    cfg = make_config(s, tau=0.01, ncycles=10, init_pop=20, target_population=300, real_amplitudes=True,
                      initial_shift=1.0, semi_stoch_space=1, semi_stoch_size=12, semi_stoch_start_iter=2 ** 62, semi_stoch_shift_iter=30,
                      seed=77, state_size=20000, spawned_state_size=20000)
    o = Oracle(s, cfg)
    o.initial_distribution()
    h00 = o.sc0(s.encode(s.aufbau_occ()).view(np.int64))
    num, den = [], []
    built = False
    for r in range(300):
        rep = o.run_report()
        assert rep.error_flags == 0
        built = built or o.determ_space().shape[0] > 0
        if built and r >= 60:
            num.append(rep.proj_energy[0])
            den.append(rep.D0_population[0])
    assert o.determ_space().shape[0] == 12
    o.close()
    assert len(num) > 150
    e, err, _ = analysis.projected_energy(num, den)
    assert abs(e + h00 - e_fci) < max(4.0 * err, 2e-3), (e + h00, e_fci, err)


def test_ci_space_contents():
    """create_ci_determ_space: every determinant of the reference's spin and
    symmetry within ex_level excitations of it."""
    s = _h2o()
    sym = fci.det_symmetry(s, s.aufbau_occ())
    f0 = s.encode(s.aufbau_occ()).view(np.int64)
    for level in (1, 2):
        cfg = make_config(s, tau=0.01, real_amplitudes=True, semi_stoch_space=4, semi_stoch_ci_level=level,
                          semi_stoch_start_iter=1, state_size=10000, spawned_state_size=10000)
        o = Oracle(s, cfg)
        o.initial_distribution()
        o.run_report()
        got = o.determ_space()
        st, po, _ = o.walkers()
        o.close()
        dets = np.array(fci.enumerate_dets(s, sym))
        xl = [bin(int(np.bitwise_xor(d, f0).view(np.uint64)[0])).count("1") // 2 for d in dets]
        want = dets[np.array(xl) <= level]
        want = want[sort_dets(want)]
        np.testing.assert_array_equal(got, want)
        assert st.shape[0] >= want.shape[0]  # all in the main list, with zero population if need be


def test_ci_space_contents_hubbard():
    """A 'ci' space of the Hubbard model in momentum space: every determinant of
    the reference's spin and crystal momentum within ex_level excitations of it
    (enumerate_determinants restricted to ex_level, as create_ci_determ_space
    asks for any system)."""
    s = systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1)
    sym = fci.det_symmetry(s, s.aufbau_occ())
    f0 = s.encode(s.aufbau_occ()).view(np.int64)
    dets = np.array(fci.enumerate_dets(s, sym))
    xl = np.array([bin(int(np.bitwise_xor(d, f0).view(np.uint64)[0])).count("1") // 2 for d in dets])
    for level in (1, 2):
        cfg = make_config(s, tau=0.01, semi_stoch_space=4, semi_stoch_ci_level=level, semi_stoch_start_iter=1,
                          state_size=20000, spawned_state_size=20000)
        o = Oracle(s, cfg)
        o.initial_distribution()
        o.run_report()
        got = o.determ_space()
        o.close()
        want = dets[xl <= level]
        want = want[sort_dets(want)]
        # a single excitation changes the momentum: level 1 is the reference alone
        assert want.shape[0] == 1 if level == 1 else want.shape[0] > 50
        np.testing.assert_array_equal(got, want)
