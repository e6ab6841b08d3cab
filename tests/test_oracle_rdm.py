"""The oracle's replica 2-RDM (src/replica_rdm.F90) on the CPU.

Two checks.  The diagonal part alone (update_rdm of every determinant with
itself) turns calc_rdm_energy into the replica-weighted mean of the diagonal
energies, sum_D w_D (H_DD - H_00) / sum_D w_D with w_D = N_D^(1) N_D^(2), a
closed formula.  And a whole replica run of H2O/STO-2G with density_matrices on
gives an RDM energy whose reblocked mean over the accumulating reports agrees
with the reference's FCI energy (tests/golden) within its error, which pins the
spawned (single and double excitation) contributions and their signs."""

import json
import os

import numpy as np
import pytest

from hande_gb300 import analysis, systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN
from tests.helpers import random_dets


def test_rdm_diagonal_energy_closed_form():
    s = systems.synthetic_molecule(6, 4, seed=3)
    rng = np.random.default_rng(7)
    cfg = make_config(s, tau=0.01, nspaces=2, density_matrices=True, real_amplitudes=True, state_size=1000,
                      spawned_state_size=1000)
    o = Oracle(s, cfg)
    dets = random_dets(s, 40, rng, include=[s.aufbau_occ()])
    order = np.lexsort(dets.view(np.uint64).T)  # one word: ascending unsigned
    dets = dets[order]
    pops = rng.integers(-5 << 31, 5 << 31, size=(dets.shape[0], 2))
    o.set_walkers(dets, pops)
    o.rdm_from_list()
    e, tr = o.rdm_energy()
    h00 = o.sc0(s.encode(s.aufbau_occ()).view(np.int64))
    w = (pops[:, 0] / 2.0 ** 31) * (pops[:, 1] / 2.0 ** 31)
    hdd = np.array([o.sc0(d) for d in dets])
    npair = s.nel * (s.nel - 1) / 2
    assert abs(tr - npair * w.sum()) < 1e-10 * abs(npair * w.sum())
    ref = (w * (hdd - h00)).sum() / w.sum()
    assert abs(e / tr - ref) < 1e-9 * max(1.0, abs(ref))
    rdm = o.rdm()
    assert np.count_nonzero(rdm - np.diag(np.diag(rdm))) == 0
    o.close()


def test_rdm_energy_h2o_matches_fci():
    s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))
    e_fci = [e for e in json.load(open(os.path.join(GOLDEN, "fci_energies.json")))
             if e["name"] == "H2O-RHF-sto-2g"][0]["energies"][0]
    cfg = make_config(s, tau=0.01, ncycles=10, init_pop=200, target_population=5000, real_amplitudes=True,
                      initial_shift=1.0,
                      nspaces=2, density_matrices=True, density_matrix_report=5, seed=31,
                      state_size=20000, spawned_state_size=20000)
    o = Oracle(s, cfg)
    o.initial_distribution()
    h00 = o.sc0(s.encode(s.aufbau_occ()).view(np.int64))
    num, tr = [], []
    for r in range(260):
        rep = o.run_report()
        assert rep.error_flags == 0
        if rep.rdm_trace != 0.0 and r >= 40:
            num.append(rep.rdm_energy)
            tr.append(rep.rdm_trace)
    o.close()
    assert len(num) > 150
    e, err, _ = analysis.projected_energy(num, tr)
    # variational: the replica RDM energy is an upper bound in expectation
    assert abs(e + h00 - e_fci) < max(4.0 * err, 2e-3), (e + h00, e_fci, err)
