"""Whole FCIQMC runs on the GPU against exact (FCI) ground-state energies.

The FCI energies are the reference's own (test_suite/fci, tests/golden); the
FCIQMC projected energy, reblocked over the post-equilibration reports
(hande_gb300.analysis, the blocking analysis pyhande applies to HANDE
output), must agree with them within 3 standard errors."""

import json
import os

import numpy as np
import pytest

from hande_gb300 import analysis, systems
from hande_gb300._abi import make_config
from tests.conftest import GOLDEN
from tests.test_gpu_parity import engine

pytestmark = pytest.mark.gpu


def _golden(name):
    for e in json.load(open(os.path.join(GOLDEN, "fci_energies.json"))):
        if e["name"] == name:
            return e["energies"][0]
    raise KeyError(name)


def _h2o():
    return systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))


def _hub3():
    return systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1)


def _exact(s):
    """Lowest eigenvalue in the reference determinant's symmetry sector: the
    reference's own FCI number where its test suite has one for that sector,
    else exact diagonalisation with the oracle's Hamiltonian (pinned against
    the reference's FCI energies in tests/test_oracle_golden.py)."""
    from oracle import fci
    from oracle.pyoracle import Oracle
    w, _ = fci.lowest(Oracle(s, tau=0.01), s, fci.det_symmetry(s, s.aufbau_occ()), nroots=1)
    return float(w[0])


CASES = [
    ("H2O-RHF-sto-2g", _h2o, lambda s: _golden("H2O-RHF-sto-2g"),
     dict(tau=0.01, init_pop=100, target_population=3000, real_amplitudes=True, seed=101), 100, 800),
    ("hubbard_k_3x3_7e", _hub3, _exact,
     dict(tau=0.01, init_pop=10, target_population=20000, seed=202), 100, 800),
]


@pytest.mark.parametrize("name,make,exact,opts,equil,nrep", CASES, ids=[c[0] for c in CASES])
def test_projected_energy_matches_fci(name, make, exact, opts, equil, nrep):
    s = make()
    e_fci = exact(s)
    cfg = make_config(s, ncycles=10, state_size=200000, spawned_state_size=200000, **opts)
    g = engine(s, cfg)
    g.initial_distribution()
    num, d0 = [], []
    for r in range(equil + nrep):
        rep = g.run_report()
        assert rep.error_flags == 0
        if r >= equil:
            num.append(rep.proj_energy[0])
            d0.append(rep.D0_population[0])
    e, err, opt = analysis.projected_energy(num, d0)
    assert np.isfinite(err)
    # E_proj of the reports excludes <D_0|H|D_0> (K_ii and the shift are
    # relative to it, as in HANDE): the total energy adds it back
    from oracle.pyoracle import Oracle
    h00 = Oracle(s, cfg).sc0(np.array(cfg.ref_det[:s.nwords], dtype=np.int64))
    total = e + h00
    assert abs(total - e_fci) < 3.0 * err + 1e-9, (total, e_fci, err)
    assert err < 5e-3
