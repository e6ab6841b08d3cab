"""Whole FCIQMC runs against the reference's own FCIQMC outputs.

tests/golden/reference_fciqmc_runs.json holds, for calculations of HANDE's test
suite, the inputs and the reblocked shift and projected energy of HANDE's own
run (extracted from its benchmark output by tests/golden/make_reference_runs.py).
The same calculation is run here -- same system, reference determinant, tau,
seed value, population control, report length -- and its report table is
reblocked with the same code and window.  The random streams differ (HANDE
draws from dSFMT, this engine from Philox), so the agreement is statistical:
each estimate must lie within 3 combined standard errors of HANDE's."""

import json
import os

import numpy as np
import pytest

from hande_gb300 import analysis, systems
from hande_gb300._abi import make_config
from tests.conftest import GOLDEN

CASES = json.load(open(os.path.join(GOLDEN, "reference_fciqmc_runs.json")))
BY_NAME = {c["name"]: c for c in CASES}
ZMAX = 3.0


def build_system(case):
    p = case["system_params"]
    if case["system"] == "hubbard_k":
        return systems.hubbard_k(p["lattice"], p["electrons"], U=p.get("U", 1.0), t=p.get("t", 1.0),
                                 ms=p.get("ms", 0))
    return systems.read_in(os.path.join(GOLDEN, p["int_file"]), nel=p["nel"], ms=p["ms"])


def build_config(case, s, nreport=None):
    q = case["qmc"]
    ncap = int(max(20 * q["target_particles"], 20000))
    return make_config(
        s, tau=q["tau"], ncycles=q["ncycles"], seed=q["rng_seed"], init_pop=q["D0_population"],
        target_population=q["target_particles"], shift_damping=q["shift_damping"],
        initial_shift=q["initial_shift"], vary_shift_from=q["vary_shift_from"],
        vary_shift_from_proje=q["vary_shift_from_proje"], real_amplitudes=q["real_amplitudes"],
        excit_gen=q["excit_gen"], initiator=q["initiator_approx"], initiator_threshold=q["initiator_pop"],
        quadrature_initiator=case["quadrature_initiator"],
        nspaces=2 if (case["replica_tricks"] or case["density_matrices"]) else 1,
        density_matrices=case["density_matrices"], reference=[d - 1 for d in case["reference_det"]],
        shift_harmonic_forcing=q.get("shift_harmonic_forcing", 0.0), state_size=ncap, spawned_state_size=ncap)


def window(shift, initial_shift):
    """The fixture generator's window: 10 reports after the shift first moves."""
    moved = np.nonzero(np.asarray(shift) != initial_shift)[0]
    first = int(moved[0]) if moved.size else len(shift)
    return first + 10


def run_and_compare(case, make_engine, nreport=None):
    s = build_system(case)
    cfg = build_config(case, s)
    e = make_engine(s, cfg)
    e.initial_distribution()
    q = case["qmc"]
    if q.get("shift_harmonic_forcing", 0.0) and not q.get("shift_harmonic_forcing_two_stage", False):
        # harmonic forcing from the first report (src/qmc.F90:209-212)
        st = e.get_state() if hasattr(e, "get_state") else e.state()
        for k in range(e.R):
            st.vary_shift[k] = 1
        e.set_state(st)
    shift, num, d0 = [], [], []
    for _ in range(nreport or case["qmc"]["nreport"]):
        r = e.run_report()
        assert r.error_flags == 0
        shift.append(r.shift[0])
        num.append(r.proj_energy[0])
        d0.append(r.D0_population[0])
    e.close()
    k0 = window(shift, case["qmc"]["initial_shift"])
    assert len(shift) - k0 >= 32, "the shift never varied long enough"
    S, Serr, _ = analysis.mean_error(shift[k0:])
    E, Eerr, _ = analysis.projected_energy(num[k0:], d0[k0:])
    ref = case["reference_stats"]
    zE = (E - ref["proj_energy"]) / np.hypot(Eerr, ref["proj_energy_error"])
    zS = (S - ref["shift"]) / np.hypot(Serr, ref["shift_error"])
    msg = "%s: E_proj %.6f(%.6f) vs HANDE %.6f(%.6f), z=%.2f; shift %.5f(%.5f) vs %.5f(%.5f), z=%.2f" % (
        case["name"], E, Eerr, ref["proj_energy"], ref["proj_energy_error"], zE, S, Serr, ref["shift"],
        ref["shift_error"], zS)
    print(msg)
    assert abs(zE) < ZMAX, msg
    assert abs(zS) < ZMAX, msg
    return E, Eerr


@pytest.mark.gpu
@pytest.mark.parametrize("name", [c["name"] for c in CASES])
def test_engine_matches_reference_run(name):
    from hande_gb300.engine import Engine
    run_and_compare(BY_NAME[name], Engine)


def exact_energy(s, cfg):
    """Lowest eigenvalue, relative to the reference's diagonal element, of the
    Hamiltonian over every determinant with the system's alpha and beta
    electron counts (the oracle's matrix elements; a few thousand
    determinants)."""
    import itertools
    import scipy.sparse as sparse
    import scipy.sparse.linalg as sla
    from oracle.pyoracle import Oracle
    o = Oracle(s, cfg)
    norb = s.nbasis // 2
    words = []
    for a in itertools.combinations(range(norb), s.nalpha):
        for b in itertools.combinations(range(norb), s.nbeta):
            words.append(int(s.encode([2 * i for i in a] + [2 * i + 1 for i in b])[0]))
    as_det = lambda x: np.array([x], dtype=np.uint64).astype(np.int64)
    e0 = o.sc0(as_det(int(cfg.ref_det[0])))
    rows, cols, vals = [], [], []
    for i, fi in enumerate(words):
        for j in range(i, len(words)):
            if bin(fi ^ words[j]).count("1") > 4:
                continue
            v = o.sc0(as_det(fi)) - e0 if i == j else o.hmatel(as_det(fi), as_det(words[j]))
            if v != 0.0:
                rows += [i, j] if i != j else [i]
                cols += [j, i] if i != j else [i]
                vals += [v, v] if i != j else [v]
    o.close()
    h = sparse.csr_matrix((vals, (rows, cols)), shape=(len(words), len(words)))
    return float(sla.eigsh(h, k=1, which="SA")[0][0])


@pytest.mark.gpu
def test_harmonic_population_control_n2():
    """HANDE's N2 STO-3G test with critically damped harmonic population control
    switched on at the target (test_suite/fciqmc/np4/N2-RHF-STO-3G-harmonic_pop_control_two_stage:
    tau 0.001, 10 cycles a report, seed 21, 100 initial walkers, target 2e4,
    shift_damping 0.04, shift_harmonic_crit_damp, shift_harmonic_forcing_two_stage).
    HANDE's own run reaches its target at report 2657 of 2800, too late for its
    statistics (133 reports, no reblocking plateau; its E_proj lies 4 standard
    errors from the exact energy), so the run here is compared with the exact
    energy of the 3136-determinant space: 4000 reports, E_proj within 3
    standard errors, and the population held at the target."""
    from hande_gb300.engine import Engine
    s = systems.read_in(os.path.join(GOLDEN, "N2-RHF-STO-3G.fcidump"))
    cfg = make_config(s, tau=0.001, ncycles=10, seed=21, init_pop=100, target_population=2e4, shift_damping=0.04,
                      shift_harmonic_forcing=0.04 ** 2 / 4, state_size=200000, spawned_state_size=200000)
    e_exact = exact_energy(s, cfg)
    e = Engine(s, cfg)
    e.initial_distribution()
    shift, num, d0, nw = [], [], [], []
    for _ in range(4000):
        r = e.run_report()
        assert r.error_flags == 0
        shift.append(r.shift[0])
        num.append(r.proj_energy[0])
        d0.append(r.D0_population[0])
        nw.append(r.nparticles[0])
    e.close()
    k0 = window(shift, 0.0)
    assert len(shift) - k0 >= 500, "the target population was reached too late"
    E, Eerr, _ = analysis.projected_energy(num[k0:], d0[k0:])
    msg = "E_proj %.6f(%.6f) vs exact %.6f" % (E, Eerr, e_exact)
    print(msg)
    assert abs(E - e_exact) < 3.0 * Eerr, msg
    assert abs(np.mean(nw[k0:]) - 2e4) < 0.1 * 2e4, np.mean(nw[k0:])
