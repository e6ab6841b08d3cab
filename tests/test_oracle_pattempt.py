"""The default pattempt_single / pattempt_double of molecular systems
(find_single_double_prob, src/qmc_common.F90:152-260): the shares of the
symmetry- and spin-allowed single and double excitations of the reference
determinant.

Pinned twice: against the values HANDE printed for five test-suite systems
(tests/golden/pattempt.json, 8 decimals in the reference's output) and
against a direct enumeration of the excitations here.  Input values, when
given, are normalised as init_excit_gen does (src/qmc.F90:963-971), with
pattempt_double = 1 - the input pattempt_single as written there."""

import json
import os
from itertools import combinations

import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN

CASES = json.load(open(os.path.join(GOLDEN, "pattempt.json")))


def _count(s, occ):
    """Numbers of single and double excitations of occ that conserve spin and
    (XOR) point-group symmetry."""
    virt = [p for p in range(s.nbasis) if p not in set(occ)]
    sym, ms = s.orb_sym, s.orb_ms
    ns = sum(1 for i in occ for a in virt if sym[i] == sym[a] and ms[i] == ms[a])
    nd = 0
    for i, j in combinations(occ, 2):
        for a, b in combinations(virt, 2):
            if ms[i] + ms[j] == ms[a] + ms[b] and (sym[i] ^ sym[j]) == (sym[a] ^ sym[b]):
                nd += 1
    return ns, nd


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_default_pattempt_matches_reference_output(case):
    s = systems.read_in(os.path.join(GOLDEN, case["int_file"]), nel=case["nel"], ms=case["ms"])
    occ = [p - 1 for p in case["det"]]
    cfg = make_config(s, tau=0.01, reference=occ, state_size=100, spawned_state_size=100)
    o = Oracle(s, cfg)
    ps, pd = o.pattempt()
    o.close()
    assert abs(ps - case["pattempt_single"]) < 5.1e-9, (ps, case["pattempt_single"])
    assert abs(pd - case["pattempt_double"]) < 5.1e-9, (pd, case["pattempt_double"])
    ns, nd = _count(s, occ)
    assert ps == ns / (ns + nd) and pd == nd / (ns + nd)


@pytest.mark.parametrize("ms", [0, 2])
def test_default_pattempt_enumeration(ms):
    s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"), nel=10, ms=ms)
    occ = s.aufbau_occ()
    o = Oracle(s, make_config(s, tau=0.01, state_size=100, spawned_state_size=100))
    ps, pd = o.pattempt()
    o.close()
    ns, nd = _count(s, occ)
    assert ps == ns / (ns + nd) and pd == nd / (ns + nd)


def test_pattempt_input_and_hubbard():
    s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))
    o = Oracle(s, make_config(s, tau=0.01, pattempt_single=0.3, pattempt_double=0.9, state_size=100,
                              spawned_state_size=100))
    assert o.pattempt() == (0.3 / (0.3 + 0.9), 1.0 - 0.3)
    o.close()
    h = systems.hubbard_k([[4, 0], [0, 4]], 8)
    o = Oracle(h, make_config(h, tau=0.01, state_size=100, spawned_state_size=100))
    assert o.pattempt() == (0.0, 1.0)
    o.close()
