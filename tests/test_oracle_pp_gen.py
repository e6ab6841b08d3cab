"""The oracle's uniform_power_pitzer, uniform_cauchy_schwarz,
heat_bath_power_pitzer and heat_bath_cauchy_schwarz generators
(gen_excit_mol_power_pitzer_occ, src/excit_gen_power_pitzer_mol.F90:1260-1547)
on the CPU.

i, j are uniform over the occupied pairs, or (heat_bath_ variants) i with
weight sum_j w_ij and j with weight w_ij, w_ij = sum over ordered a /= b of
|<ij||ab>| (init_double_weights_ab, src/excit_gen_utils.f90:68-138); a is
drawn for i among the determinant's unoccupied orbitals of i's spin with weights sqrt|<ia|ai>|
(power_pitzer) or sqrt|<ia|ia>| (cauchy_schwarz), b for j among the orbitals
of the spin and irrep that conserve both, a excluded.  The probability of an
excitation is restated here from that definition (both orders for parallel
spins) and checked against the p_gen the generator returns, and the
frequencies of many draws from one determinant against both."""

import collections
import functools
import math
import os

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle
from tests.conftest import GOLDEN
from tests.test_oracle_spin_gen import _sc2_abs


def _weight(s, p, q, cs):
    if cs:
        return math.sqrt(abs(s.v2[systems.v2_index(p >> 1, p >> 1, q >> 1, q >> 1)]))  # <pq|pq> = (pp|qq)
    if s.orb_ms[p] != s.orb_ms[q]:
        return 0.0
    return math.sqrt(abs(s.v2[systems.v2_index(p >> 1, q >> 1, q >> 1, p >> 1)]))  # <pq|qp> = (pq|qp)


def _ij_weights(s):
    ms, sym = s.orb_ms, s.orb_sym

    @functools.lru_cache(maxsize=None)
    def w(i, j):
        if i == j:
            return 0.0
        it, jt = min(i, j), max(i, j)
        tot = 0.0
        for a in range(s.nbasis):
            if a in (it, jt):
                continue
            for b in range(s.nbasis):
                if b in (a, it, jt) or sym[b] != sym[it] ^ sym[jt] ^ sym[a]:
                    continue
                if (ms[it] == ms[a] and ms[jt] == ms[b]) or (ms[it] == ms[b] and ms[jt] == ms[a]):
                    tot += _sc2_abs(s, it, jt, min(a, b), max(a, b))
        return tot
    return w


def _pij(s, occ, i, j, wij):
    """select_ij_heat_bath: p(i) p(j|i) + p(j) p(i|j)."""
    wi = {p: sum(wij(p, q) for q in range(s.nbasis)) for p in occ}
    ti = sum(wi.values())

    def cond(p, q):
        return wij(p, q) / sum(wij(p, r) for r in occ)
    return wi[i] / ti * cond(i, j) + wi[j] / ti * cond(j, i)


def _pgen_double(s, occ, i, j, a, b, cs, pdouble, pij):
    """pattempt_double * p(ij) * sum over the orders (x from i, y from j)."""
    occs = set(occ)
    ms, sym = s.orb_ms, s.orb_sym
    unocc_i = [p for p in range(s.nbasis) if p not in occs and ms[p] == ms[i]]
    wi = {p: _weight(s, i, p, cs) for p in unocc_i}
    ti = sum(wi[p] for p in unocc_i)
    tot = 0.0
    for x, y in ((a, b), (b, a)):
        if ms[x] != ms[i] or ms[y] != ms[j]:
            continue
        lst = [p for p in range(s.nbasis) if ms[p] == ms[y] and sym[p] == sym[y]]
        wj = {p: (_weight(s, j, p, cs) if p != x else 0.0) for p in lst}
        tot += wi[x] / ti * wj[y] / sum(wj.values())
    return pdouble * pij * tot


@pytest.mark.parametrize("gen", ["uniform_power_pitzer", "uniform_cauchy_schwarz", "heat_bath_power_pitzer",
                                 "heat_bath_cauchy_schwarz"])
@pytest.mark.parametrize("sysname", ["synthetic", "h2o"])
def test_pp_occ_pgen_matches_sampling(gen, sysname):
    if sysname == "h2o":
        s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))
    else:
        s = systems.synthetic_molecule(6, 4, seed=3)
    cs = "cauchy_schwarz" in gen
    wij = _ij_weights(s) if gen.startswith("heat_bath") else None
    rng = np.random.default_rng(5)
    occs = [s.aufbau_occ()]
    for _ in range(2):
        occs.append(sorted(int(x) for x in rng.choice(s.nbasis, s.nel, replace=False)))
    n = 200000
    cfg = make_config(s, tau=0.01, excit_gen=gen, seed=11, state_size=1000, spawned_state_size=1000)
    o = Oracle(s, cfg)
    _, pdouble = o.pattempt()
    for occ in occs:
        parent = s.encode(occ).view(np.int64)
        orbs, pg, hm, al, ns = o.eval_excitations(np.tile(parent, (n, 1)), np.ones(n, np.int64), 3)
        counts = collections.Counter()
        pgen = {}
        for k in np.nonzero(al)[0]:
            key = tuple(orbs[k])
            counts[key] += 1
            if key in pgen:
                # the two orders are summed in the order they were drawn: equal to rounding
                assert abs(pgen[key] - pg[k]) <= 1e-14 * pg[k]
            pgen[key] = pg[k]
        ndouble = 0
        for key, p in pgen.items():
            if key[1] >= 0:
                ndouble += 1
                i, j = key[0], key[1]
                pij = _pij(s, occ, i, j, wij) if wij else 2.0 / (s.nel * (s.nel - 1))
                ref = _pgen_double(s, occ, i, j, key[2], key[3], cs, pdouble, pij)
                assert abs(p - ref) <= 1e-12 * ref, (key, p, ref)
        assert ndouble > 10
        total = sum(pgen.values())
        frac = al.mean()
        assert abs(frac - total) < 5 * np.sqrt(frac * (1 - frac) / n) + 1e-3
        z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
        assert max(abs(x) for x in z) < 5.0
    o.close()


@pytest.mark.parametrize("sysname", ["synthetic", "h2o"])
@pytest.mark.parametrize("min_weight", [0.01, 0.0])
def test_pp_ref_pgen_matches_sampling(sysname, min_weight):
    """heat_bath_power_pitzer_ref (gen_excit_mol_power_pitzer_orderN,
    src/excit_gen_power_pitzer_mol.F90:941-1258): i, j positions of the
    reference's occupied list mapped onto the determinant, a and b from tables
    built once.  Each excitation's frequency over many draws matches its p_gen,
    including determinants far from the reference."""
    if sysname == "h2o":
        s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))
    else:
        s = systems.synthetic_molecule(6, 4, seed=3)
    rng = np.random.default_rng(8)
    occs = [s.aufbau_occ()]
    while len(occs) < 3:
        occ = sorted(int(x) for x in rng.choice(s.nbasis, s.nel, replace=False))
        if sum(s.orb_ms[p] for p in occ) == sum(s.orb_ms[p] for p in s.aufbau_occ()):
            occs.append(occ)
    n = 200000
    cfg = make_config(s, tau=0.01, excit_gen="heat_bath_power_pitzer_ref", seed=13, state_size=1000,
                      spawned_state_size=1000, power_pitzer_min_weight=min_weight)
    o = Oracle(s, cfg)
    for occ in occs:
        parent = s.encode(occ).view(np.int64)
        orbs, pg, hm, al, ns = o.eval_excitations(np.tile(parent, (n, 1)), np.ones(n, np.int64), 3)
        counts = collections.Counter()
        pgen = {}
        for k in np.nonzero(al)[0]:
            key = tuple(orbs[k])
            counts[key] += 1
            if key in pgen:
                assert abs(pgen[key] - pg[k]) <= 1e-14 * pg[k]
            pgen[key] = pg[k]
        assert sum(1 for key in pgen if key[1] >= 0) > 10
        total = sum(pgen.values())
        frac = al.mean()
        assert abs(frac - total) < 5 * np.sqrt(frac * (1 - frac) / n) + 1e-3
        z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
        assert max(abs(x) for x in z) < 5.0
    o.close()
