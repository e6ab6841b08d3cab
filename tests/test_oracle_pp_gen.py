"""The oracle's uniform_power_pitzer and uniform_cauchy_schwarz generators
(gen_excit_mol_power_pitzer_occ with uniform i, j,
src/excit_gen_power_pitzer_mol.F90:1260-1547) on the CPU.

i, j are uniform over the occupied pairs; a is drawn for i among the
determinant's unoccupied orbitals of i's spin with weights sqrt|<ia|ai>|
(power_pitzer) or sqrt|<ia|ia>| (cauchy_schwarz), b for j among the orbitals
of the spin and irrep that conserve both, a excluded.  The probability of an
excitation is restated here from that definition (both orders for parallel
spins) and checked against the p_gen the generator returns, and the
frequencies of many draws from one determinant against both."""

import collections
import math

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle


def _weight(s, p, q, cs):
    if cs:
        return math.sqrt(abs(s.v2[systems.v2_index(p >> 1, p >> 1, q >> 1, q >> 1)]))  # <pq|pq> = (pp|qq)
    if s.orb_ms[p] != s.orb_ms[q]:
        return 0.0
    return math.sqrt(abs(s.v2[systems.v2_index(p >> 1, q >> 1, q >> 1, p >> 1)]))  # <pq|qp> = (pq|qp)


def _pgen_double(s, occ, i, j, a, b, cs, pdouble):
    """pattempt_double * p(ij) * sum over the orders (x from i, y from j)."""
    nel = len(occ)
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
    return pdouble * (2.0 / (nel * (nel - 1))) * tot


@pytest.mark.parametrize("gen", ["uniform_power_pitzer", "uniform_cauchy_schwarz"])
@pytest.mark.parametrize("sysname", ["synthetic", "h2o"])
def test_pp_occ_pgen_matches_sampling(gen, sysname):
    from tests.conftest import GOLDEN
    import os
    if sysname == "h2o":
        s = systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))
    else:
        s = systems.synthetic_molecule(6, 4, seed=3)
    cs = gen == "uniform_cauchy_schwarz"
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
                ref = _pgen_double(s, occ, key[0], key[1], key[2], key[3], cs, pdouble)
                assert abs(p - ref) <= 1e-12 * ref, (key, p, ref)
        assert ndouble > 10
        total = sum(pgen.values())
        frac = al.mean()
        assert abs(frac - total) < 5 * np.sqrt(frac * (1 - frac) / n) + 1e-3
        z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
        assert max(abs(x) for x in z) < 5.0
    o.close()
