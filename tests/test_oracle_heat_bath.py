"""The oracle's heat-bath generators (src/excit_gen_heat_bath_mol.F90) on the CPU.

The generation probability p_gen that gen_excit_mol_heat_bath[_uniform]
returns is a closed formula (the four orderings of i, j and a, b, or the
uniform variant's two); the generator itself samples through alias tables.
Both are restated from the reference, so their agreement is a check of the
restatement: over many draws from one determinant, each excitation's frequency
must match its p_gen, and the allowed fraction must match the p_gen total."""

import collections

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle


def _sample(s, gen, parent, n, seed=11):
    cfg = make_config(s, tau=0.01, excit_gen=gen, seed=seed, state_size=1000, spawned_state_size=1000)
    o = Oracle(s, cfg)
    par = np.tile(parent, (n, 1))
    orbs, pg, hm, al, ns = o.eval_excitations(par, np.ones(n, np.int64), 3)
    return orbs, pg, al


@pytest.mark.parametrize("gen", ["heat_bath", "heat_bath_uniform", "heat_bath_single"])
def test_heat_bath_pgen_matches_sampling(gen):
    s = systems.synthetic_molecule(6, 4, seed=3)
    rng = np.random.default_rng(5)
    parents = [s.encode(s.aufbau_occ()).view(np.int64)]
    occ = sorted(rng.choice(s.nbasis, s.nel, replace=False))
    parents.append(s.encode(occ).view(np.int64))
    n = 200000
    for parent in parents:
        orbs, pg, al = _sample(s, gen, parent, n)
        counts = collections.Counter()
        pgen = {}
        for k in np.nonzero(al)[0]:
            key = tuple(orbs[k])
            counts[key] += 1
            if key in pgen:
                # the four orderings are summed in the order they were drawn: equal to rounding
                assert abs(pgen[key] - pg[k]) <= 1e-14 * pg[k]
            pgen[key] = pg[k]
        total = sum(pgen.values())
        frac = al.mean()
        assert abs(frac - total) < 5 * np.sqrt(frac * (1 - frac) / n) + 1e-3
        z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
        assert max(abs(x) for x in z) < 5.0


def test_heat_bath_bias_check():
    """With Coulomb-only integrals no double excitation has weight, so a valid
    single i -> a has no j: the original heat bath refuses the system
    (src/excit_gen_heat_bath_mol.F90:185-197); the uniform variant accepts it."""
    M = 5
    h = np.diag(-1.0 + 0.2 * np.arange(M)) + 0.01 * (np.ones((M, M)) - np.eye(M))
    v = np.zeros(systems.tri0(systems.tri0(M - 1, M - 1), systems.tri0(M - 1, M - 1)) + 1)
    for p in range(M):
        for q in range(M):
            v[systems.v2_index(p, p, q, q)] = 0.5 / (1 + abs(p - q))  # (pp|qq) only
    s = systems.molecular_from_arrays(h, v, 4)
    cfg = make_config(s, tau=0.01, excit_gen="heat_bath", seed=1, state_size=100, spawned_state_size=100)
    with pytest.raises(RuntimeError):
        Oracle(s, cfg)
    cfg = make_config(s, tau=0.01, excit_gen="heat_bath_uniform", seed=1, state_size=100, spawned_state_size=100)
    Oracle(s, cfg).close()
