"""The oracle's spin-resolved molecular generators (renorm_spin, no_renorm_spin,
src/excit_gen_mol.f90:103-380 with choose_ij_spin_mol :684-783) on the CPU.

choose_ij_spin_mol first decides whether the two electrons have parallel
spins (probability pattempt_parallel), then picks the pair within that spin
class; p_gen is the product of that choice with the uniform a, b choice.  Over
many draws from one determinant each excitation's frequency must match its
p_gen.  pattempt_parallel itself, when not given, is the |<ij||ab>| share of
parallel-spin pairs (find_parallel_spin_prob_mol, src/qmc_common.F90:265-378),
checked against a direct sum here."""

import collections

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle


def _sc2_abs(s, i, j, a, b):
    """|<ij|ab> - <ij|ba>| with the spin selection of slater_condon2_mol_excit."""
    def v(p, q, r, t):  # <pq|rt> = (pr|qt) over spatial orbitals
        return s.v2[systems.v2_index(p >> 1, r >> 1, q >> 1, t >> 1)]
    h = 0.0
    if s.orb_ms[i] == s.orb_ms[a]:
        h = v(i, j, a, b)
    if s.orb_ms[i] == s.orb_ms[b]:
        h = h - v(i, j, b, a)
    return abs(h)


def _parallel_share(s):
    par = orth = 0.0
    nb = s.nbasis
    for i in range(nb):
        for j in range(nb):
            if i == j:
                continue
            it, jt = min(i, j), max(i, j)
            ij_sym = s.orb_sym[it] ^ s.orb_sym[jt]
            for a in range(nb):
                if a in (i, j):
                    continue
                isymb = ij_sym ^ s.orb_sym[a]
                for b in range(nb):
                    ms = s.orb_ms
                    spin_ok = (ms[it] == ms[a] and ms[jt] == ms[b]) or (ms[it] == ms[b] and ms[jt] == ms[a])
                    if not spin_ok or s.orb_sym[b] != isymb or b in (a, i, j):
                        continue
                    h = _sc2_abs(s, it, jt, min(a, b), max(a, b))
                    if ms[it] == ms[jt]:
                        par += h
                    else:
                        orth += h
    return par / (par + orth)


def _sample(s, gen, parent, n, pp, seed=11):
    cfg = make_config(s, tau=0.01, excit_gen=gen, seed=seed, pattempt_parallel=pp, state_size=1000,
                      spawned_state_size=1000)
    o = Oracle(s, cfg)
    par = np.tile(parent, (n, 1))
    orbs, pg, hm, al, ns = o.eval_excitations(par, np.ones(n, np.int64), 3)
    pp_used = o.pattempt_parallel()
    o.close()
    return orbs, pg, al, pp_used


@pytest.mark.parametrize("gen", ["renorm_spin", "no_renorm_spin"])
@pytest.mark.parametrize("pp", [0.3, -1.0])
def test_spin_generator_pgen_matches_sampling(gen, pp):
    s = systems.synthetic_molecule(6, 4, seed=3)
    rng = np.random.default_rng(5)
    parents = [s.encode(s.aufbau_occ()).view(np.int64)]
    a = rng.choice(s.nbasis // 2, s.nalpha, replace=False)
    b = rng.choice(s.nbasis // 2, s.nbeta, replace=False)
    parents.append(s.encode(sorted([2 * int(x) for x in a] + [2 * int(x) + 1 for x in b])).view(np.int64))
    n = 200000
    for parent in parents:
        orbs, pg, al, pp_used = _sample(s, gen, parent, n, pp)
        if pp >= 0:
            assert pp_used == pp
        counts = collections.Counter()
        pgen = {}
        for k in np.nonzero(al)[0]:
            key = tuple(orbs[k])
            counts[key] += 1
            if key in pgen:
                assert pgen[key] == pg[k]
            pgen[key] = pg[k]
        total = sum(pgen.values())
        frac = al.mean()
        assert abs(frac - total) < 5 * np.sqrt(frac * (1 - frac) / n) + 1e-3
        z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
        assert max(abs(x) for x in z) < 5.0


def test_parallel_spin_probability():
    s = systems.synthetic_molecule(6, 4, seed=3)
    cfg = make_config(s, tau=0.01, excit_gen="renorm_spin", state_size=100, spawned_state_size=100)
    o = Oracle(s, cfg)
    pp = o.pattempt_parallel()
    o.close()
    ref = _parallel_share(s)
    assert 0.0 < pp < 1.0
    assert abs(pp - ref) < 1e-12 * ref


def test_spin_generator_one_beta():
    """With a single beta electron no beta-beta pair exists: those draws are
    not allowed (allowed_excitation = .false.), the others still sample
    their p_gen."""
    s = systems.synthetic_molecule(5, 3, seed=8, ms=1)
    assert s.nbeta == 1
    parent = s.encode(s.aufbau_occ()).view(np.int64)
    n = 100000
    orbs, pg, al, _ = _sample(s, "renorm_spin", parent, n, 0.5)
    pgen = {}
    counts = collections.Counter()
    for k in np.nonzero(al)[0]:
        key = tuple(orbs[k])
        counts[key] += 1
        pgen[key] = pg[k]
        if orbs[k][1] >= 0:
            assert not (s.orb_ms[orbs[k][0]] < 0 and s.orb_ms[orbs[k][1]] < 0)
    z = [(c / n - pgen[k]) / np.sqrt(pgen[k] * (1 - pgen[k]) / n) for k, c in counts.items()]
    assert max(abs(x) for x in z) < 5.0
