"""The diagonal matrix element <D|H|D> is the correctly rounded exact sum of
the slater_condon0 terms, each rounded to a 2^-s grid (ties to even), with s
the largest scale <= 60 for which twice the bound B (the sum of ceil(|term|)
over every term that can occur) times 2^s stays below 2^62.  Checked here
against exact rational arithmetic, independently of the C implementations."""

import math
from fractions import Fraction

import numpy as np

from hande_gb300 import systems
from hande_gb300.systems import v2_index
from oracle.pyoracle import Oracle
from tests.helpers import random_dets


def scale(s) -> int:
    if s.kind == "hubbard_k":
        B = math.ceil(abs(float(s.nalpha * s.nbeta) * s.coulomb_k)) + sum(math.ceil(abs(x)) for x in s.sp_eigv)
    else:
        B = math.ceil(abs(s.ecore))
        for i in range(s.nbasis):
            B += math.ceil(abs(s.h1[i // 2, i // 2]))
            for j in range(i + 1, s.nbasis):
                B += math.ceil(abs(s.v2[v2_index(i // 2, i // 2, j // 2, j // 2)]))
                if i % 2 == j % 2:
                    B += math.ceil(abs(s.v2[v2_index(i // 2, j // 2, j // 2, i // 2)]))
    return max(0, min(60, 61 - B.bit_length()))


def exact_sc0(s, occ, sh):
    def fx(x: float) -> int:
        return round(Fraction(x) * 2 ** sh)  # ties to even

    if s.kind == "hubbard_k":
        e = fx(float(s.nalpha * s.nbeta) * s.coulomb_k) + sum(fx(s.sp_eigv[p]) for p in occ)
        return e
    e = fx(s.ecore)
    for a, i in enumerate(occ):
        e += fx(s.h1[i // 2, i // 2])
        for j in occ[a + 1:]:
            si, sj = i // 2, j // 2
            J = fx(s.v2[v2_index(si, si, sj, sj)])
            K = fx(s.v2[v2_index(si, sj, sj, si)])
            e += J - K if (i % 2) == (j % 2) else J
    return e


def test_exact_diagonal_mol_and_hub():
    rng = np.random.default_rng(1)
    for s in (systems.synthetic_molecule(12, 6, seed=9), systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0)):
        o = Oracle(s, tau=0.01)
        sh = scale(s)

        def to_double(e: int) -> float:
            return float(Fraction(e, 2 ** sh))  # correctly rounded

        dets = random_dets(s, 60, rng, include=[s.aufbau_occ()])
        e0 = exact_sc0(s, s.aufbau_occ(), sh)
        for d in dets:
            occ = s.decode(d.view(np.uint64))
            e = exact_sc0(s, occ, sh)
            assert o.sc0(d) == to_double(e)
        # K_ii of a set of walkers is the rounded exact difference
        st = dets[np.argsort(dets[:, 0].view(np.uint64))]
        o.set_walkers(st, np.ones((st.shape[0], 1), np.int64))
        _, _, kii = o.walkers()
        for d, k in zip(st, kii):
            assert k == to_double(exact_sc0(s, s.decode(d.view(np.uint64)), sh) - e0)
