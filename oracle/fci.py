"""Exact diagonalisation in a determinant space with the oracle's matrix
elements (TEST INFRASTRUCTURE).

Plays the role of HANDE's FCI (src/fci_lapack.F90, fci_utils.F90
generate_hamil :237) for the small systems whose energies the reference's test
suite records; agreement pins the oracle's Slater-Condon rules, integral
indexing and symmetry tables, and hence the Hamiltonian the GPU engine is
compared against."""

from __future__ import annotations

import itertools

import numpy as np

from hande_gb300.systems import System


def det_symmetry(s: System, occ) -> int:
    """symmetry_orb_list: fold the cross product over occupied orbitals from gamma."""
    if s.kind == "hubbard_k":
        gamma = int(np.where(np.all(s.kpoints == 0, axis=1))[0][0])
        sym = gamma
        for p in occ:
            sym = int(s.sym_table[sym, p // 2])
        return sym
    sym = 0
    for p in occ:
        sym ^= int(s.orb_sym[p])
    return sym & (s.nsym_pg - 1)


def enumerate_dets(s: System, sym=None):
    """All determinants with nalpha/nbeta electrons, optionally one symmetry."""
    alpha = [2 * k for k in range(s.nbasis // 2)]
    beta = [2 * k + 1 for k in range(s.nbasis // 2)]
    dets = []
    for ca in itertools.combinations(alpha, s.nalpha):
        for cb in itertools.combinations(beta, s.nbeta):
            occ = sorted(ca + cb)
            if sym is not None and det_symmetry(s, occ) != sym:
                continue
            dets.append(s.encode(occ).astype(np.int64))
    return dets


def hamiltonian(oracle, dets) -> np.ndarray:
    n = len(dets)
    H = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            v = oracle.hmatel(dets[i], dets[j])
            H[i, j] = v
            H[j, i] = v
    return H


def lowest(oracle, s: System, sym=None, nroots: int = 1):
    dets = enumerate_dets(s, sym)
    H = hamiltonian(oracle, dets)
    w = np.linalg.eigvalsh(H)
    return w[:nroots], len(dets)
