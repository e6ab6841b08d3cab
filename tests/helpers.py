"""Shared test fixtures: seeded random determinant lists and spawned lists."""

from __future__ import annotations

import numpy as np

from hande_gb300 import systems


def random_dets(s: systems.System, n: int, rng, include=()):
    """n distinct random determinants (nalpha alpha, nbeta beta) as int64 words."""
    seen = set()
    out = []
    for occ in include:
        f = tuple(int(x) for x in s.encode(occ))
        if f not in seen:
            seen.add(f)
            out.append(f)
    na = s.nbasis // 2
    tries = 0
    while len(out) < n and tries < 50 * n:
        tries += 1
        a = rng.choice(na, s.nalpha, replace=False)
        b = rng.choice(na, s.nbeta, replace=False)
        occ = sorted([2 * int(x) for x in a] + [2 * int(x) + 1 for x in b])
        f = tuple(int(x) for x in s.encode(occ))
        if f not in seen:
            seen.add(f)
            out.append(f)
    arr = np.array(out, dtype=np.uint64).reshape(len(out), s.nwords)
    return arr.view(np.int64)


def sort_dets(d: np.ndarray) -> np.ndarray:
    """Order of HANDE's main list: unsigned, last word most significant."""
    u = d.view(np.uint64)
    keys = tuple(u[:, k] for k in range(u.shape[1]))  # lexsort: last key is primary
    return np.lexsort(keys)


def small_systems():
    return {
        "hub_k_4x4": systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0),
        "hub_k_3x3": systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1),
        "mol_h2o": None,  # filled lazily (needs the golden file)
        "mol_w1": systems.synthetic_molecule(26, 10, seed=5),
        "mol_w2": systems.synthetic_molecule(40, 12, seed=6),
    }


def main_and_spawns(s, rng, nmain, nspawn, R, real, initiator, hit_frac=0.5, dup_frac=0.4):
    """A sorted, unique main list and a spawned list sdata(W+R+1, n) that hits it,
    spawns onto new determinants, repeats determinants and cancels exactly."""
    pool = random_dets(s, nmain + nspawn, rng)
    main = pool[:nmain]
    main = main[sort_dets(main)]
    factor = (1 << 31) if real else 1
    pops = np.zeros((nmain, R), dtype=np.int64)
    for q in range(R):
        if real:
            pops[:, q] = (rng.integers(-3 * factor, 3 * factor, nmain))
        else:
            pops[:, q] = rng.integers(-20, 21, nmain)
    newp = pool[nmain:]
    W = s.nwords
    rows = []
    for k in range(nspawn):
        r = rng.random()
        if r < hit_frac:
            d = main[rng.integers(nmain)]
        else:
            d = newp[rng.integers(max(1, len(newp) // 3))]  # reuse to create duplicates
        q = int(rng.integers(R))
        if real:
            mag = int(rng.choice([rng.integers(1, factor // 4), rng.integers(factor // 4, 3 * factor),
                                  factor, 2 * factor]))
        else:
            mag = int(rng.integers(1, 4))
        sign = 1 if rng.random() < 0.5 else -1
        p = np.zeros(R, dtype=np.int64)
        p[q] = sign * mag
        flag = int(rng.integers(0, 1 << R)) if initiator else 0
        rows.append(np.concatenate([d, p, [flag]]).astype(np.int64))
        if rng.random() < dup_frac:  # exact cancellation partner
            p2 = -p
            flag2 = int(rng.integers(0, 1 << R)) if initiator else 0
            rows.append(np.concatenate([d, p2, [flag2]]).astype(np.int64))
    sdata = np.array(rows, dtype=np.int64).reshape(len(rows), W + R + 1)
    perm = rng.permutation(len(rows))
    return main, pops, sdata[perm]
