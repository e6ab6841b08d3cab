"""Host-side system set-up: the arrays HANDE holds for a system after
``init_system``, ``init_model_basis_fns``/``init_momentum_symmetry`` (Hubbard
model in momentum space) or ``read_in_integrals`` (molecular FCIDUMP).

These arrays are what crosses the C ABI (``hgpu_system`` in
``include/hande_gpu.h``); both the CUDA engine and the CPU oracle read them.
Spin orbitals are 0-based here: spin orbital ``p`` is HANDE orbital ``p+1``,
bit ``p % 64`` of word ``p // 64``; even ``p`` is alpha (Ms=+1), odd ``p`` beta.
"""

from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

DEPSILON = 1.0e-12  # lib/local/const.F90:90


def insertion_rank(arr: Sequence[float], tol: float) -> list:
    """Stable ranking with tolerance (lib/local/ranking.f90:81-138).

    Returns 0-based indices: rank[k] is the index of the k-th smallest value;
    values within ``tol`` keep their input order."""
    n = len(arr)
    rank = list(range(n))
    for i in range(1, n):
        j = i - 1
        tmp = rank[i]
        while j >= 0:
            if arr[rank[j]] - arr[tmp] < tol:
                break
            rank[j + 1] = rank[j]
            j -= 1
        rank[j + 1] = tmp
    return rank


@dataclass
class System:
    """Arrays of one system (mirror of the fields of ``sys_t`` the engine uses)."""

    kind: str                      # 'hubbard_k' or 'read_in'
    nbasis: int
    nel: int
    nalpha: int
    nbeta: int
    orb_sym: np.ndarray            # int32 [nbasis]
    orb_ms: np.ndarray             # int32 [nbasis]
    sp_eigv: np.ndarray            # float64 [nbasis]
    # hubbard_k
    nkpoints: int = 0
    sym_table: Optional[np.ndarray] = None   # int32 [nk, nk], 0-based
    inv_sym: Optional[np.ndarray] = None     # int32 [nk]
    coulomb_k: float = 0.0
    kpoints: Optional[np.ndarray] = None     # int32 [nk, ndim] (wavevector labels)
    U: float = 0.0
    t: float = 0.0
    nsites: int = 0
    # read_in
    norb: int = 0
    nsym_pg: int = 1
    h1: Optional[np.ndarray] = None          # float64 [norb, norb]
    v2: Optional[np.ndarray] = None          # float64 packed
    ecore: float = 0.0
    nbasis_sym_spin: Optional[np.ndarray] = None     # int32 [2, nsym_pg]
    sym_spin_basis_fns: Optional[np.ndarray] = None  # int32 [nsym_pg, 2, maxn]
    extra: dict = field(default_factory=dict)

    @property
    def nwords(self) -> int:
        return (self.nbasis + 63) // 64

    @property
    def nvirt_alpha(self) -> int:
        return self.nbasis // 2 - self.nalpha

    @property
    def nvirt_beta(self) -> int:
        return self.nbasis // 2 - self.nbeta

    def aufbau_occ(self) -> list:
        """Default reference: the lowest nalpha alpha and nbeta beta spin
        orbitals (src/reference_determinant.f90:124-128)."""
        return [2 * i for i in range(self.nalpha)] + [2 * i + 1 for i in range(self.nbeta)]

    def encode(self, occ: Sequence[int]) -> np.ndarray:
        """encode_det (src/determinants.f90:213): occupied spin orbitals -> words."""
        f = np.zeros(self.nwords, dtype=np.uint64)
        for p in occ:
            f[p // 64] |= np.uint64(1) << np.uint64(p % 64)
        return f

    def decode(self, f: Sequence[int]) -> list:
        """decode_det (src/determinants.f90:243): ascending occupied orbitals."""
        occ = []
        for w in range(self.nwords):
            x = int(f[w]) & 0xFFFFFFFFFFFFFFFF
            for b in range(64):
                if (x >> b) & 1:
                    occ.append(64 * w + b)
        return occ


def tri0(i: int, j: int) -> int:
    """0-based lower-triangular index, i >= j (lib/local/utils.F90:449 tri_ind, shifted)."""
    return i * (i + 1) // 2 + j


def pair_index(p: int, q: int) -> int:
    return tri0(p, q) if p >= q else tri0(q, p)


def v2_index(i: int, a: int, j: int, b: int) -> int:
    """Index of (ia|jb) in the packed 8-fold array (two_body_int_indx,
    src/molecular_integrals.F90:736-845), spatial 0-based."""
    ia = pair_index(i, a)
    jb = pair_index(j, b)
    return tri0(ia, jb) if ia >= jb else tri0(jb, ia)


# ---------------------------------------------------------------------------
# Hubbard model in momentum space
# ---------------------------------------------------------------------------

def hubbard_k(lattice, electrons: int, U: float = 1.0, t: float = 1.0, ms: int = 0,
              twist=None) -> System:
    """Build a Hubbard-model system in a Bloch basis as HANDE does.

    lattice: list of ndim lattice vectors (Lua ``lattice = {{..},{..}}``:
    vector i is column i of sys%lattice%lattice, src/lua_hande_systems.f90:251-262).
    Follows init_system (src/system.f90:458-580), init_model_basis_fns
    (src/basis.f90:258-440), calc_kinetic (src/kpoints.f90:9-53) and
    init_momentum_symmetry (src/momentum_symmetry.f90:17-80)."""
    lat = np.array(lattice, dtype=np.int64)  # lat[i] = i-th vector
    ndim = lat.shape[0]
    L = lat.T.copy()  # L[:, i] = i-th vector, as sys%lattice%lattice(:, i)
    box = np.array([math.sqrt(float(np.dot(L[:, i], L[:, i]))) for i in range(ndim)])
    nsites = int(round(float(np.prod(box))))
    rl = np.zeros((ndim, ndim))
    for i in range(ndim):
        rl[:, i] = L[:, i] / box[i] ** 2
    tw = np.zeros(ndim) if twist is None else np.array(twist, dtype=float)
    # k-point search range (src/basis.f90:293-302)
    nmax = [0, 0, 0]
    for i in range(ndim):
        lim = []
        for j in range(ndim):
            if L[i, j] != 0:
                lim.append(abs(int(np.rint(box[i] ** 2 / (2 * L[i, j])))))
            else:
                lim.append(0)
        nmax[i] = 0
    # forall (i) forall (j, lattice(i,j)/=0) limits(i,j) = ...; nmax(i) = maxval(limits(:,i))
    limits = np.zeros((3, 3), dtype=np.int64)
    for i in range(ndim):
        for j in range(ndim):
            if L[i, j] != 0:
                limits[i, j] = abs(int(np.rint(box[i] ** 2 / (2 * L[i, j]))))
    for i in range(ndim):
        nmax[i] = int(limits[:, i].max())

    def kc_of(k):
        return np.array([sum(k[j] * rl[i, j] for j in range(ndim)) for i in range(ndim)])

    kpts = []
    for k3 in range(-nmax[2], nmax[2] + 1):
        for k2 in range(-nmax[1], nmax[1] + 1):
            for k1 in range(-nmax[0], nmax[0] + 1):
                kp = (k1, k2, k3)[:ndim]
                kc = kc_of(kp)
                if np.all(kc <= 0.5 + DEPSILON) and np.all(kc > -0.5 + 1.0e-5):
                    kpts.append(kp)
    if len(kpts) != nsites:
        raise ValueError("k-point search found %d points for %d sites" % (len(kpts), nsites))
    eig = []
    for kp in kpts:
        kc = np.array([sum((kp[j] + tw[j]) * rl[i, j] for j in range(ndim)) for i in range(ndim)])
        eig.append(-2.0 * float(np.sum(np.cos(2.0 * math.pi * kc))) * t)
    rank = insertion_rank(eig, DEPSILON)
    kpts = np.array([kpts[r] for r in rank], dtype=np.int64).reshape(nsites, ndim)
    eigs = np.array([eig[r] for r in rank])
    nbasis = 2 * nsites

    # momentum symmetry table (src/momentum_symmetry.f90:48-78)
    def is_rlv(k):
        if np.all(k == 0):
            return True
        kc = kc_of(k)
        return bool(np.all(np.abs(kc - np.rint(kc)) < DEPSILON))

    gamma = -1
    for i in range(nsites):
        if np.all(kpts[i] == 0):
            gamma = i
    if gamma < 0:
        raise ValueError("Gamma-point symmetry not found")
    sym_table = np.full((nsites, nsites), -1, dtype=np.int32)
    inv_sym = np.full(nsites, -1, dtype=np.int32)
    for i in range(nsites):
        for j in range(i, nsites):
            ksum = kpts[i] + kpts[j]
            for k in range(nsites):
                if is_rlv(ksum - kpts[k]):
                    sym_table[i, j] = k
                    sym_table[j, i] = k
                    if k == gamma:
                        inv_sym[i] = j
                        inv_sym[j] = i
                    break

    nalpha = (electrons + ms) // 2
    nbeta = electrons - nalpha
    if nalpha + nbeta != electrons or nalpha - nbeta != ms:
        raise ValueError("electrons and ms are inconsistent")
    orb_sym = np.array([p // 2 for p in range(nbasis)], dtype=np.int32)
    orb_ms = np.array([1 if p % 2 == 0 else -1 for p in range(nbasis)], dtype=np.int32)
    sp = np.repeat(eigs, 2)
    return System(kind="hubbard_k", nbasis=nbasis, nel=electrons, nalpha=nalpha, nbeta=nbeta,
                  orb_sym=orb_sym, orb_ms=orb_ms, sp_eigv=sp, nkpoints=nsites,
                  sym_table=sym_table, inv_sym=inv_sym, coulomb_k=U / nsites,
                  kpoints=kpts, U=U, t=t, nsites=nsites)


# ---------------------------------------------------------------------------
# Molecular systems (FCIDUMP)
# ---------------------------------------------------------------------------

_NAMELIST_END = re.compile(r"(&END|/)\s*$", re.IGNORECASE)


def parse_fcidump(path_or_text: str, is_text: bool = False):
    """Read an FCIDUMP: header namelist &FCI NORB NELEC MS2 ORBSYM ISYM UHF
    (src/read_in.F90:80) then lines ``x i a j b`` = (ia|jb)."""
    text = path_or_text if is_text else open(path_or_text).read()
    lines = text.splitlines()
    header = []
    k = 0
    while k < len(lines):
        header.append(lines[k])
        if _NAMELIST_END.search(lines[k].strip()) or lines[k].strip().upper().startswith("&END"):
            k += 1
            break
        k += 1
    htext = " ".join(header)
    htext = re.sub(r"&FCI", " ", htext, flags=re.IGNORECASE)
    htext = re.sub(r"&END", " ", htext, flags=re.IGNORECASE)
    vals = {}
    for m in re.finditer(r"([A-Za-z0-9_]+)\s*=\s*([^=]*?)(?=(?:[A-Za-z0-9_]+\s*=)|$)", htext):
        key = m.group(1).upper()
        v = m.group(2).strip().rstrip(",").strip().rstrip("/").strip()
        vals[key] = v
    norb = int(vals.get("NORB", "0"))
    nelec = int(vals.get("NELEC", "0"))
    ms2 = int(vals.get("MS2", "0"))
    orbsym = [int(x) for x in re.split(r"[,\s]+", vals.get("ORBSYM", "")) if x.strip()]
    if len(orbsym) < norb:
        orbsym += [0] * (norb - len(orbsym))
    uhf = vals.get("UHF", ".FALSE.").upper().strip(".") in ("TRUE", "T")
    ints = []
    for line in lines[k:]:
        parts = line.split()
        if len(parts) < 5:
            continue
        ints.append((float(parts[0].replace("D", "E").replace("d", "e")), int(parts[1]),
                     int(parts[2]), int(parts[3]), int(parts[4])))
    return dict(norb=norb, nelec=nelec, ms2=ms2, orbsym=orbsym[:norb], uhf=uhf, ints=ints)


def _sp_eigv_from_fcidump(norb, nel, ints):
    """get_sp_eigv (src/read_in.F90:1129-1216)."""
    nocc = nel // 2
    sp = [0.0] * (norb + 1)
    found = False
    seen_ijij = set()
    seen_ijji = set()
    for (x, i, a, j, b) in ints:
        if i > 0 and j == 0 and a == 0 and b == 0:
            found = True
            sp[i] = x
        elif not found:
            if i == j and a == b and i == a and i > 0:
                if i <= nocc:
                    sp[i] += x
            elif i == a and j == b and b > 0:
                if (i, j) not in seen_ijij:
                    seen_ijij.add((i, j))
                    seen_ijij.add((j, i))
                    if i <= nocc:
                        sp[j] += 2 * x
                    if j <= nocc:
                        sp[i] += 2 * x
            elif ((i == b and j == a) or (i == j and a == b)) and b > 0:
                if (i, a) not in seen_ijji:
                    seen_ijji.add((i, a))
                    seen_ijji.add((a, i))
                    if i <= nocc:
                        sp[a] -= x
                    if a <= nocc:
                        sp[i] -= x
            elif i == a and j == 0 and b == 0 and i > 0:
                sp[i] += x
    return sp[1:], found


def read_in(int_file: Optional[str] = None, nel: Optional[int] = None, ms: Optional[int] = None,
            text: Optional[str] = None) -> System:
    """Molecular system from an FCIDUMP, as read_in_integrals
    (src/read_in.F90:12-860) builds it for RHF integrals without CAS or Lz:
    orbitals ranked by single-particle eigenvalue (insertion_rank, tolerance
    depsilon), point-group symmetry by XOR of irrep labels
    (src/pg_symmetry.f90), one-body integrals (first occurrence kept),
    two-body integrals (last occurrence kept) and E_core."""
    d = parse_fcidump(text if text is not None else int_file, is_text=text is not None)
    if d["uhf"]:
        raise NotImplementedError("UHF integrals are outside this engine's scope")
    norb = d["norb"]
    nelec = d["nelec"] if nel is None else nel
    ms2 = d["ms2"] if ms is None else ms
    ints = d["ints"]
    sp, _ = _sp_eigv_from_fcidump(norb, nelec, ints)
    rank = insertion_rank(sp, DEPSILON)          # rank[pos] = fcidump orbital (0-based)
    pos_of = [0] * norb
    for pos, r in enumerate(rank):
        pos_of[r] = pos
    orbsym = d["orbsym"]
    spat_sym = [int(orbsym[rank[pos]]) - 1 for pos in range(norb)]
    if min(spat_sym) < 0:
        spat_sym = [0] * norb
    nbasis = 2 * norb
    maxsym_val = max(spat_sym)
    maxsym = 1
    while maxsym < maxsym_val + 1:
        maxsym *= 2
    pg_mask = maxsym - 1
    orb_sym = np.array([spat_sym[p // 2] for p in range(nbasis)], dtype=np.int32)
    orb_ms = np.array([1 if p % 2 == 0 else -1 for p in range(nbasis)], dtype=np.int32)
    sp_eigv = np.array([sp[rank[p // 2]] for p in range(nbasis)])
    nbss = np.zeros((2, maxsym), dtype=np.int32)
    lists = [[[], []] for _ in range(maxsym)]
    for p in range(nbasis):
        ims = (orb_ms[p] + 1) // 2
        nbss[ims, orb_sym[p]] += 1
        lists[orb_sym[p]][ims].append(p)
    maxn = int(nbss.max())
    ssbf = np.full((maxsym, 2, max(maxn, 1)), -1, dtype=np.int32)
    for s in range(maxsym):
        for ims in range(2):
            for k, p in enumerate(lists[s][ims]):
                ssbf[s, ims, k] = p
    h1 = np.zeros((norb, norb))
    npair = norb * (norb + 1) // 2
    v2 = np.zeros(npair * (npair + 1) // 2)
    ecore = 0.0
    seen_h = set()
    for (x, i, a, j, b) in ints:
        ii = pos_of[i - 1] if i > 0 else -1
        aa = pos_of[a - 1] if a > 0 else -1
        jj = pos_of[j - 1] if j > 0 else -1
        bb = pos_of[b - 1] if b > 0 else -1
        if i == 0 and j == 0 and a == 0 and b == 0:
            ecore += x
        elif i > 0 and j == 0 and a == 0 and b == 0:
            continue  # single-particle eigenvalue
        elif j == 0 and b == 0:
            if ii >= 0 and aa >= 0:
                key = (max(ii, aa), min(ii, aa))
                if key in seen_h:
                    continue
                if (spat_sym[ii] ^ spat_sym[aa]) & pg_mask:
                    continue  # forbidden by symmetry: not stored (store_one_body_int)
                seen_h.add(key)
                h1[ii, aa] = x
                h1[aa, ii] = x
        else:
            if min(ii, jj, aa, bb) < 0:
                continue
            if (spat_sym[ii] ^ spat_sym[jj] ^ spat_sym[aa] ^ spat_sym[bb]) & pg_mask:
                continue
            v2[v2_index(ii, aa, jj, bb)] = x
    nalpha = (nelec + ms2) // 2
    nbeta = nelec - nalpha
    s = System(kind="read_in", nbasis=nbasis, nel=nelec, nalpha=nalpha, nbeta=nbeta,
               orb_sym=orb_sym, orb_ms=orb_ms, sp_eigv=sp_eigv, norb=norb, nsym_pg=maxsym,
               h1=h1, v2=v2, ecore=ecore, nbasis_sym_spin=nbss, sym_spin_basis_fns=ssbf)
    s.extra["fcidump_rank"] = rank
    return s


def molecular_from_arrays(h1: np.ndarray, v_chem_packed: np.ndarray, nel: int, ms: int = 0,
                          ecore: float = 0.0, orbsym: Optional[Sequence[int]] = None) -> System:
    """Molecular system from integrals already in orbital-energy order (no
    re-ranking): h1[M, M] and the packed (ia|jb) array in v2_index order."""
    norb = h1.shape[0]
    spat_sym = [0] * norb if orbsym is None else [int(x) - 1 for x in orbsym]
    nbasis = 2 * norb
    maxsym = 1
    while maxsym < max(spat_sym) + 1:
        maxsym *= 2
    orb_sym = np.array([spat_sym[p // 2] for p in range(nbasis)], dtype=np.int32)
    orb_ms = np.array([1 if p % 2 == 0 else -1 for p in range(nbasis)], dtype=np.int32)
    nbss = np.zeros((2, maxsym), dtype=np.int32)
    lists = [[[], []] for _ in range(maxsym)]
    for p in range(nbasis):
        ims = (orb_ms[p] + 1) // 2
        nbss[ims, orb_sym[p]] += 1
        lists[orb_sym[p]][ims].append(p)
    maxn = int(nbss.max())
    ssbf = np.full((maxsym, 2, maxn), -1, dtype=np.int32)
    for s_ in range(maxsym):
        for ims in range(2):
            for k, p in enumerate(lists[s_][ims]):
                ssbf[s_, ims, k] = p
    nalpha = (nel + ms) // 2
    nbeta = nel - nalpha
    return System(kind="read_in", nbasis=nbasis, nel=nel, nalpha=nalpha, nbeta=nbeta,
                  orb_sym=orb_sym, orb_ms=orb_ms,
                  sp_eigv=np.repeat(np.diag(h1).copy(), 2), norb=norb, nsym_pg=maxsym,
                  h1=np.ascontiguousarray(h1, dtype=np.float64),
                  v2=np.ascontiguousarray(v_chem_packed, dtype=np.float64), ecore=ecore,
                  nbasis_sym_spin=nbss, sym_spin_basis_fns=ssbf)


def synthetic_integrals(norb: int, seed: int, nchol: int = 80):
    """The synthetic molecular Hamiltonian of the benchmark configurations:
    h symmetric with h_pp = -2 + 0.15 p (p = 1..M) and off-diagonal N(0, 0.05^2);
    (pq|rs) = sum_{L<nchol} B^L_pq B^L_rs with each B^L symmetric Gaussian,
    std 0.3 exp(-|p-q|/8), which is 8-fold symmetric and positive semidefinite.
    Returns (h1, packed v2) in v2_index order."""
    rng = np.random.default_rng(seed)
    M = norb
    h = np.zeros((M, M))
    for p in range(M):
        h[p, p] = -2.0 + 0.15 * (p + 1)
    off = rng.normal(0.0, 0.05, size=(M, M))
    iu = np.triu_indices(M, 1)
    h[iu] = off[iu]
    h[(iu[1], iu[0])] = off[iu]
    pq = np.arange(M)
    std = 0.3 * np.exp(-np.abs(pq[:, None] - pq[None, :]) / 8.0)
    npair = M * (M + 1) // 2
    ip, iq = np.tril_indices(M)          # pair k = (p >= q), k = p(p+1)/2 + q
    Bp = np.zeros((nchol, npair))
    for L in range(nchol):
        g = rng.normal(0.0, 1.0, size=(M, M)) * std
        B = np.tril(g) + np.tril(g, -1).T
        Bp[L] = B[ip, iq]
    V = Bp.T @ Bp                         # (pq|rs) over pairs, npair x npair
    li, lj = np.tril_indices(npair)
    v2 = V[li, lj].copy()                 # tri0(ia, jb) with ia >= jb
    return h, v2


def write_fcidump(path: str, h1: np.ndarray, v2: np.ndarray, nel: int, ms2: int = 0,
                  ecore: float = 0.0, orbsym: Optional[Sequence[int]] = None,
                  sp_eigv: Optional[Sequence[float]] = None) -> None:
    """Write integrals as an FCIDUMP (chemists' (ia|jb), 8-fold unique lines,
    one-body lines, single-particle eigenvalue lines and E_core), the format
    read_in_integrals reads."""
    M = h1.shape[0]
    sym = [1] * M if orbsym is None else list(orbsym)
    with open(path, "w") as fh:
        fh.write(" &FCI NORB=%d,NELEC=%d,MS2=%d,\n" % (M, nel, ms2))
        fh.write("  ORBSYM=%s,\n" % ",".join(str(s) for s in sym))
        fh.write("  ISYM=1,\n &END\n")
        for i in range(M):
            for a in range(i + 1):
                ia = tri0(i, a)
                for j in range(M):
                    for b in range(j + 1):
                        jb = tri0(j, b)
                        if jb > ia:
                            continue
                        x = v2[tri0(ia, jb)]
                        if x != 0.0:
                            fh.write("%.17e %d %d %d %d\n" % (x, i + 1, a + 1, j + 1, b + 1))
        for i in range(M):
            for a in range(i + 1):
                if h1[i, a] != 0.0:
                    fh.write("%.17e %d %d 0 0\n" % (h1[i, a], i + 1, a + 1))
        if sp_eigv is not None:
            for i in range(M):
                fh.write("%.17e %d 0 0 0\n" % (sp_eigv[i], i + 1))
        fh.write("%.17e 0 0 0 0\n" % ecore)


def synthetic_molecule(norb: int, nel: int, seed: int = 2024, ms: int = 0, nchol: int = 80) -> System:
    """Synthetic molecule of the benchmark configurations (C1 symmetry),
    orbitals already in order of increasing h_pp."""
    h, v2 = synthetic_integrals(norb, seed, nchol)
    s = molecular_from_arrays(h, v2, nel, ms)
    s.extra["seed"] = seed
    return s
