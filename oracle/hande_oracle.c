/*
 * hande_oracle.c -- CPU restatement of HANDE's FCIQMC cycle (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file, as the checker.  It restates the reference algorithm function by
 * function; each function names the reference file:line it follows.  The
 * arithmetic follows the reference's operation order so that the values it
 * produces are the ones the reference formulae give in IEEE double precision
 * (build with -ffp-contract=off).
 *
 * Orbitals are 0-based (HANDE orbital k is p = k-1); the parity of every
 * difference and the outcome of every comparison is unchanged by the shift.
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers of the hash-partitioned driver */
#include "hande_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXW HGPU_MAX_WORDS
#define MAXB (64 * MAXW)
#define MAXEL 64
#define DEPSILON 1.0e-12 /* lib/local/const.F90:90 */

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the stream layout.   */
/* ------------------------------------------------------------------------- */

enum { P_NATTEMPT = 1, P_SPAWN = 2, P_DEATH = 3, P_ROUND_MAIN = 4, P_ROUND_SPAWN = 5, P_DETERM = 6 };

static void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* A stream of uniform doubles in [0,1): counter = (idx, sub, iteration,
 * purpose<<28 | space<<26 | block), key = (seed lo, seed hi); each block gives
 * two doubles (53 bits each). */
typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t block;
    double buf[2];
    int have;
} rstream;

static void rs_init(rstream *s, uint64_t seed, int purpose, int space, uint64_t idx, uint64_t sub,
                    uint64_t iter) {
    s->key[0] = (uint32_t)seed;
    s->key[1] = (uint32_t)(seed >> 32);
    s->ctr[0] = (uint32_t)idx;
    s->ctr[1] = (uint32_t)sub;
    s->ctr[2] = (uint32_t)iter;
    s->ctr[3] = ((uint32_t)purpose << 28) | ((uint32_t)space << 26);
    s->block = 0;
    s->have = 0;
}

static double u53(uint32_t hi, uint32_t lo) {
    uint64_t x = ((uint64_t)hi << 32) | lo;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* get_rand_close_open (lib/dSFMT_F03_interface/dSFMT_interface.F90:387). */
static double rs_next(rstream *s) {
    if (s->have == 0) {
        uint32_t c[4] = {s->ctr[0], s->ctr[1], s->ctr[2], s->ctr[3] | s->block};
        uint32_t o[4];
        philox4x32_10(c, s->key, o);
        s->block++;
        s->buf[0] = u53(o[0], o[1]);
        s->buf[1] = u53(o[2], o[3]);
        s->have = 2;
    }
    double r = s->buf[2 - s->have];
    s->have--;
    return r;
}

double oracle_uniform(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, int which) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t c[4] = {c0, c1, c2, c3}, o[4];
    philox4x32_10(c, key, o);
    return which ? u53(o[2], o[3]) : u53(o[0], o[1]);
}

/* ------------------------------------------------------------------------- */
/* Context                                                                    */
/* ------------------------------------------------------------------------- */

struct oracle_ctx {
    hgpu_config cfg;
    int kind, nbasis, nel, nalpha, nbeta, nw, nvirt_alpha, nvirt_beta, nvirt;
    int32_t *orb_sym, *orb_ms;
    double *sp_eigv;
    int nk;
    int32_t *sym_table, *inv_sym;
    double coulomb_k;
    int norb, nsym;
    double *h1, *v2;
    int64_t nv2;
    double ecore;
    int32_t *nbss, *ssbf;
    int maxss;
    uint64_t mask[MAXB][MAXW]; /* excit_mask (src/excitations.F90:25-70) */
    int64_t real_factor, cutoff;
    double pattempt_single, pattempt_double;
    /* renorm_spin / no_renorm_spin: pattempt_parallel and pgen_ij of the three
     * spin classes (alpha-alpha, beta-beta, opposite), choose_ij_spin_mol */
    int spin_ij;
    double pattempt_parallel, pgen_ij_aa, pgen_ij_bb, pgen_ij_ab;
    int R;
    uint64_t f0[MAXW];
    double H00;
    /* exact diagonal: terms on the 2^-fx_s grid (see fx_energy) */
    int fx_s;
    int64_t fx_cst, fx_E0;
    int64_t *fx_h1, *fx_J, *fx_JK, *fx_eps;
    /* main list */
    int64_t n, cap;
    uint64_t *dets;
    int64_t *pops;
    double *kii;
    /* qmc state */
    double shift[2];
    int vary_shift[2];
    double nparticles_old[2];
    int64_t iter;
    /* report accumulators */
    double acc_proj[2], acc_d0[2], acc_rspawn;
    int64_t last_nspawn_events, rep_attempts, rep_spawned, total_attempts;
    int rep_cycles;
    int error_flags;
    /* bloom_stats_t (src/bloom_handler.F90:26-71): blooms of the report, their
     * summed |amount| (encoded), the largest |amount| of the calculation */
    int64_t bloom_n, bloom_tot, bloom_max;
    /* spawned list: W det words, R pops, flag, generation order */
    int64_t sn, scap;
    uint64_t *sdets;
    int64_t *spops, *sflag, *sord, *suid;
    /* heat-bath tables (excit_gen_heat_bath_t, src/excit_gens.f90:143-153), 0-based
     * and first Fortran index fastest: ij_w[i*nb + j] = ij_weights(j,i),
     * ija_w[(i*nb + j)*nb + a] = hb_ija%weights(a,j,i), ija_tot[i*nb + j] =
     * hb_ija%weights_tot(j,i), ijab_*[((i*nb + j)*nb + a)*nb + b] and
     * ijab_tot[(i*nb + j)*nb + a] likewise. */
    /* replica 2-RDM (src/replica_rdm.F90): rdm[row * npairs + col], rows and
     * columns the distinct spin-orbital pairs p < q in tri_ind_distinct order;
     * the RDM spawns of a cycle hold (parent, child) words and R amplitudes */
    int rdm_enabled, rdm_on, reports_done;
    int64_t npairs, rsn;
    double *rdm;
    uint64_t *rsdets;
    int64_t *rspops;
    double rdm_energy, rdm_trace;
    /* heat_bath_power_pitzer_ref (excit_gen_power_pitzer_t of
     * init_excit_mol_power_pitzer_orderN): the reference's occupied list and
     * six weight/alias tables, PPN_IS (i for singles, [nel]), PPN_ID (i for
     * doubles, [nel]), PPN_IJD (j given the orbital i, [nbasis][nel]), PPN_IAS
     * (a of a single, [nbasis][maxss]), PPN_IAD (a of a double over all
     * orbitals of i's spin, [nbasis][nbasis/2]), PPN_JBD (b per irrep,
     * [nbasis*nsym][maxss]) */
    /* semi-stochastic projection (semi_stoch_t, src/semi_stoch.F90): the
     * iteration at whose start the space is built, the deterministic
     * determinants in main-list order, the Hamiltonian by column j (rows i
     * ascending, H(D_i, D_j), diagonal K_jj), the populations copied at the
     * start of the cycle, the projected amplitudes and the main-list
     * positions of the deterministic states this cycle */
    int64_t ss_iter, nd;
    int ss_on;
    uint64_t *ddets;
    int64_t *dcol_ptr, *dcol_i, *dind;
    double *dcol_h, *dvec, *dy;
    int ppn_occ[MAXEL];
    double *ppn_w[6], *ppn_U[6], *ppn_tot[6];
    int32_t *ppn_K[6];
    int ppn_stride[6];
    int hb_on;
    double *hb_i_w, *hb_ij_w, *hb_ija_w, *hb_ija_tot, *hb_ija_U, *hb_ijab_w, *hb_ijab_tot, *hb_ijab_U;
    int32_t *hb_ija_K, *hb_ijab_K;
};

/* determinant helpers ------------------------------------------------------ */

static inline int tbit(const uint64_t *f, int p) { return (int)((f[p >> 6] >> (p & 63)) & 1u); }
static inline void sbit(uint64_t *f, int p) { f[p >> 6] |= (uint64_t)1 << (p & 63); }
static inline void cbit(uint64_t *f, int p) { f[p >> 6] &= ~((uint64_t)1 << (p & 63)); }

static int popc64(uint64_t x) {
    int n = 0;
    while (x) { x &= x - 1; n++; }
    return n;
}

/* bit_str_cmp (src/bit_utils.F90:452-478): 1 if a<b, -1 if a>b, 0 if equal;
 * last word most significant, unsigned. */
static int det_cmp(const uint64_t *a, const uint64_t *b, int nw) {
    for (int i = nw - 1; i >= 0; i--) {
        if (a[i] < b[i]) return 1;
        if (a[i] > b[i]) return -1;
    }
    return 0;
}

/* decode_det (src/determinants.f90:243): ascending occupied spin orbitals. */
static int decode(const oracle_ctx *c, const uint64_t *f, int *occ) {
    int n = 0;
    for (int p = 0; p < c->nbasis; p++)
        if (tbit(f, p)) occ[n++] = p;
    return n;
}

/* ------------------------------------------------------------------------- */
/* Excitations (src/excitations.F90)                                          */
/* ------------------------------------------------------------------------- */

typedef struct {
    int nexcit;
    int from[2], to[2];
    int perm;
} excit_t;

/* get_excitation (src/excitations.F90:75-200).  The reference skips the
 * electron count of identical words when iexcit1-iexcit2 is even; that skip
 * changes perm by an even number, so counting every word gives the same parity. */
static excit_t get_excitation(const oracle_ctx *c, const uint64_t *f1, const uint64_t *f2) {
    excit_t e = {0, {-1, -1}, {-1, -1}, 0};
    int diff = 0;
    for (int w = 0; w < c->nw; w++) diff += popc64(f1[w] ^ f2[w]);
    if (diff == 0) return e;
    e.nexcit = diff / 2;
    if (e.nexcit > 2) return e;
    int shift = c->nel - e.nexcit;
    int iexcit1 = 0, iexcit2 = 0, iel1 = 0, iel2 = 0, perm = 0;
    for (int p = 0; p < c->nbasis; p++) {
        int t1 = tbit(f1, p), t2 = tbit(f2, p);
        if (t2) iel2++;
        if (t1) {
            iel1++;
            if (!t2) {
                iexcit1++;
                e.from[iexcit1 - 1] = p;
                perm += shift - iel1 + iexcit1;
            }
        } else if (t2) {
            iexcit2++;
            e.to[iexcit2 - 1] = p;
            perm += shift - iel2 + iexcit2;
        }
    }
    e.perm = (((perm % 2) + 2) % 2) == 1;
    return e;
}

/* find_excitation_permutation1 (src/excitations.F90:247-280). */
static int perm1(const oracle_ctx *c, const uint64_t *f, int i, int a) {
    int perm = 0;
    for (int w = 0; w < c->nw; w++) perm += popc64(f[w] & (c->mask[i][w] ^ c->mask[a][w]));
    if (i > a) perm -= 1;
    return (((perm % 2) + 2) % 2) == 1;
}

/* find_excitation_permutation2 (src/excitations.F90:282-330). */
static int perm2(const oracle_ctx *c, const uint64_t *f, int i, int j, int a, int b) {
    int perm = 0;
    for (int w = 0; w < c->nw; w++) {
        uint64_t ia = c->mask[i][w] ^ c->mask[a][w];
        uint64_t jb = c->mask[j][w] ^ c->mask[b][w];
        perm += popc64((f[w] & ia) ^ (f[w] & jb));
    }
    if (i > a) perm += 1;
    if (i > b) perm += 1;
    if (j > b || j < a) perm += 1;
    return (perm % 2) == 1;
}

/* create_excited_det (src/excitations.F90:365-406). */
static void excited_det(const oracle_ctx *c, const uint64_t *f, const excit_t *e, uint64_t *out) {
    for (int w = 0; w < c->nw; w++) out[w] = f[w];
    for (int k = 0; k < e->nexcit; k++) {
        cbit(out, e->from[k]);
        sbit(out, e->to[k]);
    }
}

/* ------------------------------------------------------------------------- */
/* Hubbard model in momentum space                                            */
/* ------------------------------------------------------------------------- */

static inline int kidx(int p) { return p >> 1; }

/* momentum_conserved (src/hubbard_k.f90:57-84). */
static int momentum_conserved(const oracle_ctx *c, int i, int j, int k, int l) {
    int dk = c->sym_table[kidx(i) * c->nk + kidx(j)];
    dk = c->sym_table[dk * c->nk + c->inv_sym[kidx(k)]];
    return dk == kidx(l);
}

/* get_two_e_int_hub_k (src/hubbard_k.f90:11-55). */
static double two_e_int_hub_k(const oracle_ctx *c, int p1, int p2, int p3, int p4) {
    int s12 = c->orb_ms[p1] == c->orb_ms[p2];
    int s34 = c->orb_ms[p3] == c->orb_ms[p4];
    if (!s12 && (s12 == s34) && momentum_conserved(c, p1, p2, p3, p4)) {
        if (c->orb_ms[p1] == c->orb_ms[p3]) return c->coulomb_k;
        return -c->coulomb_k;
    }
    return 0.0;
}

/* Exact diagonal energies.  <D|H|D> (slater_condon0_hub_k,
 * src/hamiltonian_hub_k.f90:91-132; slater_condon0_mol,
 * src/hamiltonian_molecular.f90:73-139) is evaluated as the exact sum of the
 * same terms, each rounded once to a multiple of 2^-s (ties to even) and
 * accumulated in 64-bit integers, then rounded once to double.  s is the largest
 * scale (<= 60) with 2 B 2^s < 2^62, B = sum over every possible term of
 * ceil(|term|).  HANDE sums the terms left to right in FP64; the two differ by a
 * few ulps. */
static int64_t fx_of(const oracle_ctx *c, double x) {
    double y = ldexp(x, c->fx_s); /* exact */
    return (int64_t)rint(y);      /* nearest integer, ties to even (default rounding mode) */
}

static double fx_val(const oracle_ctx *c, int64_t v) { return ldexp((double)v, -c->fx_s); /* one rounding */ }

static int64_t ceil_abs(double x) { return (int64_t)ceil(fabs(x)); }

static int scale_for_bound(int64_t B) {
    int bits = 0;
    while (bits < 63 && (B >> bits) != 0) bits++;
    int s = 61 - bits;
    return s > 60 ? 60 : (s < 0 ? 0 : s);
}

static int64_t fx_energy(const oracle_ctx *c, const uint64_t *f) {
    int occ[MAXB];
    int n = decode(c, f, occ);
    int64_t e = c->fx_cst;
    if (c->kind == HGPU_SYS_HUB_K) {
        for (int i = 0; i < n; i++) e += c->fx_eps[occ[i]];
        return e;
    }
    for (int a = 0; a < n; a++) {
        int i = occ[a];
        e += c->fx_h1[i >> 1];
        for (int b = a + 1; b < n; b++) {
            int j = occ[b];
            int k = (i >> 1) * c->norb + (j >> 1);
            e += (c->orb_ms[i] == c->orb_ms[j]) ? c->fx_JK[k] : c->fx_J[k];
        }
    }
    return e;
}

/* slater_condon2_hub_k_excit (src/hamiltonian_hub_k.f90:163-234). */
static double sc2_hub_k_excit(const oracle_ctx *c, const uint64_t *f, excit_t *e) {
    int t;
    if (e->from[0] > e->from[1]) { t = e->from[0]; e->from[0] = e->from[1]; e->from[1] = t; }
    if (e->to[0] > e->to[1]) { t = e->to[0]; e->to[0] = e->to[1]; e->to[1] = t; }
    double h = c->coulomb_k;
    e->perm = perm2(c, f, e->from[0], e->from[1], e->to[0], e->to[1]);
    if (e->perm) h = -h;
    if (((e->from[0] - e->to[0]) % 2) != 0) h = -h;
    return h;
}

typedef struct {
    int occ[MAXEL], occ_a[MAXEL], occ_b[MAXEL], unocc_a[MAXB];
    int nocc, na, nb, nua;
    int symunocc[2 * 64]; /* [ims*nsym + sym] */
} det_info;

/* decode_det_spinocc_spinunocc (src/determinant_decoders.f90:261-370). */
static void decode_hub_k(const oracle_ctx *c, const uint64_t *f, det_info *d) {
    d->nocc = d->na = d->nb = d->nua = 0;
    for (int p = 0; p < c->nbasis; p++) {
        if (tbit(f, p)) {
            d->occ[d->nocc++] = p;
            if ((p & 1) == 0) d->occ_a[d->na++] = p; else d->occ_b[d->nb++] = p;
        } else if ((p & 1) == 0) {
            d->unocc_a[d->nua++] = p;
        }
    }
}

/* choose_ij_hub_k (src/excit_gen_hub_k.f90:469-532). */
static void choose_ij_hub_k(const oracle_ctx *c, rstream *rs, const det_info *d, int *i, int *j, int *ij_sym) {
    double r = rs_next(rs);
    int ind = (int)(r * (double)c->nalpha * (double)c->nbeta) + 1;
    int ii = (int)(((double)ind - 1.0) / (double)c->nbeta) + 1;
    int jj = ind - (ii - 1) * c->nbeta;
    *i = d->occ_a[ii - 1];
    *j = d->occ_b[jj - 1];
    *ij_sym = c->sym_table[kidx(*i) * c->nk + kidx(*j)];
}

/* beta partner b of alpha orbital a for total momentum ij_sym (find_ab_hub_k). */
static inline int hub_k_partner(const oracle_ctx *c, int ij_sym, int a) {
    return 2 * c->sym_table[ij_sym * c->nk + c->inv_sym[kidx(a)]] + 1;
}

/* calc_pgen_hub_k (src/excit_gen_hub_k.f90:651-770). */
static double calc_pgen_hub_k(const oracle_ctx *c, int ab_sym, const uint64_t *f, const det_info *d) {
    int forbidden = 0;
    for (int k = 0; k < c->nvirt_alpha; k++) {
        int b = hub_k_partner(c, ab_sym, d->unocc_a[k]);
        if (tbit(f, b)) forbidden++;
    }
    return 1.0 / (double)(c->nalpha * c->nbeta * (c->nvirt_alpha - forbidden));
}

/* find_ab_hub_k (src/excit_gen_hub_k.f90:579-649). */
static int find_ab_hub_k(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int ij_sym,
                         int *a, int *b) {
    int r = (int)(rs_next(rs) * (double)c->nvirt_alpha) + 1;
    *a = d->unocc_a[r - 1];
    *b = hub_k_partner(c, ij_sym, *a);
    return !tbit(f, *b);
}

/* ------------------------------------------------------------------------- */
/* Molecular systems                                                          */
/* ------------------------------------------------------------------------- */

static inline int64_t tri0(int64_t i, int64_t j) { return i * (i + 1) / 2 + j; }

/* two_body_int_indx (src/molecular_integrals.F90:736-845), RHF. */
static inline double v2_get(const oracle_ctx *c, int i, int j, int a, int b) {
    int si = i >> 1, sj = j >> 1, sa = a >> 1, sb = b >> 1;
    int64_t ia = si >= sa ? tri0(si, sa) : tri0(sa, si);
    int64_t jb = sj >= sb ? tri0(sj, sb) : tri0(sb, sj);
    int64_t idx = ia >= jb ? tri0(ia, jb) : tri0(jb, ia);
    return c->v2[idx];
}

/* get_one_body_int_mol_nonzero (src/molecular_integrals.F90:685-734). */
static inline double h1_get(const oracle_ctx *c, int i, int j) { return c->h1[(i >> 1) * c->norb + (j >> 1)]; }

static inline int ims_of(const oracle_ctx *c, int p) { return (c->orb_ms[p] + 1) / 2; } /* 0 beta, 1 alpha */

/* slater_condon1_mol_excit (src/hamiltonian_molecular.f90:199-259). */
static double sc1_mol_excit(const oracle_ctx *c, const int *occ, int i, int a, int perm) {
    double h = h1_get(c, i, a);
    for (int iel = 0; iel < c->nel; iel++) {
        int k = occ[iel];
        if (k != i) {
            h = h + v2_get(c, i, k, a, k);
            if (c->orb_ms[k] == c->orb_ms[i]) h = h - v2_get(c, i, k, k, a);
        }
    }
    if (perm) h = -h;
    return h;
}

/* slater_condon2_mol_excit (src/hamiltonian_molecular.f90:300-346). */
static double sc2_mol_excit(const oracle_ctx *c, int i, int j, int a, int b, int perm) {
    double h = 0.0;
    if (c->orb_ms[i] == c->orb_ms[a]) h = v2_get(c, i, j, a, b);
    if (c->orb_ms[i] == c->orb_ms[b]) h = h - v2_get(c, i, j, b, a);
    if (perm) h = -h;
    return h;
}

/* decode_det_occ_symunocc (src/determinant_decoders.f90:166-180). */
static void decode_mol(const oracle_ctx *c, const uint64_t *f, det_info *d) {
    d->nocc = decode(c, f, d->occ);
    for (int k = 0; k < 2 * c->nsym; k++) d->symunocc[k] = c->nbss[k];
    for (int i = 0; i < d->nocc; i++) {
        int p = d->occ[i];
        d->symunocc[ims_of(c, p) * c->nsym + c->orb_sym[p]]--;
    }
}

#define SYMUNOCC(d, ims, s) ((d)->symunocc[(ims) * c->nsym + (s)])
#define NBSS(ims, s) (c->nbss[(ims) * c->nsym + (s)])
#define SSBF(ind, ims, s) (c->ssbf[((s) * 2 + (ims)) * c->maxss + (ind)])

/* cross_product_pg_sym / pg_sym_conj (src/pg_symmetry.f90) without Lz. */
static inline int cross(const oracle_ctx *c, int a, int b) { return (a ^ b) & (c->nsym - 1); }

/* find_single_double_prob, read_in branch (src/qmc_common.F90:152-260): the
 * shares of the symmetry- and spin-allowed single and double excitations of
 * the reference determinant, each divided by their sum. */
static void single_double_prob(const oracle_ctx *c, double *psingle, double *pdouble) {
    const int nsym = c->nsym;
    int *virt = (int *)calloc((size_t)2 * nsym, sizeof(int));
    int occ[MAXEL], n = 0;
    for (int p = 0; p < c->nbasis; p++)
        if (tbit(c->f0, p)) occ[n++] = p;
    for (int ims = 0; ims < 2; ims++)
        for (int s = 0; s < nsym; s++) virt[ims * nsym + s] = NBSS(ims, s);
    for (int i = 0; i < n; i++) virt[ims_of(c, occ[i]) * nsym + c->orb_sym[occ[i]]]--;
    int64_t nsingles = 0, ndoubles = 0;
    for (int i = 0; i < n; i++) nsingles += virt[ims_of(c, occ[i]) * nsym + c->orb_sym[occ[i]]];
    for (int i = 0; i < n; i++) {
        const int m1 = ims_of(c, occ[i]);
        for (int j = i + 1; j < n; j++) {
            const int m2 = ims_of(c, occ[j]);
            for (int sa = 0; sa < nsym; sa++) {
                const int sb = cross(c, sa, cross(c, c->orb_sym[occ[i]], c->orb_sym[occ[j]]));
                const int64_t va1 = virt[m1 * nsym + sa], vb2 = virt[m2 * nsym + sb];
                if (sa == sb) {
                    if (m1 == m2) ndoubles += (va1 * (vb2 - 1)) / 2;
                    else ndoubles += va1 * vb2;
                } else if (sa < sb) {
                    ndoubles += va1 * vb2;
                    if (m1 != m2) ndoubles += (int64_t)virt[m2 * nsym + sa] * virt[m1 * nsym + sb];
                }
            }
        }
    }
    free(virt);
    *psingle = (double)nsingles / (double)(nsingles + ndoubles);
    *pdouble = (double)ndoubles / (double)(nsingles + ndoubles);
}

/* choose_ij_mol (src/excit_gen_mol.f90:620-660). */
static void choose_ij_mol(const oracle_ctx *c, rstream *rs, const det_info *d, int *i, int *j, int *ij_sym,
                          int *ij_spin, double *pgen_ij) {
    double x = rs_next(rs) * (double)c->nel * (double)(c->nel - 1) / 2.0;
    int ind = (int)x + 1;
    int j_ind = (int)(1.50 + sqrt((double)(2 * ind) - 1.750));
    int i_ind = ind - ((j_ind - 1) * (j_ind - 2)) / 2;
    *i = d->occ[i_ind - 1];
    *j = d->occ[j_ind - 1];
    *ij_sym = cross(c, c->orb_sym[*i], c->orb_sym[*j]);
    *ij_spin = c->orb_ms[*i] + c->orb_ms[*j];
    *pgen_ij = 2.0 / (double)(c->nel * (c->nel - 1));
}

/* choose_ij_spin_mol (src/excit_gen_mol.f90:684-783): first parallel or
 * opposite spins, then the pair; returns 0 when the spin class has too few
 * electrons (allowed_excitation = .false.). */
static int choose_ij_spin_mol(const oracle_ctx *c, rstream *rs, const det_info *d, int *i, int *j, int *ij_sym,
                              int *ij_spin, double *pgen_ij) {
    int occa[128], occb[128], na = 0, nb = 0;
    for (int k = 0; k < d->nocc; k++) {
        if (c->orb_ms[d->occ[k]] > 0) occa[na++] = d->occ[k];
        else occb[nb++] = d->occ[k];
    }
    if (rs_next(rs) < c->pattempt_parallel) {
        int alpha = rs_next(rs) < ((double)c->nalpha / (double)(c->nalpha + c->nbeta));
        int n = alpha ? c->nalpha : c->nbeta;
        const int *occ = alpha ? occa : occb;
        if (n < 2) return 0;
        int ind = (int)(rs_next(rs) * (double)(n * (n - 1)) / 2.0) + 1;
        int j_ind = (int)(1.50 + sqrt((double)(2 * ind) - 1.750));
        int i_ind = ind - ((j_ind - 1) * (j_ind - 2)) / 2;
        *i = occ[i_ind - 1];
        *j = occ[j_ind - 1];
        *pgen_ij = alpha ? c->pgen_ij_aa : c->pgen_ij_bb;
    } else {
        if (c->nbeta < 1 || c->nalpha < 1) return 0;
        int i_ind = (int)(rs_next(rs) * (double)c->nalpha) + 1;
        int j_ind = (int)(rs_next(rs) * (double)c->nbeta) + 1;
        *i = occa[i_ind - 1];
        *j = occb[j_ind - 1];
        if (*j < *i) {
            int t = *i;
            *i = *j;
            *j = t;
        }
        *pgen_ij = c->pgen_ij_ab;
    }
    *ij_sym = cross(c, c->orb_sym[*i], c->orb_sym[*j]);
    *ij_spin = c->orb_ms[*i] + c->orb_ms[*j];
    return 1;
}

/* find_parallel_spin_prob_mol (src/qmc_common.F90:265-378): the share of
 * sum |<ij||ab>| over allowed (i, j, a, b) carried by parallel-spin i, j.  The
 * sums run over j, a, b for each i and the per-i sums are added in i order
 * (the reference's order within one process' range of i). */
static double find_parallel_spin_prob_mol(const oracle_ctx *c) {
    double par = 0.0, orth = 0.0;
    for (int i = 0; i < c->nbasis; i++) {
        double pi = 0.0, oi = 0.0;
        for (int j = 0; j < c->nbasis; j++) {
            if (i == j) continue;
            int it = j < i ? j : i, jt = j < i ? i : j;
            int ij_sym = cross(c, c->orb_sym[it], c->orb_sym[jt]);
            for (int a = 0; a < c->nbasis; a++) {
                if (a == i || a == j) continue;
                int isymb = cross(c, ij_sym, c->orb_sym[a]);
                for (int b = 0; b < c->nbasis; b++) {
                    int spin_ok = (c->orb_ms[it] == c->orb_ms[a] && c->orb_ms[jt] == c->orb_ms[b]) ||
                                  (c->orb_ms[it] == c->orb_ms[b] && c->orb_ms[jt] == c->orb_ms[a]);
                    if (!spin_ok || c->orb_sym[b] != isymb || b == a || b == i || b == j) continue;
                    int at = b < a ? b : a, bt = b < a ? a : b;
                    double h = fabs(sc2_mol_excit(c, it, jt, at, bt, 0));
                    if (c->orb_ms[it] == c->orb_ms[jt]) pi = pi + h;
                    else oi = oi + h;
                }
            }
        }
        par = par + pi;
        orth = orth + oi;
    }
    return par / (par + orth);
}

/* spin-dependent (fac, shift, na) of choose_ab_mol / find_ab_mol, 0-based:
 * spin -2 -> beta orbitals 2k+1, spin 2 -> alpha 2k, spin 0 -> any. */
static inline int pick_a(const oracle_ctx *c, int spin, double r) {
    if (spin == 0) return (int)(r * (double)c->nbasis);
    int k = (int)(r * (double)(c->nbasis / 2));
    return spin == -2 ? 2 * k + 1 : 2 * k;
}

/* choose_ab_mol (src/excit_gen_mol.f90:802-948). */
static int choose_ab_mol(const oracle_ctx *c, rstream *rs, const uint64_t *f, int sym, int spin,
                         const det_info *d, int *a_out, int *b_out) {
    int allowed = 0;
    int ia = spin == -2 ? 0 : 1; /* ims of the spin-parallel case */
    for (int isyma = 0; isyma < c->nsym; isyma++) {
        int isymb = cross(c, isyma, sym);
        if (spin == 0) {
            if ((SYMUNOCC(d, 0, isyma) > 0 && SYMUNOCC(d, 1, isymb) > 0) ||
                (SYMUNOCC(d, 1, isyma) > 0 && SYMUNOCC(d, 0, isymb) > 0)) { allowed = 1; break; }
        } else {
            if (SYMUNOCC(d, ia, isyma) > 0 &&
                (SYMUNOCC(d, ia, isymb) > 1 || (SYMUNOCC(d, ia, isymb) == 1 && isyma != isymb))) {
                allowed = 1;
                break;
            }
        }
    }
    if (!allowed) return 0;
    int a, b = -1;
    for (;;) {
        a = pick_a(c, spin, rs_next(rs));
        if (!tbit(f, a)) {
            int imsb = (spin - c->orb_ms[a] + 3) / 2 - 1;
            int isymb = cross(c, sym, c->orb_sym[a]);
            int nu = SYMUNOCC(d, imsb, isymb);
            if (nu > 1 || (nu == 1 && (isymb != c->orb_sym[a] || spin == 0))) {
                for (;;) {
                    int ind = (int)((double)NBSS(imsb, isymb) * rs_next(rs));
                    b = SSBF(ind, imsb, isymb);
                    if (b != a && !tbit(f, b)) break;
                }
                break;
            }
        }
    }
    if (a > b) { int t = a; a = b; b = t; }
    *a_out = a;
    *b_out = b;
    return 1;
}

/* find_ab_mol (src/excit_gen_mol.f90:1018-1138). */
static int find_ab_mol(const oracle_ctx *c, rstream *rs, const uint64_t *f, int sym, int spin, int *a_out,
                       int *b_out) {
    int a, b;
    for (;;) {
        a = pick_a(c, spin, rs_next(rs));
        if (!tbit(f, a)) break;
    }
    int imsb = (spin - c->orb_ms[a] + 3) / 2 - 1;
    int isymb = cross(c, sym, c->orb_sym[a]);
    int allowed;
    if (NBSS(imsb, isymb) == 0) {
        allowed = 0;
    } else if (spin != 0 && isymb == c->orb_sym[a] && NBSS(imsb, isymb) == 1) {
        allowed = 0;
    } else {
        for (;;) {
            int ind = (int)((double)NBSS(imsb, isymb) * rs_next(rs));
            b = SSBF(ind, imsb, isymb);
            if (b != a) break;
        }
        allowed = !tbit(f, b);
        if (a > b) { int t = a; a = b; b = t; }
    }
    *a_out = a;
    *b_out = allowed ? b : -1;
    return allowed;
}

/* choose_ia_mol (src/excit_gen_mol.f90:521-618), op_sym = gamma. */
static int choose_ia_mol(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int *i_out,
                         int *a_out) {
    int allowed = 0;
    for (int k = 0; k < c->nel; k++) {
        int p = d->occ[k];
        if (SYMUNOCC(d, ims_of(c, p), c->orb_sym[p]) != 0) { allowed = 1; break; }
    }
    if (!allowed) return 0;
    int i, a;
    for (;;) {
        i = d->occ[(int)(rs_next(rs) * (double)c->nel)];
        int imsa = ims_of(c, i), isyma = c->orb_sym[i];
        if (SYMUNOCC(d, imsa, isyma) != 0) {
            for (;;) {
                int ind = (int)((double)NBSS(imsa, isyma) * rs_next(rs));
                a = SSBF(ind, imsa, isyma);
                if (!tbit(f, a)) break;
            }
            break;
        }
    }
    *i_out = i;
    *a_out = a;
    return 1;
}

/* find_ia_mol (src/excit_gen_mol.f90:950-1016). */
static int find_ia_mol(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int *i_out,
                       int *a_out) {
    int i = d->occ[(int)(rs_next(rs) * (double)c->nel)];
    int imsa = ims_of(c, i), isyma = c->orb_sym[i];
    int ind = (int)((double)NBSS(imsa, isyma) * rs_next(rs));
    *i_out = i;
    if (NBSS(imsa, isyma) == 0) return 0;
    int a = SSBF(ind, imsa, isyma);
    *a_out = a;
    return !tbit(f, a);
}

/* calc_pgen_single_mol (src/excit_gen_mol.f90:1140-1200). */
static double calc_pgen_single_mol(const oracle_ctx *c, const det_info *d, int a) {
    int ni = c->nel;
    for (int k = 0; k < c->nel; k++) {
        int p = d->occ[k];
        if (SYMUNOCC(d, ims_of(c, p), c->orb_sym[p]) == 0) ni--;
    }
    return 1.0 / (double)(ni * SYMUNOCC(d, ims_of(c, a), c->orb_sym[a]));
}

/* calc_pgen_double_mol (src/excit_gen_mol.f90:1202-1327). */
static double calc_pgen_double_mol(const oracle_ctx *c, int ij_sym, int a, int b, int spin, const det_info *d) {
    int imsa = ims_of(c, a), imsb = ims_of(c, b);
    int n_aij;
    double p_bija, p_aijb;
    if (spin == 0) {
        n_aij = c->nvirt;
        for (int isyma = 0; isyma < c->nsym; isyma++) {
            int isymb = cross(c, isyma, ij_sym);
            if (SYMUNOCC(d, 0, isymb) == 0) n_aij -= SYMUNOCC(d, 1, isyma);
            if (SYMUNOCC(d, 1, isymb) == 0) n_aij -= SYMUNOCC(d, 0, isyma);
        }
        p_aijb = 1.0 / (double)SYMUNOCC(d, imsa, c->orb_sym[a]);
        p_bija = 1.0 / (double)SYMUNOCC(d, imsb, c->orb_sym[b]);
    } else {
        int is = spin == -2 ? 0 : 1;
        n_aij = spin == -2 ? c->nvirt_beta : c->nvirt_alpha;
        for (int isyma = 0; isyma < c->nsym; isyma++) {
            int isymb = cross(c, isyma, ij_sym);
            if (SYMUNOCC(d, is, isymb) == 0)
                n_aij -= SYMUNOCC(d, is, isyma);
            else if (isyma == isymb && SYMUNOCC(d, is, isymb) == 1)
                n_aij -= SYMUNOCC(d, is, isyma);
        }
        if (c->orb_sym[a] == c->orb_sym[b]) {
            p_aijb = 1.0 / (double)(SYMUNOCC(d, imsa, c->orb_sym[a]) - 1);
            p_bija = 1.0 / (double)(SYMUNOCC(d, imsb, c->orb_sym[b]) - 1);
        } else {
            p_aijb = 1.0 / (double)SYMUNOCC(d, imsa, c->orb_sym[a]);
            p_bija = 1.0 / (double)SYMUNOCC(d, imsb, c->orb_sym[b]);
        }
    }
    return (1.0 / (double)n_aij) * (p_bija + p_aijb);
}

/* calc_pgen_single_mol_no_renorm (src/excit_gen_mol.f90:1329-1366). */
static double calc_pgen_single_mol_no_renorm(const oracle_ctx *c, int a) {
    return 1.0 / (double)(c->nel * NBSS(ims_of(c, a), c->orb_sym[a]));
}

/* calc_pgen_double_mol_no_renorm (src/excit_gen_mol.f90:1368-1445). */
static double calc_pgen_double_mol_no_renorm(const oracle_ctx *c, int a, int b, int spin) {
    int n_aij = spin == -2 ? c->nvirt_beta : (spin == 0 ? c->nvirt : c->nvirt_alpha);
    int imsa = ims_of(c, a), isyma = c->orb_sym[a], imsb = ims_of(c, b), isymb = c->orb_sym[b];
    double p_bija, p_aijb;
    if (isyma == isymb && imsa == imsb) {
        p_aijb = 1.0 / (double)(NBSS(imsa, isyma) - 1);
        p_bija = 1.0 / (double)(NBSS(imsb, isymb) - 1);
    } else {
        p_aijb = 1.0 / (double)NBSS(imsa, isyma);
        p_bija = 1.0 / (double)NBSS(imsb, isymb);
    }
    return (1.0 / (double)n_aij) * (p_bija + p_aijb);
}

/* ------------------------------------------------------------------------- */
/* Excitation generation: one spawning attempt                                */
/* ------------------------------------------------------------------------- */

typedef struct {
    excit_t e;
    double pgen, hmatel;
    int allowed;
    int64_t nspawn;
    int64_t nspawn_rdm; /* spawn_rdm's unweighted attempt (src/spawning.F90:588-676) */
} attempt_t;

/* stochastic_round_spawned_particle (src/stoch_utils.f90:87-136). */
static int64_t round_spawned(int64_t cutoff, double pspawn, rstream *rs) {
    int64_t nspawn;
    if (pspawn < (double)cutoff) {
        if (pspawn > rs_next(rs) * (double)cutoff) nspawn = cutoff;
        else nspawn = 0;
    } else {
        nspawn = (int64_t)pspawn;
        double padd = pspawn - (double)nspawn;
        if (padd > rs_next(rs)) nspawn = nspawn + 1;
    }
    return nspawn;
}

/* Fortran sign(a, b) for integers: |a| with the sign of b (b >= 0 -> +). */
static inline int64_t isign64(int64_t a, int64_t b) {
    int64_t m = a < 0 ? -a : a;
    return b >= 0 ? m : -m;
}

/* set_child_sign (src/spawning.F90:680-709). */
static inline int64_t child_sign(double hmatel, int64_t parent, int64_t nspawn) {
    if (hmatel > 0.0) return -isign64(nspawn, parent);
    return isign64(nspawn, parent);
}

/* spawn_lattice_split_gen (src/spawning.F90:215-315) with gen_excit_init_hub_k /
 * gen_excit_finalise_hub_k (src/excit_gen_hub_k.f90:29-156) or the no_renorm
 * pair (:158-277). */
static void attempt_hub_k(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int64_t parent,
                          attempt_t *out, int complete) {
    int i, j, ij_sym, a = -1, b = -1;
    double pgen, abs_h;
    memset(out, 0, sizeof(*out));
    out->e.nexcit = 2;
    choose_ij_hub_k(c, rs, d, &i, &j, &ij_sym);
    int renorm = c->cfg.excit_gen != HGPU_EXCIT_GEN_NO_RENORM;
    if (renorm) {
        pgen = calc_pgen_hub_k(c, ij_sym, f, d);
        out->allowed = 1.0 / pgen > DEPSILON;
        abs_h = fabs(c->coulomb_k);
    } else {
        out->allowed = find_ab_hub_k(c, rs, f, d, ij_sym, &a, &b);
        if (out->allowed) {
            pgen = 1.0 / (double)(c->nalpha * c->nbeta * c->nvirt_alpha);
            abs_h = fabs(c->coulomb_k);
        } else {
            pgen = 1.0;
            abs_h = 0.0;
        }
    }
    out->pgen = pgen;
    double pspawn = (double)c->real_factor * c->cfg.tau * abs_h / pgen;
    int64_t nspawn = round_spawned(c->cutoff, pspawn, rs);
    out->e.from[0] = i;
    out->e.from[1] = j;
    if (nspawn != 0 || (complete && out->allowed)) {
        /* gen_excit_finalise_hub_k: choose_ab_hub_k redraws until b is free */
        if (renorm) {
            int ok = 0;
            while (!ok) ok = find_ab_hub_k(c, rs, f, d, ij_sym, &a, &b);
        }
        out->e.to[0] = a;
        out->e.to[1] = b;
        out->hmatel = sc2_hub_k_excit(c, f, &out->e);
        if (nspawn != 0) nspawn = child_sign(out->hmatel, parent, nspawn);
    } else {
        out->e.to[0] = a;
        out->e.to[1] = b;
        out->hmatel = abs_h;
    }
    out->nspawn = nspawn;
}

/* ------------------------------------------------------------------------- */
/* Heat-bath generators (src/excit_gen_heat_bath_mol.F90)                     */
/* ------------------------------------------------------------------------- */

#define HB_IJ(c, i, j) ((c)->hb_ij_w[(size_t)(i) * (c)->nbasis + (j)])
#define HB_IJA(c, i, j, a) ((c)->hb_ija_w[((size_t)(i) * (c)->nbasis + (j)) * (c)->nbasis + (a)])
#define HB_IJA_TOT(c, i, j) ((c)->hb_ija_tot[(size_t)(i) * (c)->nbasis + (j)])
#define HB_IJAB(c, i, j, a, b) \
    ((c)->hb_ijab_w[(((size_t)(i) * (c)->nbasis + (j)) * (c)->nbasis + (a)) * (c)->nbasis + (b)])
#define HB_IJAB_TOT(c, i, j, a) ((c)->hb_ijab_tot[((size_t)(i) * (c)->nbasis + (j)) * (c)->nbasis + (a)])

/* generate_alias_tables (lib/local/alias.f90:100-184), 0-based: the last
 * overfull entry is paired with the last underfull one until either list is
 * empty. */
static void alias_build(int n, const double *w, double tot, double *U, int32_t *K) {
    int under[MAXB], over[MAXB], nu = 0, no = 0;
    double f = (double)n / tot;
    for (int i = 0; i < n; i++) {
        U[i] = w[i] * f;
        if (U[i] <= 1.0) under[nu++] = i;
        else over[no++] = i;
        K[i] = i;
    }
    while (no > 0 && nu > 0) {
        int ov = over[no - 1], un = under[nu - 1];
        K[un] = ov;
        nu--;
        U[ov] = U[ov] - (1.0 - U[un]);
        if (U[ov] < 1.0) {
            under[nu++] = over[no - 1];
            no--;
        }
    }
}

/* select_weighted_value_precalc (lib/local/alias.f90:13-60). */
static int alias_draw(rstream *rs, int n, const double *U, const int32_t *K) {
    double x = rs_next(rs) * (double)n;
    int k = (int)floor(x);
    x = x - (double)k;
    return x < U[k] ? k : K[k];
}

/* select_weighted_value (lib/local/alias.f90:62-98): alias table built on the fly. */
static int alias_select(rstream *rs, int n, const double *w, double tot) {
    double U[MAXB];
    int32_t K[MAXB];
    alias_build(n, w, tot, U, K);
    return alias_draw(rs, n, U, K);
}

/* init_excit_mol_heat_bath (src/excit_gen_heat_bath_mol.F90:14-243), serial
 * loop order.  Alias tables that the reference leaves unset (zero total weight)
 * are U = 0, K = self here.  Returns -1 where the reference stops with "Not all
 * possible single excitations can be accounted for" (original = 1 only). */
static int init_heat_bath(oracle_ctx *c, int original) {
    int nb = c->nbasis;
    size_t n2 = (size_t)nb * nb, n3 = n2 * nb, n4 = n3 * nb;
    c->hb_i_w = (double *)calloc(nb, sizeof(double));
    c->hb_ij_w = (double *)calloc(n2, sizeof(double));
    c->hb_ija_w = (double *)calloc(n3, sizeof(double));
    c->hb_ija_tot = (double *)calloc(n2, sizeof(double));
    c->hb_ija_U = (double *)calloc(n3, sizeof(double));
    c->hb_ija_K = (int32_t *)calloc(n3, sizeof(int32_t));
    c->hb_ijab_w = (double *)calloc(n4, sizeof(double));
    c->hb_ijab_tot = (double *)calloc(n3, sizeof(double));
    c->hb_ijab_U = (double *)calloc(n4, sizeof(double));
    c->hb_ijab_K = (int32_t *)calloc(n4, sizeof(int32_t));
    int *j_nonzero = (int *)calloc(n2, sizeof(int)); /* [i*nb + a] */
    if (!c->hb_ijab_U || !c->hb_ijab_K || !c->hb_ijab_w || !j_nonzero) return -2;
    c->hb_on = 1;
    int bias = 0;
    for (int i = 0; i < nb; i++) {
        double i_weight = 0.0;
        for (int j = 0; j < nb; j++) {
            double ij_weight = 0.0;
            HB_IJA_TOT(c, i, j) = 0.0;
            if (i != j) {
                int it = j < i ? j : i, jt = j < i ? i : j;
                int ij_sym = cross(c, c->orb_sym[it], c->orb_sym[jt]);
                double ija_weights_tot = 0.0, i_weight_extra = 0.0;
                for (int a = 0; a < nb; a++) {
                    double ija_weight = 0.0;
                    HB_IJAB_TOT(c, i, j, a) = 0.0;
                    if (a != i && a != j) {
                        int isymb = cross(c, ij_sym, c->orb_sym[a]);
                        for (int b = 0; b < nb; b++) {
                            double ijab_weight = 0.0;
                            if (((c->orb_ms[it] == c->orb_ms[a] && c->orb_ms[jt] == c->orb_ms[b]) ||
                                 (c->orb_ms[it] == c->orb_ms[b] && c->orb_ms[jt] == c->orb_ms[a])) &&
                                c->orb_sym[b] == isymb && b != a && b != i && b != j) {
                                int at = b < a ? b : a, bt = b < a ? a : b;
                                double h = fabs(sc2_mol_excit(c, it, jt, at, bt, 0));
                                i_weight_extra = i_weight_extra + h;
                                ij_weight = ij_weight + h;
                                ija_weight = ija_weight + h;
                                ijab_weight = ijab_weight + h;
                            }
                            HB_IJAB(c, i, j, a, b) = ijab_weight;
                            HB_IJAB_TOT(c, i, j, a) = HB_IJAB_TOT(c, i, j, a) + ijab_weight;
                        }
                    }
                    HB_IJA(c, i, j, a) = ija_weight;
                    ija_weights_tot = ija_weights_tot + ija_weight;
                    if (ija_weight > DEPSILON) j_nonzero[(size_t)i * nb + a]++;
                }
                i_weight = i_weight + i_weight_extra;
                HB_IJA_TOT(c, i, j) = HB_IJA_TOT(c, i, j) + ija_weights_tot;
            }
            HB_IJ(c, i, j) = ij_weight;
        }
        c->hb_i_w[i] = i_weight;
        for (int a = 0; a < nb; a++) {
            if (j_nonzero[(size_t)i * nb + a] < nb - c->nel && original && i != a) {
                if (c->orb_sym[a] == c->orb_sym[i] && c->orb_ms[a] == c->orb_ms[i]) bias = 1;
            }
        }
    }
    free(j_nonzero);
    for (size_t t = 0; t < n3; t++) c->hb_ija_K[t] = (int32_t)(t % nb);
    for (size_t t = 0; t < n4; t++) c->hb_ijab_K[t] = (int32_t)(t % nb);
    for (int i = 0; i < nb; i++) {
        for (int j = 0; j < nb; j++) {
            if (fabs(HB_IJA_TOT(c, i, j)) > 0.0) {
                size_t o3 = ((size_t)i * nb + j) * nb;
                alias_build(nb, c->hb_ija_w + o3, HB_IJA_TOT(c, i, j), c->hb_ija_U + o3, c->hb_ija_K + o3);
                for (int a = 0; a < nb; a++) {
                    if (fabs(HB_IJAB_TOT(c, i, j, a)) > 0.0) {
                        size_t o4 = (o3 + a) * nb;
                        alias_build(nb, c->hb_ijab_w + o4, HB_IJAB_TOT(c, i, j, a), c->hb_ijab_U + o4,
                                    c->hb_ijab_K + o4);
                    }
                }
            }
        }
    }
    return bias ? -1 : 0;
}

/* The psingle of a single i -> a inside the heat-bath double branch
 * (src/excit_gen_heat_bath_mol.F90:350-366, :396-409, ...): 0 when i -> a breaks
 * spin or symmetry, else |h_ia| / (W + |h_ia|) below W = weights_tot(a,j,i), 0.5 above. */
static double hb_psingle(const oracle_ctx *c, const det_info *d, int i, int a, double wtot, double *abs_h) {
    if (c->orb_sym[a] != c->orb_sym[i] || c->orb_ms[a] != c->orb_ms[i]) return 0.0;
    double h = fabs(sc1_mol_excit(c, d->occ, i, a, 0));
    if (abs_h) *abs_h = h;
    return h < wtot ? h / (wtot + h) : 0.5;
}

/* select_ij_heat_bath (src/excit_gen_utils.f90:9-66) after find_i_d_weights
 * (:142-167). */
typedef struct {
    double wi[MAXEL], ijw[MAXEL], jiw[MAXEL];
    double wi_tot, ij_tot, ji_tot;
    int i_ind, j_ind, i, j;
} hb_ij_t;

static int select_ij_heat_bath(const oracle_ctx *c, rstream *rs, const det_info *d, hb_ij_t *s) {
    int nel = c->nel;
    s->wi_tot = 0.0;
    for (int p = 0; p < nel; p++) {
        s->wi[p] = c->hb_i_w[d->occ[p]];
        s->wi_tot = s->wi_tot + s->wi[p];
    }
    s->i_ind = alias_select(rs, nel, s->wi, s->wi_tot);
    s->i = d->occ[s->i_ind];
    s->ij_tot = 0.0;
    for (int p = 0; p < nel; p++) {
        s->ijw[p] = HB_IJ(c, s->i, d->occ[p]);
        s->ij_tot = s->ij_tot + s->ijw[p];
    }
    s->j_ind = -1;
    s->j = -1;
    if (!(s->ij_tot > 0.0)) return 0;
    s->j_ind = alias_select(rs, nel, s->ijw, s->ij_tot);
    s->j = d->occ[s->j_ind];
    s->ji_tot = 0.0;
    for (int p = 0; p < nel; p++) {
        s->jiw[p] = HB_IJ(c, s->j, d->occ[p]);
        s->ji_tot = s->ji_tot + s->jiw[p];
    }
    return 1;
}

/* gen_excit_mol_heat_bath (src/excit_gen_heat_bath_mol.F90:258-547). */
static void gen_heat_bath(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, attempt_t *out,
                          double *pgen_out, double *hmatel_out) {
    hb_ij_t s;
    out->e.nexcit = 2;
    int allowed = select_ij_heat_bath(c, rs, d, &s);
    int i = s.i, j = s.j;
    out->e.from[0] = i;
    out->e.from[1] = j;
    if (!(allowed && fabs(HB_IJA_TOT(c, i, j)) > 0.0)) allowed = 0;
    int a = -1, b = -1, dbl = 1;
    double psingle = 0.0, hmod_ia = 0.0;
    if (allowed) {
        size_t o3 = ((size_t)i * c->nbasis + j) * c->nbasis;
        a = alias_draw(rs, c->nbasis, c->hb_ija_U + o3, c->hb_ija_K + o3);
        if (!tbit(f, a)) {
            if (c->orb_sym[a] == c->orb_sym[i] && c->orb_ms[a] == c->orb_ms[i]) {
                hmod_ia = fabs(sc1_mol_excit(c, d->occ, i, a, perm1(c, f, i, a)));
                double x = rs_next(rs);
                double wt = HB_IJAB_TOT(c, i, j, a);
                psingle = hmod_ia < wt ? hmod_ia / (wt + hmod_ia) : 0.5;
                dbl = !(x < psingle);
            } else {
                dbl = 1;
                psingle = 0.0;
            }
        } else {
            allowed = 0;
        }
    }
    double pgen = 1.0, hmatel = 0.0;
    if (allowed) {
        if (dbl) {
            size_t o4 = (((size_t)i * c->nbasis + j) * c->nbasis + a) * c->nbasis;
            b = alias_draw(rs, c->nbasis, c->hb_ijab_U + o4, c->hb_ijab_K + o4);
            if (!tbit(f, b)) {
                double p_ij = (s.wi[s.i_ind] / s.wi_tot) * (s.ijw[s.j_ind] / s.ij_tot);
                double p_ji = (s.wi[s.j_ind] / s.wi_tot) * (s.jiw[s.i_ind] / s.ji_tot);
                double pgen_ija = p_ij * (HB_IJA(c, i, j, a) / HB_IJA_TOT(c, i, j)) * (1.0 - psingle) *
                                  (HB_IJAB(c, i, j, a, b) / HB_IJAB_TOT(c, i, j, a));
                psingle = hb_psingle(c, d, i, b, HB_IJAB_TOT(c, i, j, b), NULL);
                double pgen_ijb = p_ij * (HB_IJA(c, i, j, b) / HB_IJA_TOT(c, i, j)) * (1.0 - psingle) *
                                  (HB_IJAB(c, i, j, b, a) / HB_IJAB_TOT(c, i, j, b));
                psingle = hb_psingle(c, d, j, a, HB_IJAB_TOT(c, j, i, a), NULL);
                double pgen_jia = p_ji * (HB_IJA(c, j, i, a) / HB_IJA_TOT(c, j, i)) * (1.0 - psingle) *
                                  (HB_IJAB(c, j, i, a, b) / HB_IJAB_TOT(c, j, i, a));
                psingle = hb_psingle(c, d, j, b, HB_IJAB_TOT(c, j, i, b), NULL);
                double pgen_jib = p_ji * (HB_IJA(c, j, i, b) / HB_IJA_TOT(c, j, i)) * (1.0 - psingle) *
                                  (HB_IJAB(c, j, i, b, a) / HB_IJAB_TOT(c, j, i, b));
                pgen = pgen_ija + pgen_ijb + pgen_jia + pgen_jib;
                int f0 = i < j ? i : j, f1 = i < j ? j : i, t0 = a < b ? a : b, t1 = a < b ? b : a;
                out->e.from[0] = f0;
                out->e.from[1] = f1;
                out->e.to[0] = t0;
                out->e.to[1] = t1;
                out->e.perm = perm2(c, f, f0, f1, t0, t1);
                hmatel = sc2_mol_excit(c, f0, f1, t0, t1, out->e.perm);
            } else {
                allowed = 0;
            }
        } else {
            out->e.nexcit = 1;
            out->e.from[1] = -1;
            out->e.to[0] = a;
            out->e.perm = perm1(c, f, i, a);
            hmatel = sc1_mol_excit(c, d->occ, i, a, out->e.perm);
            pgen = 0.0;
            for (int q = 0; q < c->nel; q++) {
                int oq = d->occ[q];
                /* a q that has no double excitation with i (weights_tot(q,i) = 0) adds
                 * 0 * (0/0) in the reference, a NaN p_gen; its true contribution is 0 */
                if (i != oq && a != oq && HB_IJA_TOT(c, i, oq) > 0.0) {
                    double wt = HB_IJAB_TOT(c, i, oq, a);
                    double psq = hmod_ia < wt ? hmod_ia / (wt + hmod_ia) : 0.5;
                    pgen = pgen + psq * (s.ijw[q] / s.ij_tot) * (HB_IJA(c, i, oq, a) / HB_IJA_TOT(c, i, oq));
                }
            }
            pgen = pgen * (s.wi[s.i_ind] / s.wi_tot);
        }
    }
    out->allowed = allowed;
    *pgen_out = allowed ? pgen : 1.0;
    *hmatel_out = allowed ? hmatel : 0.0;
}

/* slater_condon1_mol (src/hamiltonian_molecular.f90:140-196) with perm = false:
 * 0 unless i and a share spin and symmetry. */
static double sc1_mol_checked(const oracle_ctx *c, const int *occ, int i, int a) {
    if (c->orb_sym[i] != c->orb_sym[a] || c->orb_ms[i] != c->orb_ms[a]) return 0.0;
    return sc1_mol_excit(c, occ, i, a, 0);
}

/* find_ia_single_weights (src/excit_gen_utils.f90:169-212) and
 * gen_single_excit_heat_bath_exact (src/excit_gen_heat_bath_mol.F90:732-807):
 * i chosen with weight sum_a |H_ia|, then a with weight |H_ia|. */
static void gen_single_heat_bath_exact(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d,
                                       attempt_t *out, double *pgen_out, double *hmatel_out) {
    int nel = c->nel, nvirt = c->nvirt;
    int unocc[MAXB], nu = 0;
    for (int p = 0; p < c->nbasis; p++)
        if (!tbit(f, p)) unocc[nu++] = p;
    double wi[MAXEL], row[MAXB], tot = 0.0;
    for (int ii = 0; ii < nel; ii++) {
        wi[ii] = 0.0;
        for (int aa = 0; aa < nvirt; aa++) wi[ii] = wi[ii] + fabs(sc1_mol_checked(c, d->occ, d->occ[ii], unocc[aa]));
        tot = tot + wi[ii];
    }
    out->e.nexcit = 1;
    if (tot < DEPSILON) {
        out->allowed = 0;
        *pgen_out = 1.0;
        *hmatel_out = 0.0;
        return;
    }
    int i_ind = alias_select(rs, nel, wi, tot);
    int i = d->occ[i_ind];
    for (int aa = 0; aa < nvirt; aa++) row[aa] = fabs(sc1_mol_checked(c, d->occ, i, unocc[aa]));
    int a_ind = alias_select(rs, nvirt, row, wi[i_ind]);
    int a = unocc[a_ind];
    out->allowed = 1;
    out->e.from[0] = i;
    out->e.to[0] = a;
    *pgen_out = c->pattempt_single * (wi[i_ind] / tot) * (row[a_ind] / wi[i_ind]);
    out->e.perm = perm1(c, f, i, a);
    *hmatel_out = sc1_mol_excit(c, d->occ, i, a, out->e.perm);
}

/* gen_excit_mol_heat_bath_uniform, double branch
 * (src/excit_gen_heat_bath_mol.F90:619-705). */
static void gen_heat_bath_uniform_double(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d,
                                         attempt_t *out, double *pgen_out, double *hmatel_out) {
    hb_ij_t s;
    out->e.nexcit = 2;
    int allowed = select_ij_heat_bath(c, rs, d, &s);
    int i = s.i, j = s.j;
    if (!(allowed && fabs(HB_IJA_TOT(c, i, j)) > 0.0)) allowed = 0;
    double pgen = 1.0, hmatel = 0.0;
    double pij = 0.0;
    if (s.j_ind >= 0)
        pij = ((s.wi[s.i_ind] / s.wi_tot) * (s.ijw[s.j_ind] / s.ij_tot)) +
              ((s.wi[s.j_ind] / s.wi_tot) * (s.jiw[s.i_ind] / s.ji_tot));
    if (j >= 0 && j < i) {
        int t = j;
        j = i;
        i = t;
    }
    out->e.from[0] = i;
    out->e.from[1] = j;
    int a = -1, b = -1;
    if (allowed) {
        size_t o3 = ((size_t)i * c->nbasis + j) * c->nbasis;
        a = alias_draw(rs, c->nbasis, c->hb_ija_U + o3, c->hb_ija_K + o3);
        if (fabs(HB_IJAB_TOT(c, i, j, a)) > 0.0 && !tbit(f, a)) {
            size_t o4 = (o3 + a) * c->nbasis;
            b = alias_draw(rs, c->nbasis, c->hb_ijab_U + o4, c->hb_ijab_K + o4);
            allowed = !tbit(f, b);
        } else {
            allowed = 0;
        }
    }
    if (allowed) {
        int t0 = a < b ? a : b, t1 = a < b ? b : a;
        out->e.to[0] = t0;
        out->e.to[1] = t1;
        out->e.perm = perm2(c, f, i, j, t0, t1);
        hmatel = sc2_mol_excit(c, i, j, t0, t1, out->e.perm);
        pgen = (1.0 - c->pattempt_single) * pij *
               (((HB_IJA(c, i, j, a) / HB_IJA_TOT(c, i, j)) * (HB_IJAB(c, i, j, a, b) / HB_IJAB_TOT(c, i, j, a))) +
                ((HB_IJA(c, i, j, b) / HB_IJA_TOT(c, i, j)) * (HB_IJAB(c, i, j, b, a) / HB_IJAB_TOT(c, i, j, b))));
    }
    out->allowed = allowed;
    *pgen_out = pgen;
    *hmatel_out = hmatel;
}

/* gen_excit_mol / gen_excit_mol_no_renorm (src/excit_gen_mol.f90:16-284) with
 * spawn_standard + attempt_to_spawn (src/spawning.F90:34-123, :711-768). */
/* ------------------------------------------------------------------------- */
/* uniform_power_pitzer / uniform_cauchy_schwarz                              */
/* (gen_excit_mol_power_pitzer_occ, src/excit_gen_power_pitzer_mol.F90)      */
/* ------------------------------------------------------------------------- */

/* The weight of q for an electron in p: sqrt|<pq|qp>| for power_pitzer
 * (get_two_body_int_ex_mol_real, src/hamiltonian_molecular.f90:392-411) or
 * sqrt|<pq|pq>| for cauchy_schwarz (get_two_body_int_cou_mol_real, :413-434),
 * both through get_two_body_int_mol_real's spin check
 * (src/molecular_integrals.F90:1147-1177). */
static double pp_weight(const oracle_ctx *c, int p, int q) {
    double v = 0.0;
    if (c->cfg.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC || c->cfg.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ)
        v = v2_get(c, p, q, p, q);
    else if (c->orb_ms[p] == c->orb_ms[q]) v = v2_get(c, p, q, q, p);
    return sqrt(fabs(v));
}

/* create_weighted_excitation_list_mol (src/hamiltonian_molecular.f90:348-390):
 * the weights of p over a list, 0 for the entry equal to skip, and their sum in
 * list order. */
static double pp_weight_list(const oracle_ctx *c, int p, int skip, const int *list, int n, double *w) {
    double tot = 0.0;
    for (int k = 0; k < n; k++) {
        if (list[k] != skip) {
            w[k] = pp_weight(c, p, list[k]);
            tot = tot + w[k];
        } else {
            w[k] = 0.0;
        }
    }
    return tot;
}

/* binary_search over an ascending integer list (src/search.f90): the position
 * of x, or where it would be inserted. */
static int int_lower_bound(const int *list, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (list[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* init_double_weights_ab (src/excit_gen_utils.f90:68-138): the sum of
 * |<ij||ab>| over every ordered pair a /= b that conserves spin and symmetry
 * (occupied orbitals included, i and j excluded), in the reference's loop
 * order, added to w (the argument is intent(inout) there). */
static double double_weights_ab(const oracle_ctx *c, int i, int j, double w) {
    const int it = i < j ? i : j, jt = i < j ? j : i;
    const int ij_sym = cross(c, c->orb_sym[it], c->orb_sym[jt]);
    for (int a = 0; a < c->nbasis; a++) {
        if (a == it || a == jt) continue;
        const int isymb = cross(c, ij_sym, c->orb_sym[a]);
        for (int b = 0; b < c->nbasis; b++) {
            const int spin = (c->orb_ms[it] == c->orb_ms[a] && c->orb_ms[jt] == c->orb_ms[b]) ||
                             (c->orb_ms[it] == c->orb_ms[b] && c->orb_ms[jt] == c->orb_ms[a]);
            if (spin && c->orb_sym[b] == isymb && a != b && b != it && b != jt) {
                const int at = b < a ? b : a, bt = b < a ? a : b;
                w = w + fabs(sc2_mol_excit(c, it, jt, at, bt, 0));
            }
        }
    }
    return w;
}

/* init_excit_mol_power_pitzer_orderM_ij (src/excit_gen_power_pitzer_mol.F90:574-648):
 * ppm_ij_d_weights and ppm_i_d_weights (the sum over j in order), kept in
 * the arrays select_ij_heat_bath reads. */
static void init_pp_ij(oracle_ctx *c) {
    const int nb = c->nbasis;
    c->hb_i_w = (double *)calloc((size_t)nb, sizeof(double));
    c->hb_ij_w = (double *)calloc((size_t)nb * nb, sizeof(double));
    for (int i = 0; i < nb; i++) {
        double i_weight_extra = 0.0;
        for (int j = 0; j < nb; j++) {
            double w = 0.0;
            if (i != j) w = double_weights_ab(c, i, j, 0.0);
            c->hb_ij_w[(size_t)i * nb + j] = w;
            i_weight_extra = i_weight_extra + w;
        }
        c->hb_i_w[i] = i_weight_extra;
    }
}

/* The double excitations of gen_excit_mol_power_pitzer_occ
 * (src/excit_gen_power_pitzer_mol.F90:1260-1547): i, j uniform, or by
 * select_ij_heat_bath over ppm_ij_d_weights for the heat_bath_ variants; a
 * from the determinant's unoccupied orbitals of i's spin, b from the orbitals
 * of the spin and irrep that conserve both (b /= a), each by an alias table
 * built for the attempt; for parallel spins p_gen adds the reverse order (b
 * from i, a from j). */
static void gen_pp_occ_double(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d,
                              attempt_t *out, double *pgen, double *hmatel) {
    int i, j, ij_sym, ij_spin;
    double pgen_ij;
    out->e.nexcit = 2;
    if (c->cfg.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
        c->cfg.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ) {
        hb_ij_t q;
        const int ok = select_ij_heat_bath(c, rs, d, &q);
        i = q.i;
        j = q.j;
        pgen_ij = 0.0;
        if (ok)
            pgen_ij = ((q.wi[q.i_ind] / q.wi_tot) * (q.ijw[q.j_ind] / q.ij_tot)) +
                      ((q.wi[q.j_ind] / q.wi_tot) * (q.jiw[q.i_ind] / q.ji_tot));
        if (j >= 0 && j < i) {
            const int t = j;
            j = i;
            i = t;
        }
        out->e.from[0] = i;
        out->e.from[1] = j;
        if (!ok) {
            out->allowed = 0;
            out->e.to[0] = out->e.to[1] = -1;
            *hmatel = 0.0;
            *pgen = 1.0;
            return;
        }
        ij_sym = cross(c, c->orb_sym[i], c->orb_sym[j]);
        ij_spin = c->orb_ms[i] + c->orb_ms[j];
    } else {
        choose_ij_mol(c, rs, d, &i, &j, &ij_sym, &ij_spin, &pgen_ij);
        out->e.from[0] = i;
        out->e.from[1] = j;
    }
    int unocc[MAXB], nv = 0;
    for (int p = 0; p < c->nbasis; p++)
        if (!tbit(f, p) && c->orb_ms[p] == c->orb_ms[i]) unocc[nv++] = p;
    double ia_w[MAXB], jb_w[MAXB], ja_w[MAXB];
    int allowed = 0, a = -1, b = -1;
    if (nv > 0) {
        double ia_tot = pp_weight_list(c, i, -1, unocc, nv, ia_w);
        if (ia_tot > 0.0) {
            int a_ind = alias_select(rs, nv, ia_w, ia_tot);
            a = unocc[a_ind];
            int isymb = cross(c, ij_sym, c->orb_sym[a]);
            int imsb = (ij_spin - c->orb_ms[a] + 1) / 2; /* 0 beta, 1 alpha */
            int nb = NBSS(imsb, isymb);
            int list[MAXB];
            for (int q = 0; q < nb; q++) list[q] = SSBF(q, imsb, isymb);
            double jb_tot = nb > 0 ? pp_weight_list(c, j, a, list, nb, jb_w) : 0.0;
            if (jb_tot > 0.0) {
                int b_ind = alias_select(rs, nb, jb_w, jb_tot);
                b = list[b_ind];
                if (!tbit(f, b)) {
                    double pg;
                    if (ij_spin == 0) {
                        pg = ia_w[a_ind] / ia_tot * jb_w[b_ind] / jb_tot;
                    } else {
                        int b_rev = int_lower_bound(unocc, nv, b);
                        int isyma = cross(c, ij_sym, isymb);
                        int na = NBSS(imsb, isyma);
                        int alist[MAXB];
                        for (int q = 0; q < na; q++) alist[q] = SSBF(q, imsb, isyma);
                        double ja_tot = pp_weight_list(c, j, b, alist, na, ja_w);
                        int a_rev = int_lower_bound(alist, na, a);
                        pg = (ia_w[a_ind] * jb_w[b_ind]) / (ia_tot * jb_tot) +
                             (ia_w[b_rev] * ja_w[a_rev]) / (ia_tot * ja_tot);
                    }
                    *pgen = c->pattempt_double * pg * pgen_ij;
                    allowed = 1;
                }
            }
        }
    }
    out->allowed = allowed;
    if (allowed) {
        out->e.to[0] = a < b ? a : b;
        out->e.to[1] = a < b ? b : a;
        out->e.perm = perm2(c, f, out->e.from[0], out->e.from[1], out->e.to[0], out->e.to[1]);
        *hmatel = sc2_mol_excit(c, out->e.from[0], out->e.from[1], out->e.to[0], out->e.to[1], out->e.perm);
    } else {
        out->e.to[0] = out->e.to[1] = -1;
        *hmatel = 0.0;
        *pgen = 1.0;
    }
}

/* ------------------------------------------------------------------------- */
/* heat_bath_power_pitzer_ref (src/excit_gen_power_pitzer_mol.F90:215-572,    */
/* 941-1258)                                                                  */
/* ------------------------------------------------------------------------- */

enum { PPN_IS = 0, PPN_ID = 1, PPN_IJD = 2, PPN_IAS = 3, PPN_IAD = 4, PPN_JBD = 5 };
#define PPN_W(c, t, r, k) ((c)->ppn_w[t][(size_t)(r) * (c)->ppn_stride[t] + (k)])

/* check_min_weight_ratio (src/excit_gen_power_pitzer_mol.F90:140-213): raises
 * the non-zero weights below min_weight, chosen so that they carry min_ratio
 * of their mean share, and recomputes the total. */
static void min_weight_ratio(double *w, double *tot, int n, double min_ratio) {
    double min_weight_tmp = 0.0, min_weight;
    int nz = 0;
    if (!(*tot > 0.0 && min_ratio > 0.0)) return;
    for (int i = 0; i < n; i++)
        if (w[i] > 0.0) nz++;
    min_weight = (min_ratio / (double)nz) * *tot;
    for (int it = 0; it < 100000 && fabs(min_weight_tmp - min_weight) > DEPSILON; it++) {
        min_weight_tmp = min_weight;
        double keep = 0.0;
        int cnt = 0;
        for (int k = 0; k < n; k++) {
            if (w[k] > 0.0 && w[k] < min_weight) cnt++;
            else keep = keep + w[k];
        }
        if (cnt == nz) break;
        min_weight = (min_ratio / (double)nz) * (keep / (1.0 - (min_ratio * (double)cnt / (double)nz)));
    }
    double t = 0.0;
    for (int j = 0; j < n; j++) {
        if (w[j] > 0.0 && w[j] < min_weight) w[j] = min_weight;
        t = t + w[j];
    }
    *tot = t;
}

/* single_excitation_weight_mol (src/hamiltonian_molecular.f90:444-523): the
 * mean over the reference's occupied j and virtual b of
 * |<ij|ja> - <ij|aj> + <ib|ab> - <ib|ba>|, each integral zero unless its spins
 * match (get_two_body_int_mol_real); a has i's irrep in every call. */
static double single_excitation_weight(const oracle_ctx *c, int i, int a) {
    const int *ms = c->orb_ms;
    int n_jb = 0;
    double weight = 0.0;
    for (int jj = 0; jj < c->nel; jj++) {
        const int j = c->ppn_occ[jj];
        for (int b = 0; b < c->nbasis; b++) {
            if (tbit(c->f0, b)) continue;
            n_jb++;
            const double t1 = (ms[i] == ms[j] && ms[j] == ms[a]) ? v2_get(c, i, j, j, a) : 0.0;
            const double t2 = ms[i] == ms[a] ? v2_get(c, i, j, a, j) : 0.0;
            const double t3 = ms[i] == ms[a] ? v2_get(c, i, b, a, b) : 0.0;
            const double t4 = (ms[i] == ms[b] && ms[b] == ms[a]) ? v2_get(c, i, b, b, a) : 0.0;
            weight = weight + fabs(t1 - t2 + t3 - t4);
        }
    }
    return weight / (double)n_jb;
}

static void ppn_alloc(oracle_ctx *c, int t, int rows, int stride) {
    c->ppn_stride[t] = stride;
    c->ppn_w[t] = (double *)calloc((size_t)rows * stride, sizeof(double));
    c->ppn_U[t] = (double *)calloc((size_t)rows * stride, sizeof(double));
    c->ppn_K[t] = (int32_t *)calloc((size_t)rows * stride, sizeof(int32_t));
    c->ppn_tot[t] = (double *)calloc((size_t)rows, sizeof(double));
}

/* Row r of table t: optional min-weight floor, then its alias table. */
static void ppn_finish_row(oracle_ctx *c, int t, int r, int n, int floor) {
    double *w = &PPN_W(c, t, r, 0);
    if (floor) min_weight_ratio(w, &c->ppn_tot[t][r], n, c->cfg.power_pitzer_min_weight);
    alias_build(n, w, c->ppn_tot[t][r], &c->ppn_U[t][(size_t)r * c->ppn_stride[t]],
                &c->ppn_K[t][(size_t)r * c->ppn_stride[t]]);
}

/* init_excit_mol_power_pitzer_orderN (src/excit_gen_power_pitzer_mol.F90:215-572). */
static void init_ppn(oracle_ctx *c) {
    const int nel = c->nel, nb = c->nbasis, half = nb / 2;
    int n = 0;
    for (int p = 0; p < nb; p++)
        if (tbit(c->f0, p)) c->ppn_occ[n++] = p;
    ppn_alloc(c, PPN_IS, 1, nel);
    ppn_alloc(c, PPN_ID, 1, nel);
    ppn_alloc(c, PPN_IJD, nb, nel);
    ppn_alloc(c, PPN_IAS, nb, c->maxss);
    ppn_alloc(c, PPN_IAD, nb, half);
    ppn_alloc(c, PPN_JBD, nb * c->nsym, c->maxss);
    /* i of a single: summed single weights over a of i's spin and irrep */
    for (int i = 0; i < nel; i++) {
        const int oi = c->ppn_occ[i];
        double w = 0.0;
        for (int a = 0; a < nb; a++)
            if (a != oi && c->orb_sym[a] == c->orb_sym[oi] && c->orb_ms[a] == c->orb_ms[oi])
                w = w + single_excitation_weight(c, oi, a);
        if (w < DEPSILON) w = 10.0 * DEPSILON;
        PPN_W(c, PPN_IS, 0, i) = w;
    }
    for (int i = 0; i < nel; i++) c->ppn_tot[PPN_IS][0] = c->ppn_tot[PPN_IS][0] + PPN_W(c, PPN_IS, 0, i);
    ppn_finish_row(c, PPN_IS, 0, nel, 1);
    /* a of a single from any orbital i */
    for (int i = 0; i < nb; i++) {
        const int ims = ims_of(c, i), sym = c->orb_sym[i], na = NBSS(ims, sym);
        double tot = 0.0;
        for (int a = 0; a < na; a++) {
            double w = 0.0;
            const int q = SSBF(a, ims, sym);
            if (q != i) {
                w = single_excitation_weight(c, i, q);
                if (w < DEPSILON) w = 10.0 * DEPSILON;
            }
            PPN_W(c, PPN_IAS, i, a) = w;
            tot = tot + w;
        }
        c->ppn_tot[PPN_IAS][i] = tot;
        ppn_finish_row(c, PPN_IAS, i, na, 1);
    }
    /* i of a double: one accumulator over j and then a, b */
    for (int i = 0; i < nel; i++) {
        double w = 0.0;
        for (int j = 0; j < nel; j++)
            if (i != j) w = double_weights_ab(c, c->ppn_occ[i], c->ppn_occ[j], w);
        if (w < DEPSILON) w = 10.0 * DEPSILON;
        PPN_W(c, PPN_ID, 0, i) = w;
    }
    for (int i = 0; i < nel; i++) c->ppn_tot[PPN_ID][0] = c->ppn_tot[PPN_ID][0] + PPN_W(c, PPN_ID, 0, i);
    ppn_finish_row(c, PPN_ID, 0, nel, 1);
    /* j (a position in the reference's list) given any orbital i */
    for (int i = 0; i < nb; i++) {
        double tot = 0.0;
        for (int j = 0; j < nel; j++) {
            double w = 0.0;
            if (c->ppn_occ[j] != i) w = double_weights_ab(c, i, c->ppn_occ[j], 0.0);
            if (w < DEPSILON) w = 10.0 * DEPSILON;
            PPN_W(c, PPN_IJD, i, j) = w;
            tot = tot + w;
        }
        c->ppn_tot[PPN_IJD][i] = tot;
        ppn_finish_row(c, PPN_IJD, i, nel, 1);
    }
    /* a of a double over all orbitals of i's spin, b per irrep (i itself weighted 0) */
    for (int i = 0; i < nb; i++) {
        const int ims = ims_of(c, i);
        int list[MAXB];
        for (int k = 0; k < half; k++) list[k] = 2 * k + (ims == 0);
        c->ppn_tot[PPN_IAD][i] = pp_weight_list(c, i, i, list, half, &PPN_W(c, PPN_IAD, i, 0));
        ppn_finish_row(c, PPN_IAD, i, half, 0);
        for (int bsym = 0; bsym < c->nsym; bsym++) {
            const int nbs = NBSS(ims, bsym), r = i * c->nsym + bsym;
            if (nbs <= 0) continue;
            for (int q = 0; q < nbs; q++) list[q] = SSBF(q, ims, bsym);
            c->ppn_tot[PPN_JBD][r] = pp_weight_list(c, i, i, list, nbs, &PPN_W(c, PPN_JBD, r, 0));
            ppn_finish_row(c, PPN_JBD, r, nbs, 0);
        }
    }
}

/* find_diff_ref_cdet (src/excit_gen_utils.f90:220-269) with
 * get_excitation_locations (src/excitations.F90:467-543): for each position of
 * the reference's occupied list, the determinant's orbital standing in for it
 * (itself when occupied in both; otherwise the determinant's extra orbitals in
 * order, swapped forward to match spins). */
static void ref_cdet_occ_list(const oracle_ctx *c, const uint64_t *f, const det_info *d, int *map) {
    int ref_store[MAXEL], det_store[MAXEL], nex = 0, np = 0;
    for (int k = 0; k < c->nel; k++) {
        map[k] = c->ppn_occ[k];
        if (!tbit(f, c->ppn_occ[k])) ref_store[nex++] = k;
    }
    for (int k = 0; k < c->nel; k++)
        if (!tbit(c->f0, d->occ[k])) det_store[np++] = k;
    for (int ii = 0; ii < nex; ii++) {
        const int ms_ref = c->orb_ms[c->ppn_occ[ref_store[ii]]];
        if (ms_ref != c->orb_ms[d->occ[det_store[ii]]]) {
            int jj = ii + 1;
            while (jj < nex && ms_ref != c->orb_ms[d->occ[det_store[jj]]]) jj++;
            if (jj < nex) {
                const int t = det_store[ii];
                det_store[ii] = det_store[jj];
                det_store[jj] = t;
            }
        }
        map[ref_store[ii]] = d->occ[det_store[ii]];
    }
}

/* gen_excit_mol_power_pitzer_orderN (src/excit_gen_power_pitzer_mol.F90:941-1258):
 * i (and j) drawn as positions of the reference's occupied list and mapped
 * onto the determinant; a, b from the precomputed tables of the mapped
 * orbitals. */
static void gen_ppn(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, attempt_t *out,
                    double *pgen_out, double *hmatel_out) {
    int map[MAXEL];
    ref_cdet_occ_list(c, f, d, map);
    const int nel = c->nel;
    int allowed = 0;
    double pgen = 1.0, hmatel = 0.0;
    if (rs_next(rs) < c->pattempt_single) {
        out->e.nexcit = 1;
        const int i_ind = alias_draw(rs, nel, c->ppn_U[PPN_IS], c->ppn_K[PPN_IS]);
        const int i = map[i_ind];
        const int ims = ims_of(c, i), sym = c->orb_sym[i], na = NBSS(ims, sym);
        int a = -1, a_ind = -1;
        if (na > 0) {
            const size_t off = (size_t)i * c->ppn_stride[PPN_IAS];
            a_ind = alias_draw(rs, na, c->ppn_U[PPN_IAS] + off, c->ppn_K[PPN_IAS] + off);
            a = SSBF(a_ind, ims, sym);
            allowed = !tbit(f, a);
        }
        out->e.from[0] = i;
        out->e.to[0] = allowed ? a : -1;
        if (allowed) {
            pgen = (PPN_W(c, PPN_IS, 0, i_ind) / c->ppn_tot[PPN_IS][0]) *
                   (PPN_W(c, PPN_IAS, i, a_ind) / c->ppn_tot[PPN_IAS][i]);
            pgen = c->pattempt_single * pgen;
            out->e.perm = perm1(c, f, i, a);
            hmatel = sc1_mol_excit(c, d->occ, i, a, out->e.perm);
        }
    } else {
        out->e.nexcit = 2;
        const int i_ind = alias_draw(rs, nel, c->ppn_U[PPN_ID], c->ppn_K[PPN_ID]);
        int i = map[i_ind];
        const size_t offj = (size_t)i * c->ppn_stride[PPN_IJD];
        const int j_ind = alias_draw(rs, nel, c->ppn_U[PPN_IJD] + offj, c->ppn_K[PPN_IJD] + offj);
        int j = map[j_ind];
        int ij_spin = 0, a = -1, b = -1;
        if (j != i) {
            allowed = 1;
            pgen = (PPN_W(c, PPN_ID, 0, i_ind) / c->ppn_tot[PPN_ID][0]) *
                   (PPN_W(c, PPN_IJD, i, j_ind) / c->ppn_tot[PPN_IJD][i]);
            ij_spin = c->orb_ms[i] + c->orb_ms[j];
            pgen = pgen + ((PPN_W(c, PPN_ID, 0, j_ind) / c->ppn_tot[PPN_ID][0]) *
                           (PPN_W(c, PPN_IJD, j, i_ind) / c->ppn_tot[PPN_IJD][j]));
            if (j < i) {
                const int t = j;
                j = i;
                i = t;
            }
        }
        out->e.from[0] = i;
        out->e.from[1] = j;
        int a_ind = -1, isymb = 0, imsb = 0, ij_sym = 0;
        if (allowed) {
            const int half = c->nbasis / 2, imsa = ims_of(c, i);
            const size_t off = (size_t)i * c->ppn_stride[PPN_IAD];
            a_ind = alias_draw(rs, half, c->ppn_U[PPN_IAD] + off, c->ppn_K[PPN_IAD] + off);
            a = 2 * a_ind + (imsa == 0);
            if (tbit(f, a)) allowed = 0;
        }
        if (allowed) {
            ij_sym = cross(c, c->orb_sym[i], c->orb_sym[j]);
            isymb = cross(c, ij_sym, c->orb_sym[a]);
            imsb = ims_of(c, j);
            if (NBSS(imsb, isymb) == 0) allowed = 0;
        }
        if (allowed) {
            const int rb = j * c->nsym + isymb;
            const size_t off = (size_t)rb * c->ppn_stride[PPN_JBD];
            const int b_ind = alias_draw(rs, NBSS(imsb, isymb), c->ppn_U[PPN_JBD] + off, c->ppn_K[PPN_JBD] + off);
            b = SSBF(b_ind, imsb, isymb);
            if (a != b && !tbit(f, b)) {
                const double tot_a = c->ppn_tot[PPN_IAD][i], tot_b = c->ppn_tot[PPN_JBD][rb];
                if (ij_spin == 0) {
                    pgen = pgen * (PPN_W(c, PPN_IAD, i, a_ind) / tot_a * PPN_W(c, PPN_JBD, rb, b_ind) / tot_b);
                } else {
                    const int b_rev = b >> 1;
                    const int isyma = cross(c, ij_sym, isymb), ra = j * c->nsym + isyma;
                    int list[MAXB];
                    const int nl = NBSS(imsb, isyma);
                    for (int q = 0; q < nl; q++) list[q] = SSBF(q, imsb, isyma);
                    const int a_rev = int_lower_bound(list, nl, a);
                    pgen = pgen * (PPN_W(c, PPN_IAD, i, a_ind) / tot_a * PPN_W(c, PPN_JBD, rb, b_ind) / tot_b +
                                   PPN_W(c, PPN_IAD, i, b_rev) / tot_a * PPN_W(c, PPN_JBD, ra, a_rev) /
                                       c->ppn_tot[PPN_JBD][ra]);
                }
                pgen = c->pattempt_double * pgen;
            } else {
                allowed = 0;
            }
        }
        if (allowed) {
            out->e.to[0] = a < b ? a : b;
            out->e.to[1] = a < b ? b : a;
            out->e.perm = perm2(c, f, i, j, out->e.to[0], out->e.to[1]);
            hmatel = sc2_mol_excit(c, i, j, out->e.to[0], out->e.to[1], out->e.perm);
        } else {
            out->e.to[0] = out->e.to[1] = -1;
        }
    }
    out->allowed = allowed;
    if (!allowed) {
        pgen = 1.0;
        hmatel = 0.0;
    }
    *pgen_out = pgen;
    *hmatel_out = hmatel;
}

static void attempt_mol(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int64_t parent,
                        attempt_t *out) {
    memset(out, 0, sizeof(*out));
    out->e.from[0] = out->e.from[1] = out->e.to[0] = out->e.to[1] = -1;
    int gen = c->cfg.excit_gen;
    /* gen_excit_mol_heat_bath_uniform takes its singles from gen_single_excit_mol
     * (heat_bath_uniform) or gen_single_excit_heat_bath_exact (heat_bath_single) */
    const int pp = gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC || gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC ||
                   gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ || gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ;
    int renorm = gen == HGPU_EXCIT_GEN_RENORM || gen == HGPU_EXCIT_GEN_RENORM_SPIN ||
                 gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM || pp;
    double pgen, hmatel;
    if (gen == HGPU_EXCIT_GEN_HEAT_BATH) {
        gen_heat_bath(c, rs, f, d, out, &pgen, &hmatel);
    } else if (gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN) {
        gen_ppn(c, rs, f, d, out, &pgen, &hmatel);
    } else if (gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE && rs_next(rs) < c->pattempt_single) {
        gen_single_heat_bath_exact(c, rs, f, d, out, &pgen, &hmatel);
    } else if (gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE) {
        gen_heat_bath_uniform_double(c, rs, f, d, out, &pgen, &hmatel);
    } else if (rs_next(rs) < c->pattempt_single) {
        int i = -1, a = -1, ok;
        out->e.nexcit = 1;
        if (renorm) ok = choose_ia_mol(c, rs, f, d, &i, &a);
        else ok = find_ia_mol(c, rs, f, d, &i, &a);
        out->allowed = ok;
        out->e.from[0] = i;
        out->e.to[0] = ok ? a : -1;
        if (ok) {
            pgen = c->pattempt_single *
                   (renorm ? calc_pgen_single_mol(c, d, a) : calc_pgen_single_mol_no_renorm(c, a));
            out->e.perm = perm1(c, f, i, a);
            hmatel = sc1_mol_excit(c, d->occ, i, a, out->e.perm);
        } else {
            hmatel = 0.0;
            pgen = 1.0;
        }
    } else if (gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM) {
        gen_heat_bath_uniform_double(c, rs, f, d, out, &pgen, &hmatel);
    } else if (pp) {
        gen_pp_occ_double(c, rs, f, d, out, &pgen, &hmatel);
    } else {
        int i, j, ij_sym, ij_spin, a = -1, b = -1, ok;
        double pgen_ij;
        out->e.nexcit = 2;
        i = j = -1;
        if (c->spin_ij) ok = choose_ij_spin_mol(c, rs, d, &i, &j, &ij_sym, &ij_spin, &pgen_ij);
        else {
            choose_ij_mol(c, rs, d, &i, &j, &ij_sym, &ij_spin, &pgen_ij);
            ok = 1;
        }
        if (ok && renorm) ok = choose_ab_mol(c, rs, f, ij_sym, ij_spin, d, &a, &b);
        else if (ok) ok = find_ab_mol(c, rs, f, ij_sym, ij_spin, &a, &b);
        out->allowed = ok;
        out->e.from[0] = i;
        out->e.from[1] = j;
        if (ok) {
            out->e.to[0] = a;
            out->e.to[1] = b;
            if (renorm)
                pgen = c->pattempt_double * pgen_ij * calc_pgen_double_mol(c, ij_sym, a, b, ij_spin, d);
            else
                pgen = c->pattempt_double * pgen_ij * calc_pgen_double_mol_no_renorm(c, a, b, ij_spin);
            out->e.perm = perm2(c, f, i, j, a, b);
            hmatel = sc2_mol_excit(c, i, j, a, b, out->e.perm);
        } else {
            hmatel = 0.0;
            pgen = 1.0;
        }
    }
    out->pgen = pgen;
    out->hmatel = hmatel;
    /* attempt_to_spawn */
    double pspawn = c->cfg.tau * fabs(hmatel) / pgen;
    pspawn = pspawn * (double)c->real_factor;
    int64_t nspawn = round_spawned(c->cutoff, pspawn, rs);
    if (nspawn > 0) nspawn = child_sign(hmatel, parent, nspawn);
    out->nspawn = nspawn;
    /* spawn_rdm: attempt_to_spawn with tau = 1 and hmatel = -1 for the replica
     * sampling of the 2-RDM, after the spawn itself (src/spawning.F90:664-671) */
    out->nspawn_rdm = 0;
    if (c->rdm_on && out->allowed) {
        double prdm = 1.0 * fabs(-1.0) / pgen;
        prdm = prdm * (double)c->real_factor;
        int64_t nr = round_spawned(c->cutoff, prdm, rs);
        if (nr > 0) nr = child_sign(-1.0, parent, nr);
        out->nspawn_rdm = nr;
    }
}

static void decode_any(const oracle_ctx *c, const uint64_t *f, det_info *d) {
    if (c->kind == HGPU_SYS_HUB_K) decode_hub_k(c, f, d);
    else decode_mol(c, f, d);
}

static void attempt(const oracle_ctx *c, rstream *rs, const uint64_t *f, const det_info *d, int64_t parent,
                    attempt_t *out, int complete) {
    if (c->kind == HGPU_SYS_HUB_K) attempt_hub_k(c, rs, f, d, parent, out, complete);
    else attempt_mol(c, rs, f, d, parent, out);
}

static double sc0(const oracle_ctx *c, const uint64_t *f) { return fx_val(c, fx_energy(c, f)); }

/* dat(1) = K_ii = <D_i|H|D_i> - E_HF (src/annihilation.f90:855), from the exact difference. */
static double kii_of(const oracle_ctx *c, const uint64_t *f) { return fx_val(c, fx_energy(c, f) - c->fx_E0); }

/* get_hmatel_hub_k (src/hamiltonian_hub_k.f90:12-89) / get_hmatel_mol
 * (src/hamiltonian_molecular.f90:12-65). */
static double hmatel_any(const oracle_ctx *c, const uint64_t *f1, const uint64_t *f2) {
    excit_t e = get_excitation(c, f1, f2);
    if (e.nexcit == 0) return sc0(c, f1);
    if (c->kind == HGPU_SYS_HUB_K) {
        if (e.nexcit != 2) return 0.0;
        double h = two_e_int_hub_k(c, e.from[0], e.from[1], e.to[0], e.to[1]);
        return e.perm ? -h : h;
    }
    if (e.nexcit == 1) {
        if (c->orb_sym[e.from[0]] != c->orb_sym[e.to[0]] || c->orb_ms[e.from[0]] != c->orb_ms[e.to[0]]) return 0.0;
        int occ[MAXB];
        decode(c, f1, occ);
        return sc1_mol_excit(c, occ, e.from[0], e.to[0], e.perm);
    }
    if (e.nexcit == 2) {
        int i = e.from[0], j = e.from[1], a = e.to[0], b = e.to[1];
        if (cross(c, c->orb_sym[i], c->orb_sym[j]) != cross(c, c->orb_sym[a], c->orb_sym[b])) return 0.0;
        /* slater_condon2_mol: get_two_body_int_mol_real checks the spins */
        double h = 0.0, x = 0.0;
        if (c->orb_ms[i] == c->orb_ms[a] && c->orb_ms[j] == c->orb_ms[b]) h = v2_get(c, i, j, a, b);
        if (c->orb_ms[i] == c->orb_ms[b] && c->orb_ms[j] == c->orb_ms[a]) x = v2_get(c, i, j, b, a);
        h = h - x;
        return e.perm ? -h : h;
    }
    return 0.0;
}

/* ------------------------------------------------------------------------- */
/* Per-determinant steps                                                      */
/* ------------------------------------------------------------------------- */

/* decide_nattempts (src/qmc_common.F90:379-406). */
static int64_t decide_nattempts(rstream *rs, double population) {
    double ap = fabs(population);
    int64_t n = (int64_t)ap;
    double pextra = ap - (double)n;
    if (fabs(pextra) > DEPSILON) {
        if (pextra > rs_next(rs)) n = n + 1;
    }
    return n;
}

/* stochastic_death (src/death.f90:11-130) with quasi-Newton and Chebyshev
 * off: weight = quasi_newton_pop_control = dmqmc_factor = 1 and p_d reduces
 * to tau*(K_ii - S). */
static int64_t stochastic_death(const oracle_ctx *c, rstream *rs, double Kii, double shift, int64_t *population) {
    double pd = c->cfg.tau * (Kii - shift);
    pd = pd * fabs((double)*population);
    int64_t kill = (int64_t)pd;
    pd = pd - (double)kill;
    double r = rs_next(rs);
    if (fabs(pd) > r) {
        if (pd > 0.0) kill = kill + 1;
        else kill = kill - 1;
    }
    if (*population < 0) *population = *population + kill;
    else *population = *population - kill;
    return kill < 0 ? -kill : kill;
}

/* set_parent_flag (src/ifciqmc.f90:14-57): bit s set if NOT an initiator in
 * space s.  With quadrature_initiator (HANDE's default) and an even number of
 * spaces, each pair of spaces is tested together on N_1^2 + N_2^2. */
static int64_t parent_flag(const oracle_ctx *c, const double *real_pop) {
    int64_t flag = 0;
    if (c->cfg.quadrature_initiator && c->R % 2 == 0) {
        for (int s = 0; s < c->R; s += 2) {
            const double magnitude = real_pop[s] * real_pop[s] + real_pop[s + 1] * real_pop[s + 1];
            if (!(magnitude > c->cfg.initiator_pop * c->cfg.initiator_pop)) flag |= (int64_t)3 << s;
        }
        return flag;
    }
    for (int s = 0; s < c->R; s++)
        if (!(fabs(real_pop[s]) > c->cfg.initiator_pop)) flag |= (int64_t)1 << s;
    return flag;
}

/* update_proj_energy_hub_k / update_proj_energy_mol
 * (src/energy_evaluation.F90:795-849, :906-985). */
static void update_proj_energy(oracle_ctx *c, const uint64_t *f, const det_info *d, const excit_t *ex, double pop,
                               int s) {
    excit_t e = *ex;
    if (e.nexcit == 0) {
        c->acc_d0[s] += pop;
        return;
    }
    if (c->kind == HGPU_SYS_HUB_K) {
        if (e.nexcit == 2) {
            double h = two_e_int_hub_k(c, e.from[0], e.from[1], e.to[0], e.to[1]);
            if (e.perm) h = -h;
            c->acc_proj[s] += h * pop;
        }
        return;
    }
    if (e.nexcit == 1) {
        if (c->orb_ms[e.from[0]] == c->orb_ms[e.to[0]] && c->orb_sym[e.from[0]] == c->orb_sym[e.to[0]]) {
            double h = sc1_mol_excit(c, d->occ, e.from[0], e.to[0], e.perm);
            c->acc_proj[s] += h * pop;
        }
    } else if (e.nexcit == 2) {
        int i = e.from[0], j = e.from[1], a = e.to[0], b = e.to[1];
        if (c->orb_ms[i] + c->orb_ms[j] == c->orb_ms[a] + c->orb_ms[b]) {
            if (cross(c, c->orb_sym[i], c->orb_sym[j]) == cross(c, c->orb_sym[a], c->orb_sym[b])) {
                double h = sc2_mol_excit(c, i, j, a, b, e.perm);
                c->acc_proj[s] += h * pop;
            }
        }
    }
    (void)f;
}

/* ------------------------------------------------------------------------- */
/* Annihilation                                                               */
/* ------------------------------------------------------------------------- */

static _Thread_local const oracle_ctx *g_sort_ctx; /* per thread: the partitioned driver sorts on many */

static int cmp_spawn(const void *x, const void *y) {
    const oracle_ctx *c = g_sort_ctx;
    int64_t i = *(const int64_t *)x, j = *(const int64_t *)y;
    int r = det_cmp(&c->sdets[i * c->nw], &c->sdets[j * c->nw], c->nw);
    if (r != 0) return r == 1 ? -1 : 1;
    if (c->sord[i] < c->sord[j]) return -1;
    if (c->sord[i] > c->sord[j]) return 1;
    return 0;
}

/* Sort the spawned list by determinant; entries on the same determinant keep
 * their generation order (the reference's qsort, src/sort.f90:213-394, leaves
 * that order unspecified; a stable order makes the oracle deterministic). */
static void sort_spawns(oracle_ctx *c) {
    int64_t n = c->sn;
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) perm[i] = i;
    g_sort_ctx = c;
    qsort(perm, (size_t)n, sizeof(int64_t), cmp_spawn);
    uint64_t *d2 = (uint64_t *)malloc(sizeof(uint64_t) * c->nw * (n > 0 ? n : 1));
    int64_t *p2 = (int64_t *)malloc(sizeof(int64_t) * c->R * (n > 0 ? n : 1));
    int64_t *f2 = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    int64_t *o2 = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    for (int64_t k = 0; k < n; k++) {
        int64_t i = perm[k];
        memcpy(&d2[k * c->nw], &c->sdets[i * c->nw], sizeof(uint64_t) * c->nw);
        memcpy(&p2[k * c->R], &c->spops[i * c->R], sizeof(int64_t) * c->R);
        f2[k] = c->sflag[i];
        o2[k] = c->sord[i];
    }
    memcpy(c->sdets, d2, sizeof(uint64_t) * c->nw * n);
    memcpy(c->spops, p2, sizeof(int64_t) * c->R * n);
    memcpy(c->sflag, f2, sizeof(int64_t) * n);
    memcpy(c->sord, o2, sizeof(int64_t) * n);
    free(perm); free(d2); free(p2); free(f2); free(o2);
}

static void scopy(oracle_ctx *c, int64_t dst, int64_t src) {
    if (dst == src) return;
    memcpy(&c->sdets[dst * c->nw], &c->sdets[src * c->nw], sizeof(uint64_t) * c->nw);
    memcpy(&c->spops[dst * c->R], &c->spops[src * c->R], sizeof(int64_t) * c->R);
    c->sflag[dst] = c->sflag[src];
    c->sord[dst] = c->sord[src];
    c->suid[dst] = c->suid[src];
}

static int all_zero(const int64_t *p, int R) {
    for (int s = 0; s < R; s++)
        if (p[s] != 0) return 0;
    return 1;
}

/* annihilate_spawn_t (src/spawn_data.F90:859-935). */
static void annihilate_spawn_t(oracle_ctx *c) {
    int64_t ub = c->sn; /* number of entries (1-based upper bound) */
    if (ub == 0) return;
    int64_t islot = 0, k = 0; /* 0-based */
    for (;;) {
        scopy(c, islot, k);
        int done = 0;
        for (;;) {
            k++;
            if (k > ub - 1) { done = 1; break; }
            if (det_cmp(&c->sdets[k * c->nw], &c->sdets[islot * c->nw], c->nw) == 0) {
                for (int s = 0; s < c->R; s++) c->spops[islot * c->R + s] += c->spops[k * c->R + s];
            } else {
                break;
            }
        }
        if (done) break;
        if (islot == ub - 1) break;
        if (!all_zero(&c->spops[islot * c->R], c->R)) islot++;
    }
    if (all_zero(&c->spops[islot * c->R], c->R)) islot--;
    c->sn = islot + 1;
}

/* Fortran sign(1, int(x)) for an int_s population: int() converts to default
 * (32-bit) integer, which keeps the low 32 bits. */
static inline int sign1_int32(int64_t x) {
    int32_t v = (int32_t)(uint32_t)(uint64_t)x;
    return v >= 0 ? 1 : -1;
}

/* annihilate_spawn_t_initiator (src/spawn_data.F90:937-1101). */
static void annihilate_spawn_t_initiator(oracle_ctx *c) {
    int64_t ub = c->sn;
    if (ub == 0) return;
    int64_t islot = 0, k = 0;
    int64_t events[2], ipop[2];
    for (;;) {
        scopy(c, islot, k);
        for (int s = 0; s < c->R; s++) {
            if (!((c->sflag[k] >> s) & 1)) {
                ipop[s] = c->spops[k * c->R + s];
                events[s] = 0;
            } else {
                ipop[s] = 0;
                events[s] = sign1_int32(c->spops[k * c->R + s]);
            }
        }
        for (;;) {
            k++;
            int same = k <= ub - 1;
            if (same) same = det_cmp(&c->sdets[k * c->nw], &c->sdets[islot * c->nw], c->nw) == 0;
            if (same) {
                for (int s = 0; s < c->R; s++) {
                    int64_t v = c->spops[k * c->R + s];
                    if (!((c->sflag[k] >> s) & 1)) ipop[s] += v;
                    else if (v < 0) events[s] -= 1;
                    else if (v > 0) events[s] += 1;
                }
                for (int s = 0; s < c->R; s++) c->spops[islot * c->R + s] += c->spops[k * c->R + s];
            } else {
                int64_t flag = 0;
                for (int s = 0; s < c->R; s++) {
                    int64_t tot = c->spops[islot * c->R + s];
                    if (ipop[s] != 0 && (tot >= 0 ? 1 : -1) == (ipop[s] >= 0 ? 1 : -1)) {
                        /* keep: sign-coherent with the initiator-sourced particles */
                    } else if (llabs(events[s]) > 1) {
                        /* keep: multiple coherent events */
                    } else {
                        flag += (int64_t)1 << s;
                    }
                }
                c->sflag[islot] = flag;
                break;
            }
        }
        if (islot == ub - 1 || k > ub - 1) break;
        if (!all_zero(&c->spops[islot * c->R], c->R)) islot++;
    }
    if (all_zero(&c->spops[islot * c->R], c->R)) islot--;
    c->sn = islot + 1;
}

/* binary_search_i0_list (src/search.f90:47-170), 0-based, [istart, iend]. */
static int64_t bsearch_main(const oracle_ctx *c, const uint64_t *item, int64_t istart, int64_t iend, int *hit) {
    int64_t pos;
    *hit = 0;
    if (istart > iend) return istart;
    int64_t lo = istart, hi = iend;
    pos = lo;
    while (hi != lo) {
        pos = (hi + lo) / 2;
        int cmp = det_cmp(&c->dets[pos * c->nw], item, c->nw);
        if (cmp == 0) { *hit = 1; return pos; }
        if (cmp == 1) lo = pos + 1;
        else hi = pos;
    }
    int cmp = det_cmp(&c->dets[hi * c->nw], item, c->nw);
    if (cmp == 0) { *hit = 1; return hi; }
    if (cmp == 1) return hi + 1;
    return hi;
}

/* annihilate_main_list (src/annihilation.f90:294-370) and
 * annihilate_main_list_initiator (:372-486). */
static void annihilate_main_list(oracle_ctx *c, int initiator) {
    int64_t nann = 0, istart = 0, iend = c->n - 1;
    for (int64_t i = 0; i < c->sn; i++) {
        int hit;
        int64_t pos = bsearch_main(c, &c->sdets[i * c->nw], istart, iend, &hit);
        if (hit) {
            for (int s = 0; s < c->R; s++) {
                int64_t sp = c->spops[i * c->R + s];
                if (!initiator) {
                    c->pops[pos * c->R + s] += sp;
                } else if (c->pops[pos * c->R + s] != 0) {
                    c->pops[pos * c->R + s] += sp;
                } else if (!((c->sflag[i] >> s) & 1)) {
                    c->pops[pos * c->R + s] = sp;
                }
            }
            nann++;
            istart = pos + 1;
        } else if (!initiator) {
            scopy(c, i - nann, i);
        } else {
            int discard = 1;
            int64_t keep[2];
            for (int s = 0; s < c->R; s++) {
                if ((c->sflag[i] >> s) & 1) keep[s] = 0;
                else { keep[s] = c->spops[i * c->R + s]; discard = 0; }
            }
            if (discard) {
                nann++;
            } else {
                scopy(c, i - nann, i);
                for (int s = 0; s < c->R; s++) c->spops[(i - nann) * c->R + s] = keep[s];
            }
        }
    }
    c->sn -= nann;
}

/* stochastic_round_int_64 (src/stoch_utils.f90:51-85) for one entry. */
static void stochastic_round_pops(const oracle_ctx *c, int64_t *pop, int purpose, int64_t idx) {
    for (int s = 0; s < c->R; s++) {
        int64_t p = pop[s];
        if (llabs(p) < c->real_factor && p != 0) {
            rstream rs;
            rs_init(&rs, (uint64_t)c->cfg.seed, purpose, s, (uint64_t)idx, 0, (uint64_t)c->iter);
            double r = rs_next(&rs) * (double)c->real_factor;
            if ((double)llabs(p) > r) pop[s] = isign64(c->real_factor, p);
            else pop[s] = 0;
        }
    }
}

/* check_if_determ (src/semi_stoch.F90:795-824): the index of f in the
 * deterministic space, or -1. */
static int64_t ss_find(const oracle_ctx *c, const uint64_t *f) {
    int64_t lo = 0, hi = c->nd;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        int cmp = det_cmp(&c->ddets[mid * c->nw], f, c->nw);
        if (cmp == 0) return mid;
        if (cmp == 1) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

/* remove_unoccupied_dets (src/annihilation.f90:537-598). */
static void remove_unoccupied_dets(oracle_ctx *c) {
    int64_t nzero = 0;
    for (int64_t i = 0; i < c->n; i++) {
        const int determ = c->ss_on && ss_find(c, &c->dets[i * c->nw]) >= 0;
        if (c->cfg.real_amplitudes && !determ) stochastic_round_pops(c, &c->pops[i * c->R], P_ROUND_MAIN, i);
        if (all_zero(&c->pops[i * c->R], c->R) && !determ) {
            nzero++;
        } else if (nzero > 0) {
            int64_t k = i - nzero;
            memcpy(&c->dets[k * c->nw], &c->dets[i * c->nw], sizeof(uint64_t) * c->nw);
            memcpy(&c->pops[k * c->R], &c->pops[i * c->R], sizeof(int64_t) * c->R);
            c->kii[k] = c->kii[i];
        }
    }
    c->n -= nzero;
}

/* round_low_population_spawns (src/annihilation.f90:600-675); the rounding
 * stream of an entry is keyed by the position of its determinant's first entry
 * in the sorted spawned list (the number of spawned entries below it). */
static void round_low_population_spawns(oracle_ctx *c) {
    int64_t nrem = 0;
    for (int64_t i = 0; i < c->sn; i++) {
        stochastic_round_pops(c, &c->spops[i * c->R], P_ROUND_SPAWN, c->suid[i]);
        if (all_zero(&c->spops[i * c->R], c->R)) nrem++;
        else scopy(c, i - nrem, i);
    }
    c->sn -= nrem;
}

/* insert_new_walkers / insert_new_walker (src/annihilation.f90:677-901): a
 * merge of two sorted lists, with dat(1) = sc0 - H00 for new determinants. */
static void insert_new_walkers(oracle_ctx *c) {
    if (c->n + c->sn > c->cap) {
        c->error_flags |= HGPU_FLAG_MAIN_OVERFLOW;
        return;
    }
    int64_t n = c->n, m = c->sn, tot = n + m;
    uint64_t *nd = (uint64_t *)malloc(sizeof(uint64_t) * c->nw * (tot > 0 ? tot : 1));
    int64_t *np = (int64_t *)malloc(sizeof(int64_t) * c->R * (tot > 0 ? tot : 1));
    double *nk = (double *)malloc(sizeof(double) * (tot > 0 ? tot : 1));
    int64_t i = 0, j = 0, k = 0;
    while (i < n || j < m) {
        int take_spawn;
        if (i >= n) take_spawn = 1;
        else if (j >= m) take_spawn = 0;
        else take_spawn = det_cmp(&c->sdets[j * c->nw], &c->dets[i * c->nw], c->nw) == 1;
        if (take_spawn) {
            memcpy(&nd[k * c->nw], &c->sdets[j * c->nw], sizeof(uint64_t) * c->nw);
            memcpy(&np[k * c->R], &c->spops[j * c->R], sizeof(int64_t) * c->R);
            nk[k] = kii_of(c, &c->sdets[j * c->nw]);
            j++;
        } else {
            memcpy(&nd[k * c->nw], &c->dets[i * c->nw], sizeof(uint64_t) * c->nw);
            memcpy(&np[k * c->R], &c->pops[i * c->R], sizeof(int64_t) * c->R);
            nk[k] = c->kii[i];
            i++;
        }
        k++;
    }
    memcpy(c->dets, nd, sizeof(uint64_t) * c->nw * tot);
    memcpy(c->pops, np, sizeof(int64_t) * c->R * tot);
    memcpy(c->kii, nk, sizeof(double) * tot);
    c->n = tot;
    free(nd); free(np); free(nk);
}

/* direct_annihilation (src/annihilation.f90:9-80) with
 * annihilate_main_list_wrapper (:214-292). */
static void direct_annihilation(oracle_ctx *c) {
    int initiator = c->cfg.initiator_approx;
    if (c->sn > 0) {
        sort_spawns(c);
        /* the rounding stream of a new determinant is keyed by the sorted
         * position of its first spawned entry, which the self-annihilation
         * carries along with the entry */
        for (int64_t i = 0; i < c->sn; i++) c->suid[i] = i;
        if (initiator) annihilate_spawn_t_initiator(c);
        else annihilate_spawn_t(c);
    }
    if (c->sn >= 1) {
        annihilate_main_list(c, initiator);
        remove_unoccupied_dets(c);
        if (c->cfg.real_amplitudes) round_low_population_spawns(c);
        insert_new_walkers(c);
    } else {
        remove_unoccupied_dets(c);
    }
}

/* ------------------------------------------------------------------------- */
/* The Monte Carlo cycle (src/fciqmc.f90:293-413)                             */
/* ------------------------------------------------------------------------- */

static void add_spawn(oracle_ctx *c, const uint64_t *f, int s, int64_t nspawn, int64_t flag, int64_t ord) {
    if (c->sn >= c->scap) {
        c->error_flags |= HGPU_FLAG_SPAWN_OVERFLOW;
        return;
    }
    int64_t k = c->sn++;
    memcpy(&c->sdets[k * c->nw], f, sizeof(uint64_t) * c->nw);
    for (int t = 0; t < c->R; t++) c->spops[k * c->R + t] = 0;
    c->spops[k * c->R + s] = nspawn;
    c->sflag[k] = flag;
    c->sord[k] = ord;
}

static int64_t abs_pop_sum(const oracle_ctx *c, int s) {
    int64_t t = 0;
    for (int64_t i = 0; i < c->n; i++) t += llabs(c->pops[i * c->R + s]);
    return t;
}

static double nparticles(const oracle_ctx *c, int s) {
    return (double)abs_pop_sum(c, s) / (double)c->real_factor;
}

/* ------------------------------------------------------------------------- */
/* Replica 2-RDM (src/replica_rdm.F90)                                        */
/* ------------------------------------------------------------------------- */

/* tri_ind_distinct_reorder (lib/local/utils.F90:579-611), 0-based orbitals and index. */
static inline int64_t tri_pair(int p, int q) {
    int64_t hi = p > q ? p : q, lo = p > q ? q : p;
    return hi * (hi - 1) / 2 + lo;
}

/* create_spawned_particle_replica_rdm (src/spawning.F90:2019-2061). */
static void add_rdm_spawn(oracle_ctx *c, const uint64_t *parent, const uint64_t *child, int s, int64_t n) {
    if (c->rsn >= c->scap) {
        c->error_flags |= HGPU_FLAG_SPAWN_OVERFLOW;
        return;
    }
    int64_t k = c->rsn++;
    memcpy(&c->rsdets[k * 2 * c->nw], parent, sizeof(uint64_t) * c->nw);
    memcpy(&c->rsdets[k * 2 * c->nw + c->nw], child, sizeof(uint64_t) * c->nw);
    for (int t = 0; t < c->R; t++) c->rspops[k * c->R + t] = 0;
    c->rspops[k * c->R + s] = n;
}

/* update_rdm (src/replica_rdm.F90:12-82): one pair of determinants. */
static void update_rdm(oracle_ctx *c, const uint64_t *f1, const uint64_t *f2, const int *occ1, double pop1,
                       double pop2, double prob) {
    excit_t e = get_excitation(c, f1, f2);
    double matel = pop1 * pop2 / prob;
    if (e.perm) matel = -matel;
    const int64_t np = c->npairs;
    if (e.nexcit == 0) {
        for (int i = 0; i < c->nel; i++)
            for (int j = i + 1; j < c->nel; j++) {
                int64_t ind = tri_pair(occ1[i], occ1[j]);
                c->rdm[ind * np + ind] = c->rdm[ind * np + ind] + matel;
            }
    } else if (e.nexcit == 1) {
        int p = e.to[0], q = e.from[0];
        for (int i = 0; i < c->nel; i++) {
            int orb = occ1[i];
            if (orb == q) continue;
            if (orb < p && orb < q) {
                int64_t k = tri_pair(orb, p) * np + tri_pair(orb, q);
                c->rdm[k] = c->rdm[k] + matel;
            } else if (orb > p && orb > q) {
                int64_t k = tri_pair(orb, p) * np + tri_pair(q, orb);
                c->rdm[k] = c->rdm[k] + matel;
            } else {
                int64_t k = tri_pair(p, orb) * np + tri_pair(orb, q);
                c->rdm[k] = c->rdm[k] - matel;
            }
        }
    } else if (e.nexcit == 2) {
        int64_t k = tri_pair(e.to[0], e.to[1]) * np + tri_pair(e.from[0], e.from[1]);
        c->rdm[k] = c->rdm[k] + matel;
    }
}

static _Thread_local const oracle_ctx *g_rdm_ctx;

static int cmp_rdm_spawn(const void *x, const void *y) {
    const oracle_ctx *c = g_rdm_ctx;
    int64_t i = *(const int64_t *)x, j = *(const int64_t *)y;
    int r = det_cmp(&c->rsdets[i * 2 * c->nw], &c->rsdets[j * 2 * c->nw], 2 * c->nw);
    if (r != 0) return r == 1 ? -1 : 1;
    return i < j ? -1 : (i > j ? 1 : 0);
}

/* update_rdm_from_spawns (src/replica_rdm.F90:84-159): the RDM spawns sorted
 * by (parent, child) words and annihilated (annihilate_wrapper_spawn_t), each
 * found in the main list through its child, then the diagonal of every
 * occupied determinant. */
static void update_rdm_from_spawns(oracle_ctx *c) {
    const int nw = c->nw, R = c->R;
    int64_t n = c->rsn;
    if (n > 0) {
        int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * n);
        uint64_t *d2 = (uint64_t *)malloc(sizeof(uint64_t) * 2 * nw * n);
        int64_t *p2 = (int64_t *)malloc(sizeof(int64_t) * R * n);
        for (int64_t i = 0; i < n; i++) perm[i] = i;
        g_rdm_ctx = c;
        qsort(perm, (size_t)n, sizeof(int64_t), cmp_rdm_spawn);
        /* sort, then sum equal keys and drop the ones that sum to zero */
        int64_t m = -1;
        for (int64_t k = 0; k < n; k++) {
            const uint64_t *key = &c->rsdets[perm[k] * 2 * nw];
            if (m >= 0 && det_cmp(&d2[m * 2 * nw], key, 2 * nw) == 0) {
                for (int t = 0; t < R; t++) p2[m * R + t] += c->rspops[perm[k] * R + t];
                continue;
            }
            if (m >= 0 && all_zero(&p2[m * R], R)) m--;
            m++;
            memcpy(&d2[m * 2 * nw], key, sizeof(uint64_t) * 2 * nw);
            for (int t = 0; t < R; t++) p2[m * R + t] = c->rspops[perm[k] * R + t];
        }
        if (m >= 0 && all_zero(&p2[m * R], R)) m--;
        int64_t istart = 0, iend = c->n - 1;
        int occ[MAXEL];
        for (int64_t k = 0; k <= m; k++) {
            const uint64_t *fp = &d2[k * 2 * nw], *fc = &d2[k * 2 * nw + nw];
            int hit;
            int64_t pos = bsearch_main(c, fc, istart, iend, &hit);
            if (hit) {
                decode(c, fc, occ);
                for (int sp = 0; sp < 2; sp++)
                    update_rdm(c, fc, fp, occ, (double)c->pops[pos * R + sp] / (double)c->real_factor,
                               (double)p2[k * R + (1 - sp)] / (double)c->real_factor, 2.0);
            }
            istart = pos;
        }
        free(perm); free(d2); free(p2);
    }
    int occ[MAXEL];
    for (int64_t i = 0; i < c->n; i++) {
        const uint64_t *f = &c->dets[i * nw];
        decode(c, f, occ);
        update_rdm(c, f, f, occ, (double)c->pops[i * R + 0] / (double)c->real_factor,
                   (double)c->pops[i * R + 1] / (double)c->real_factor, 1.0);
    }
    c->rsn = 0;
}

/* get_two_e_int_mol (src/hamiltonian_molecular.f90:579-597): <ij||ab> with the
 * spin and symmetry checks of get_two_body_int_mol. */
static double two_e_int(const oracle_ctx *c, int i, int j, int a, int b) {
    int sym_ok = ((c->orb_sym[i] ^ c->orb_sym[j] ^ c->orb_sym[a] ^ c->orb_sym[b]) & (c->nsym - 1)) == 0;
    double x = 0.0, y = 0.0;
    if (sym_ok && c->orb_ms[i] == c->orb_ms[a] && c->orb_ms[j] == c->orb_ms[b]) x = v2_get(c, i, j, a, b);
    if (sym_ok && c->orb_ms[i] == c->orb_ms[b] && c->orb_ms[j] == c->orb_ms[a]) y = v2_get(c, i, j, b, a);
    return x - y;
}

/* get_one_e_int_mol (src/hamiltonian_molecular.f90:599-617). */
static double one_e_int(const oracle_ctx *c, int i, int j) {
    if (c->orb_sym[i] != c->orb_sym[j] || c->orb_ms[i] != c->orb_ms[j]) return 0.0;
    return h1_get(c, i, j);
}

/* orbs_from_index (lib/local/utils.F90:613-628), 0-based index and orbitals. */
static void orbs_of_pair(int64_t ind, int *p, int *q) {
    int64_t i1 = ind + 1;
    int qq = (int)(1.50 + sqrt((double)(2 * i1) - 1.750));
    int pp = (int)(i1 - ((int64_t)(qq - 1) * (qq - 2)) / 2);
    *p = pp - 1;
    *q = qq - 1;
}

/* calc_rdm_energy (src/replica_rdm.F90:215-264). */
static void calc_rdm_energy(oracle_ctx *c, double *energy, double *trace) {
    const int64_t np = c->npairs;
    double tr = 0.0, e = 0.0;
    for (int64_t i = 0; i < np; i++) tr = tr + c->rdm[i * np + i];
    const double nm1 = (double)(c->nel - 1);
    for (int64_t i = 0; i < np; i++) {
        int a, b;
        orbs_of_pair(i, &a, &b);
        for (int64_t j = 0; j < np; j++) {
            double r = c->rdm[i * np + j];
            if (fabs(r) < DEPSILON) continue;
            int cc, d;
            orbs_of_pair(j, &cc, &d);
            e = e + r * two_e_int(c, a, b, cc, d);
            if (a == cc) e = e + r * one_e_int(c, b, d) / nm1;
            if (b == d) e = e + r * one_e_int(c, a, cc) / nm1;
            if (a == d) e = e - r * one_e_int(c, b, cc) / nm1;
            if (b == cc) e = e - r * one_e_int(c, a, d) / nm1;
        }
    }
    e = e * (double)c->nel * (double)(c->nel - 1) * 0.5;
    e = e + (c->ecore - c->H00) * tr;
    *energy = e;
    *trace = tr;
}

/* ------------------------------------------------------------------------- */
/* Semi-stochastic projection (src/semi_stoch.F90): 'high' space, separate    */
/* annihilation                                                               */
/* ------------------------------------------------------------------------- */

static void ss_free(oracle_ctx *c) {
    free(c->ddets); free(c->dcol_ptr); free(c->dcol_i); free(c->dcol_h);
    free(c->dvec); free(c->dy); free(c->dind);
    c->ddets = NULL; c->dcol_ptr = c->dcol_i = c->dind = NULL; c->dcol_h = c->dvec = c->dy = NULL;
    c->nd = 0;
    c->ss_on = 0;
}

/* init_semi_stoch_t (src/semi_stoch.F90:134-377) for a 'ci' space (ci_space)
 * or a 'high' space:
 * find_most_populated_dets (:1318-1385, the target_size entries of largest
 * sum over spaces of |population|, scanning the main list in order and
 * replacing the first smallest), sorted; add_determ_dets_to_psip_list
 * (:728-793, absent ones enter with zero population); create_determ_hamil
 * (:533-685, |H| > depsilon kept; diagonal K_jj, the main list's exact
 * difference). */
typedef struct {
    uint64_t *d;
    int64_t n, cap;
} detlist_t;

/* The symmetry change of a 'ci' determinant's holes and particles so far, with
 * spin orbital p added as a hole or a particle: molecular irreps combine by XOR
 * (identity 0); Hubbard crystal momenta by sym_table, a hole adding -k and a
 * particle +k (identity the Gamma point). */
static int ci_sym(const oracle_ctx *c, int sym, int p, int hole) {
    if (c->kind != HGPU_SYS_HUB_K) return sym ^ c->orb_sym[p];
    const int k = c->orb_sym[p];
    return c->sym_table[sym * c->nk + (hole ? c->inv_sym[k] : k)];
}

static int ci_sym_identity(const oracle_ctx *c) {
    return c->kind == HGPU_SYS_HUB_K ? c->sym_table[0 * c->nk + c->inv_sym[0]] : 0;
}

/* Particles of a 'ci' determinant: k more virtual orbitals from position v on,
 * whose alpha count and symmetry change must come to na and the identity. */
static void ci_particles(const oracle_ctx *c, const int *virt, int nv, int v, int k, int na, int sym,
                         uint64_t *f, detlist_t *out) {
    if (k == 0) {
        if (na != 0 || sym != ci_sym_identity(c)) return;
        if (out->n == out->cap) {
            out->cap = out->cap ? 2 * out->cap : 64;
            out->d = (uint64_t *)realloc(out->d, sizeof(uint64_t) * c->nw * out->cap);
        }
        memcpy(&out->d[out->n * c->nw], f, sizeof(uint64_t) * c->nw);
        out->n++;
        return;
    }
    for (int q = v; q <= nv - k; q++) {
        const int p = virt[q], a = c->orb_ms[p] > 0;
        if (na - a < 0) continue;
        f[p >> 6] |= (uint64_t)1 << (p & 63);
        ci_particles(c, virt, nv, q + 1, k - 1, na - a, ci_sym(c, sym, p, 0), f, out);
        f[p >> 6] &= ~((uint64_t)1 << (p & 63));
    }
}

/* Holes of a 'ci' determinant: k more occupied orbitals from position o on. */
static void ci_holes(const oracle_ctx *c, const int *occ, int no, const int *virt, int nv, int o, int k, int kk,
                     int na, int sym, uint64_t *f, detlist_t *out) {
    if (k == 0) {
        ci_particles(c, virt, nv, 0, kk, na, sym, f, out);
        return;
    }
    for (int q = o; q <= no - k; q++) {
        const int p = occ[q];
        f[p >> 6] &= ~((uint64_t)1 << (p & 63));
        ci_holes(c, occ, no, virt, nv, q + 1, k - 1, kk, na + (c->orb_ms[p] > 0), ci_sym(c, sym, p, 1), f, out);
        f[p >> 6] |= (uint64_t)1 << (p & 63);
    }
}

/* create_ci_determ_space (src/semi_stoch.F90:1763-1805) with the calculation's
 * reference: every determinant of its spin and symmetry within ci_level
 * excitations of it (enumerate_determinants restricted to ex_level). */
static detlist_t ci_space(const oracle_ctx *c) {
    detlist_t out = {NULL, 0, 0};
    int occ[MAXEL], virt[MAXB], no = 0, nv = 0;
    for (int p = 0; p < c->nbasis; p++) {
        if (tbit(c->f0, p)) occ[no++] = p;
        else virt[nv++] = p;
    }
    uint64_t f[MAXW];
    memcpy(f, c->f0, sizeof(f));
    for (int k = 0; k <= c->cfg.semi_stoch_ci_level && k <= no && k <= nv; k++)
        ci_holes(c, occ, no, virt, nv, 0, k, k, 0, ci_sym_identity(c), f, &out);
    return out;
}

static void ss_init(oracle_ctx *c) {
    ss_free(c);
    const int nw = c->nw, R = c->R;
    if (c->cfg.semi_stoch_space == 4) {
        detlist_t L = ci_space(c);
        c->nd = L.n;
        c->ddets = L.d;
    }
    int64_t K = c->cfg.semi_stoch_space == 4 ? c->nd : (c->cfg.semi_stoch_size < c->n ? c->cfg.semi_stoch_size : c->n);
    if (K < 1) return;
    uint64_t *sel = c->cfg.semi_stoch_space == 4 ? c->ddets : (uint64_t *)malloc(sizeof(uint64_t) * nw * K);
    if (c->cfg.semi_stoch_space == 1) {
        int64_t *pop = (int64_t *)malloc(sizeof(int64_t) * K);
        for (int64_t i = 0; i < K; i++) {
            memcpy(&sel[i * nw], &c->dets[i * nw], sizeof(uint64_t) * nw);
            int64_t p = 0;
            for (int s = 0; s < R; s++) p += llabs(c->pops[i * R + s]);
            pop[i] = p;
        }
        int64_t min_pop = pop[0], min_ind = 0;
        for (int64_t i = 1; i < K; i++)
            if (pop[i] < min_pop) { min_pop = pop[i]; min_ind = i; }
        for (int64_t i = K; i < c->n; i++) {
            int64_t p = 0;
            for (int s = 0; s < R; s++) p += llabs(c->pops[i * R + s]);
            if (p > min_pop) {
                memcpy(&sel[min_ind * nw], &c->dets[i * nw], sizeof(uint64_t) * nw);
                pop[min_ind] = p;
                min_pop = pop[0];
                min_ind = 0;
                for (int64_t j = 1; j < K; j++)
                    if (pop[j] < min_pop) { min_pop = pop[j]; min_ind = j; }
            }
        }
        free(pop);
    }
    /* qsort into the main list's order (insertion sort: small spaces) */
    for (int64_t i = 1; i < K; i++) {
        uint64_t t[MAXW];
        memcpy(t, &sel[i * nw], sizeof(uint64_t) * nw);
        int64_t j = i - 1;
        while (j >= 0 && det_cmp(t, &sel[j * nw], nw) == 1) {
            memcpy(&sel[(j + 1) * nw], &sel[j * nw], sizeof(uint64_t) * nw);
            j--;
        }
        memcpy(&sel[(j + 1) * nw], t, sizeof(uint64_t) * nw);
    }
    c->nd = K;
    c->ddets = sel;
    /* absent determinants join the main list with zero population */
    int64_t istart = 0;
    for (int64_t k = 0; k < K; k++) {
        int hit;
        int64_t pos = bsearch_main(c, &sel[k * nw], istart, c->n - 1, &hit);
        if (!hit) {
            if (c->n + 1 > c->cap) {
                c->error_flags |= HGPU_FLAG_MAIN_OVERFLOW;
                break;
            }
            memmove(&c->dets[(pos + 1) * nw], &c->dets[pos * nw], sizeof(uint64_t) * nw * (size_t)(c->n - pos));
            memmove(&c->pops[(pos + 1) * R], &c->pops[pos * R], sizeof(int64_t) * R * (size_t)(c->n - pos));
            memmove(&c->kii[pos + 1], &c->kii[pos], sizeof(double) * (size_t)(c->n - pos));
            memcpy(&c->dets[pos * nw], &sel[k * nw], sizeof(uint64_t) * nw);
            for (int s = 0; s < R; s++) c->pops[pos * R + s] = 0;
            c->kii[pos] = kii_of(c, &sel[k * nw]);
            c->n++;
        }
        istart = pos + 1;
    }
    /* the Hamiltonian by column */
    c->dcol_ptr = (int64_t *)calloc((size_t)K + 1, sizeof(int64_t));
    int64_t cap = 16, nnz = 0;
    c->dcol_i = (int64_t *)malloc(sizeof(int64_t) * cap);
    c->dcol_h = (double *)malloc(sizeof(double) * cap);
    for (int64_t j = 0; j < K; j++) {
        c->dcol_ptr[j] = nnz;
        for (int64_t i = 0; i < K; i++) {
            double h = i == j ? kii_of(c, &sel[j * nw]) : hmatel_any(c, &sel[i * nw], &sel[j * nw]);
            if (!(fabs(h) > DEPSILON)) continue;
            if (nnz == cap) {
                cap *= 2;
                c->dcol_i = (int64_t *)realloc(c->dcol_i, sizeof(int64_t) * cap);
                c->dcol_h = (double *)realloc(c->dcol_h, sizeof(double) * cap);
            }
            c->dcol_i[nnz] = i;
            c->dcol_h[nnz] = h;
            nnz++;
        }
    }
    c->dcol_ptr[K] = nnz;
    c->dvec = (double *)calloc((size_t)(K * R), sizeof(double));
    c->dy = (double *)calloc((size_t)(K * R), sizeof(double));
    c->dind = (int64_t *)calloc((size_t)K, sizeof(int64_t));
    c->ss_on = 1;
}

/* determ_proj_separate_annihil (src/semi_stoch.F90:1009-1094) without
 * quasi-Newton (rho_minus_qn_weight = 0, quasi_newton_pop_control = 1), then
 * deterministic_annihilation (src/annihilation.f90:488-535): the projected
 * amplitudes, stochastically rounded to the walker unit, added to the main list. */
static void ss_project(oracle_ctx *c) {
    const int R = c->R;
    const double a = -1.0 * c->cfg.tau;
    for (int s = 0; s < R; s++) {
        const double scale = -c->cfg.tau * (0.0 - c->shift[s] * 1.0);
        for (int64_t k = 0; k < c->nd; k++) c->dy[k * R + s] = scale * c->dvec[k * R + s];
        for (int64_t j = 0; j < c->nd; j++) {
            double y = c->dy[j * R + s];
            for (int64_t z = c->dcol_ptr[j]; z < c->dcol_ptr[j + 1]; z++)
                y = y + a * c->dcol_h[z] * c->dvec[c->dcol_i[z] * R + s];
            c->dy[j * R + s] = y;
        }
    }
    for (int64_t k = 0; k < c->nd; k++) {
        const int64_t ind = c->dind[k];
        for (int s = 0; s < R; s++) {
            double amp = c->dy[k * R + s] * (double)c->real_factor;
            const int64_t sign = amp < 0.0 ? -1 : 1;
            amp = fabs(amp);
            int64_t n = (int64_t)amp;
            amp = amp - (double)n;
            rstream rs;
            rs_init(&rs, (uint64_t)c->cfg.seed, P_DETERM, s, (uint64_t)k, 0, (uint64_t)c->iter);
            if (amp > rs_next(&rs)) n = n + 1;
            c->pops[ind * R + s] += sign * n;
        }
    }
}

/* determ_proj_combined_annihil (src/semi_stoch.F90:897-975) without
 * quasi-Newton (rho_minus_qn_weight = 0, quasi_newton_pop_control = 1): for each
 * deterministic state (row) and space, out = sum_j H(row, j) v_j over the row in
 * ascending column order (csrpgemv_single_row, lib/local/csr.f90:206-235; the
 * symmetric matrix's row is its stored column), out = -tau (out + (E 0 - 1 S) v_row),
 * then create_spawned_particle_determ (:1096-1146): out in walker units,
 * rounded up with probability of its fraction, appended to the spawned list as a
 * spawn from an initiator (flag 0) after every spawning attempt's entries. */
static void ss_project_combined(oracle_ctx *c) {
    const int R = c->R;
    for (int64_t r = 0; r < c->nd; r++) {
        for (int s = 0; s < R; s++) {
            double out = 0.0;
            for (int64_t z = c->dcol_ptr[r]; z < c->dcol_ptr[r + 1]; z++)
                out = out + c->dcol_h[z] * c->dvec[c->dcol_i[z] * R + s];
            const double coef = 0.0 * 0.0 - 1.0 * c->shift[s];
            out = -c->cfg.tau * (out + coef * c->dvec[r * R + s]);
            const double scaled = out * (double)c->real_factor;
            const int64_t sign = scaled < 0.0 ? -1 : 1;
            const double amp = fabs(scaled);
            int64_t n = (int64_t)amp;
            rstream rs;
            rs_init(&rs, (uint64_t)c->cfg.seed, P_DETERM, s, (uint64_t)r, 0, (uint64_t)c->iter);
            if (amp - (double)n > rs_next(&rs)) n = n + 1;
            add_spawn(c, &c->ddets[r * c->nw], s, n * sign, 0, c->sn);
        }
    }
}

/* accumulate_bloom_stats (src/bloom_handler.F90:104-145) with FCIQMC's fixed-n
 * threshold of 3 particles (init_bloom_stats_t, src/fciqmc.f90:214): the
 * report's count and particle sum, the calculation's largest bloom.  The sum is
 * kept exactly in encoded units (HANDE adds each real(nspawn)/factor in FP64). */
static void accumulate_bloom_stats(oracle_ctx *c, int64_t nspawn) {
    const int64_t a = nspawn < 0 ? -nspawn : nspawn;
    if (a < 3 * c->real_factor) return;
    c->bloom_n++;
    c->bloom_tot += a;
    if (a > c->bloom_max) c->bloom_max = a;
}

/* The first half of a Monte Carlo cycle: the loop over the occupied
 * determinants (src/fciqmc.f90:307-392) -- estimators, attempts, spawning into
 * the spawned list, death.  Returns the number of deaths; *nattempts_acc is
 * init_mc_cycle's nattempts (2 N_w at the start of the cycle). */
static int64_t mc_cycle_spawn(oracle_ctx *c, int64_t *nattempts_acc_out) {
    c->iter++;
    if (c->cfg.semi_stoch_space != 0 && c->iter == c->ss_iter) ss_init(c);
    /* init_mc_cycle (src/qmc_common.F90:950-1017) */
    int64_t nattempts_acc = llround(2.0 * nparticles(c, 0));
    int64_t ndeath = 0;
    c->sn = 0;
    uint64_t child[MAXW];
    for (int64_t idet = 0; idet < c->n; idet++) {
        const uint64_t *f = &c->dets[idet * c->nw];
        det_info d;
        decode_any(c, f, &d);
        double real_pop[2];
        for (int s = 0; s < c->R; s++) real_pop[s] = (double)c->pops[idet * c->R + s] / (double)c->real_factor;
        int64_t flag = parent_flag(c, real_pop);
        /* set_determ_info (src/semi_stoch.F90:826-857); deterministic states
         * are initiators (set_parent_flag, src/ifciqmc.f90:14-58) */
        const int64_t dk = c->ss_on ? ss_find(c, f) : -1;
        if (dk >= 0) {
            for (int s = 0; s < c->R; s++) c->dvec[dk * c->R + s] = real_pop[s];
            c->dind[dk] = idet;
            flag = 0;
        }
        excit_t ex = get_excitation(c, f, c->f0);
        for (int s = 0; s < c->R; s++) {
            update_proj_energy(c, f, &d, &ex, real_pop[s], s);
            rstream rs;
            rs_init(&rs, (uint64_t)c->cfg.seed, P_NATTEMPT, s, (uint64_t)idet, 0, (uint64_t)c->iter);
            int64_t nat = decide_nattempts(&rs, real_pop[s]);
            c->rep_attempts += nat;
            c->total_attempts += nat;
            int64_t parent = c->pops[idet * c->R + s];
            for (int64_t a = 0; a < nat; a++) {
                attempt_t at;
                rs_init(&rs, (uint64_t)c->cfg.seed, P_SPAWN, s, (uint64_t)idet, (uint64_t)a, (uint64_t)c->iter);
                at.nspawn_rdm = 0;
                attempt(c, &rs, f, &d, parent, &at, 0);
                if (at.nspawn != 0) {
                    excited_det(c, f, &at.e, child);
                    /* no spawning between deterministic states (src/fciqmc.f90:777-790) */
                    if (dk < 0 || ss_find(c, child) < 0) {
                        add_spawn(c, child, s, at.nspawn, c->cfg.initiator_approx ? flag : 0, c->sn);
                        accumulate_bloom_stats(c, at.nspawn);
                    }
                }
                if (at.nspawn_rdm != 0) {
                    excited_det(c, f, &at.e, child);
                    add_rdm_spawn(c, f, child, s, at.nspawn_rdm);
                }
            }
            if (dk < 0) {
                rs_init(&rs, (uint64_t)c->cfg.seed, P_DEATH, s, (uint64_t)idet, 0, (uint64_t)c->iter);
                ndeath += stochastic_death(c, &rs, c->kii[idet], c->shift[s], &c->pops[idet * c->R + s]);
            }
        }
    }
    *nattempts_acc_out = nattempts_acc;
    return ndeath;
}

/* The second half: projection of the deterministic space, direct_annihilation,
 * the RDM update and end_mc_cycle (src/fciqmc.f90:393-405). */
static void mc_cycle_finish(oracle_ctx *c, int64_t ndeath, int64_t nattempts_acc) {
    /* combined annihilation: the projection's spawns join the list first, and
     * calc_events_spawn_t counts them (direct_annihilation, src/annihilation.f90:52) */
    if (c->ss_on && c->cfg.semi_stoch_combined) ss_project_combined(c);
    int64_t nspawn_events = c->sn; /* calc_events_spawn_t */
    c->rep_spawned += c->sn;
    if (c->ss_on && !c->cfg.semi_stoch_combined) ss_project(c);
    direct_annihilation(c);
    if (c->rdm_on) update_rdm_from_spawns(c);
    c->last_nspawn_events = nspawn_events;
    /* end_mc_cycle / spawning_rate (src/qmc_common.F90:1240-1304) */
    if (nattempts_acc > 0)
        c->acc_rspawn += ((double)nspawn_events + (double)ndeath / (double)c->real_factor) / (double)nattempts_acc;
    c->rep_cycles++;
}

static void mc_cycle(oracle_ctx *c) {
    int64_t nattempts_acc;
    const int64_t ndeath = mc_cycle_spawn(c, &nattempts_acc);
    mc_cycle_finish(c, ndeath, nattempts_acc);
}

/* ------------------------------------------------------------------------- */
/* Public API                                                                 */
/* ------------------------------------------------------------------------- */

oracle_ctx *oracle_create(const hgpu_config *cfg, const hgpu_system *sys) {
    if (sys->nwords > MAXW || sys->nbasis > MAXB || sys->nel > MAXEL) return NULL;
    oracle_ctx *c = (oracle_ctx *)calloc(1, sizeof(oracle_ctx));
    c->cfg = *cfg;
    c->kind = sys->kind;
    c->nbasis = sys->nbasis;
    c->nel = sys->nel;
    c->nalpha = sys->nalpha;
    c->nbeta = sys->nbeta;
    c->nw = sys->nwords;
    c->nvirt_alpha = sys->nbasis / 2 - sys->nalpha;
    c->nvirt_beta = sys->nbasis / 2 - sys->nbeta;
    c->nvirt = sys->nbasis - sys->nel;
    c->orb_sym = (int32_t *)malloc(sizeof(int32_t) * c->nbasis);
    c->orb_ms = (int32_t *)malloc(sizeof(int32_t) * c->nbasis);
    c->sp_eigv = (double *)malloc(sizeof(double) * c->nbasis);
    memcpy(c->orb_sym, sys->orb_sym, sizeof(int32_t) * c->nbasis);
    memcpy(c->orb_ms, sys->orb_ms, sizeof(int32_t) * c->nbasis);
    memcpy(c->sp_eigv, sys->sp_eigv, sizeof(double) * c->nbasis);
    if (c->kind == HGPU_SYS_HUB_K) {
        c->nk = sys->nkpoints;
        c->sym_table = (int32_t *)malloc(sizeof(int32_t) * c->nk * c->nk);
        c->inv_sym = (int32_t *)malloc(sizeof(int32_t) * c->nk);
        memcpy(c->sym_table, sys->sym_table, sizeof(int32_t) * c->nk * c->nk);
        memcpy(c->inv_sym, sys->inv_sym, sizeof(int32_t) * c->nk);
        c->coulomb_k = sys->coulomb_k;
        c->nsym = 1;
    } else {
        c->norb = sys->norb;
        c->nsym = sys->nsym_pg;
        c->h1 = (double *)malloc(sizeof(double) * c->norb * c->norb);
        memcpy(c->h1, sys->h1, sizeof(double) * c->norb * c->norb);
        c->nv2 = sys->nv2;
        c->v2 = (double *)malloc(sizeof(double) * c->nv2);
        memcpy(c->v2, sys->v2, sizeof(double) * c->nv2);
        c->ecore = sys->ecore;
        c->maxss = sys->max_sym_spin;
        c->nbss = (int32_t *)malloc(sizeof(int32_t) * 2 * c->nsym);
        memcpy(c->nbss, sys->nbasis_sym_spin, sizeof(int32_t) * 2 * c->nsym);
        c->ssbf = (int32_t *)malloc(sizeof(int32_t) * c->nsym * 2 * c->maxss);
        memcpy(c->ssbf, sys->sym_spin_basis_fns, sizeof(int32_t) * c->nsym * 2 * c->maxss);
    }
    for (int p = 0; p < c->nbasis; p++) {
        for (int w = 0; w < MAXW; w++) c->mask[p][w] = 0;
        for (int q = p + 1; q < c->nbasis; q++) c->mask[p][q >> 6] |= (uint64_t)1 << (q & 63);
    }
    c->R = cfg->nspaces > 0 ? cfg->nspaces : 1;
    c->real_factor = cfg->real_amplitudes ? ((int64_t)1 << 31) : 1;
    /* alloc_spawn_t: cutoff = ceiling(cutoff*real_factor); 0 for integer walkers
     * (src/spawn_data.F90:215, src/qmc.F90:1484-1485) */
    c->cutoff = cfg->real_amplitudes ? (int64_t)ceil(cfg->spawn_cutoff * (double)c->real_factor) : 0;
    for (int w = 0; w < MAXW; w++) c->f0[w] = w < c->nw ? cfg->ref_det[w] : 0;
    /* init_excit_gen (src/qmc.F90:951-972) */
    if (cfg->pattempt_single < 0 || cfg->pattempt_double < 0) {
        if (c->kind == HGPU_SYS_HUB_K) { c->pattempt_single = 0.0; c->pattempt_double = 1.0; }
        else single_double_prob(c, &c->pattempt_single, &c->pattempt_double);
    } else {
        c->pattempt_single = cfg->pattempt_single / (cfg->pattempt_single + cfg->pattempt_double);
        c->pattempt_double = 1.0 - cfg->pattempt_single;
    }
    /* pattempt_parallel (src/qmc.F90:974-988) and the pgen_ij of each spin
     * class, in choose_ij_spin_mol's rounding order */
    c->spin_ij = c->kind == HGPU_SYS_READ_IN &&
                 (cfg->excit_gen == HGPU_EXCIT_GEN_RENORM_SPIN || cfg->excit_gen == HGPU_EXCIT_GEN_NO_RENORM_SPIN);
    if (c->spin_ij) {
        double pp = cfg->pattempt_parallel < 0.0 ? find_parallel_spin_prob_mol(c) : cfg->pattempt_parallel;
        double na = (double)c->nalpha, nb = (double)c->nbeta;
        c->pattempt_parallel = pp;
        c->pgen_ij_aa = c->nalpha >= 2 ? pp * (na / (na + nb)) * 2.0 * (1.0 / na) * (1.0 / (na - 1.0)) : 0.0;
        c->pgen_ij_bb = c->nbeta >= 2 ? pp * (nb / (na + nb)) * 2.0 * (1.0 / nb) * (1.0 / (nb - 1.0)) : 0.0;
        c->pgen_ij_ab = (1.0 - pp) * (1.0 / (double)(c->nalpha * c->nbeta));
    }
    if (c->kind == HGPU_SYS_HUB_K) {
        double c0 = (double)(c->nalpha * c->nbeta) * c->coulomb_k;
        int64_t B = ceil_abs(c0);
        for (int p = 0; p < c->nbasis; p++) B += ceil_abs(c->sp_eigv[p]);
        c->fx_s = scale_for_bound(B);
        c->fx_cst = fx_of(c, c0);
        c->fx_eps = (int64_t *)malloc(sizeof(int64_t) * c->nbasis);
        for (int p = 0; p < c->nbasis; p++) c->fx_eps[p] = fx_of(c, c->sp_eigv[p]);
    } else {
        int M = c->norb;
        int64_t B = ceil_abs(c->ecore);
        for (int i = 0; i < c->nbasis; i++) {
            B += ceil_abs(c->h1[(i >> 1) * M + (i >> 1)]);
            for (int j = i + 1; j < c->nbasis; j++) {
                B += ceil_abs(v2_get(c, i, j, i, j));
                if (c->orb_ms[i] == c->orb_ms[j]) B += ceil_abs(v2_get(c, i, j, j, i));
            }
        }
        c->fx_s = scale_for_bound(B);
        c->fx_cst = fx_of(c, c->ecore);
        c->fx_h1 = (int64_t *)malloc(sizeof(int64_t) * M);
        c->fx_J = (int64_t *)malloc(sizeof(int64_t) * M * M);
        c->fx_JK = (int64_t *)malloc(sizeof(int64_t) * M * M);
        for (int p = 0; p < M; p++) {
            c->fx_h1[p] = fx_of(c, c->h1[p * M + p]);
            for (int q = 0; q < M; q++) {
                int64_t J = fx_of(c, v2_get(c, 2 * p, 2 * q, 2 * p, 2 * q)); /* <ij|ij> = (ii|jj) */
                int64_t K = fx_of(c, v2_get(c, 2 * p, 2 * q, 2 * q, 2 * p)); /* <ij|ji> = (ij|ji) */
                c->fx_J[p * M + q] = J;
                c->fx_JK[p * M + q] = J - K;
            }
        }
    }
    if (c->kind == HGPU_SYS_READ_IN &&
        (cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH || cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM ||
         cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE)) {
        if (init_heat_bath(c, cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH) != 0) {
            oracle_destroy(c);
            return NULL;
        }
    }
    if (c->kind == HGPU_SYS_READ_IN && (cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
                                        cfg->excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ))
        init_pp_ij(c);
    if (c->kind == HGPU_SYS_READ_IN && cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN) init_ppn(c);
    c->fx_E0 = fx_energy(c, c->f0);
    c->H00 = fx_val(c, c->fx_E0);
    c->cap = cfg->walker_length > 0 ? cfg->walker_length : 1000000;
    c->scap = cfg->spawned_walker_length > 0 ? cfg->spawned_walker_length : 1000000;
    c->dets = (uint64_t *)calloc((size_t)(c->cap * c->nw), sizeof(uint64_t));
    c->pops = (int64_t *)calloc((size_t)(c->cap * c->R), sizeof(int64_t));
    c->kii = (double *)calloc((size_t)c->cap, sizeof(double));
    c->sdets = (uint64_t *)calloc((size_t)(c->scap * c->nw), sizeof(uint64_t));
    c->spops = (int64_t *)calloc((size_t)(c->scap * c->R), sizeof(int64_t));
    c->sflag = (int64_t *)calloc((size_t)c->scap, sizeof(int64_t));
    c->sord = (int64_t *)calloc((size_t)c->scap, sizeof(int64_t));
    c->suid = (int64_t *)calloc((size_t)c->scap, sizeof(int64_t));
    for (int s = 0; s < 2; s++) c->shift[s] = cfg->initial_shift;
    /* semi_stoch_iter = max(start_iter, mc_cycles_done + 1) (src/fciqmc.f90:229) */
    c->ss_iter = INT64_MAX;
    if (cfg->semi_stoch_space != 0) c->ss_iter = cfg->semi_stoch_start_iter > 1 ? cfg->semi_stoch_start_iter : 1;
    if ((cfg->semi_stoch_space != 0 && cfg->semi_stoch_space != 1 && cfg->semi_stoch_space != 4) ||
        (cfg->semi_stoch_space != 0 && cfg->density_matrices)) {
        oracle_destroy(c);
        return NULL;
    }
    if (cfg->density_matrices) {
        if (c->kind != HGPU_SYS_READ_IN || c->R != 2) {
            oracle_destroy(c);
            return NULL;
        }
        c->rdm_enabled = 1;
        c->npairs = (int64_t)c->nbasis * (c->nbasis - 1) / 2;
        c->rdm = (double *)calloc((size_t)(c->npairs * c->npairs), sizeof(double));
        c->rsdets = (uint64_t *)calloc((size_t)(c->scap * 2 * c->nw), sizeof(uint64_t));
        c->rspops = (int64_t *)calloc((size_t)(c->scap * c->R), sizeof(int64_t));
    }
    return c;
}

void oracle_destroy(oracle_ctx *c) {
    if (!c) return;
    ss_free(c);
    free(c->orb_sym); free(c->orb_ms); free(c->sp_eigv);
    free(c->sym_table); free(c->inv_sym); free(c->h1); free(c->v2); free(c->nbss); free(c->ssbf);
    free(c->fx_h1); free(c->fx_J); free(c->fx_JK); free(c->fx_eps);
    free(c->dets); free(c->pops); free(c->kii);
    free(c->sdets); free(c->spops); free(c->sflag); free(c->sord); free(c->suid);
    free(c->rdm); free(c->rsdets); free(c->rspops);
    for (int t = 0; t < 6; t++) {
        free(c->ppn_w[t]); free(c->ppn_U[t]); free(c->ppn_K[t]); free(c->ppn_tot[t]);
    }
    free(c->hb_i_w); free(c->hb_ij_w); free(c->hb_ija_w); free(c->hb_ija_tot); free(c->hb_ija_U);
    free(c->hb_ija_K); free(c->hb_ijab_w); free(c->hb_ijab_tot); free(c->hb_ijab_U); free(c->hb_ijab_K);
    free(c);
}

/* initial_distribution (src/qmc.F90:1507-1560). */
int oracle_initial_distribution(oracle_ctx *c) {
    c->n = 1;
    memcpy(c->dets, c->f0, sizeof(uint64_t) * c->nw);
    for (int s = 0; s < c->R; s++) c->pops[s] = (int64_t)llround(c->cfg.D0_population) * c->real_factor;
    c->kii[0] = 0.0;
    for (int s = 0; s < c->R; s++) {
        c->nparticles_old[s] = nparticles(c, s);
        c->shift[s] = c->cfg.initial_shift;
        c->vary_shift[s] = 0;
    }
    return 0;
}

/* A list that did not come from the calculation's own cycles need not hold the
 * deterministic states: the space is dropped and built again at the next
 * iteration, as a restarted calculation does (src/fciqmc.f90:229-235). */
static void ss_reschedule(oracle_ctx *c) {
    if (c->cfg.semi_stoch_space == 0) return;
    int all_vary = 1;
    for (int s = 0; s < c->R; s++) all_vary = all_vary && c->vary_shift[s];
    c->ss_iter = c->cfg.semi_stoch_start_iter > c->iter + 1 ? c->cfg.semi_stoch_start_iter : c->iter + 1;
    if (all_vary && c->cfg.semi_stoch_shift_iter != -1) c->ss_iter = c->iter + 1;
    ss_free(c);
}

int oracle_set_walkers(oracle_ctx *c, const int64_t *states, const int64_t *pops, const double *dat, int64_t n) {
    if (n > c->cap) return HGPU_ERR_INVALID;
    ss_reschedule(c);
    c->n = n;
    memcpy(c->dets, states, sizeof(uint64_t) * c->nw * n);
    memcpy(c->pops, pops, sizeof(int64_t) * c->R * n);
    for (int64_t i = 0; i < n; i++) c->kii[i] = dat ? dat[i] : kii_of(c, &c->dets[i * c->nw]);
    for (int s = 0; s < c->R; s++) c->nparticles_old[s] = nparticles(c, s);
    return 0;
}

int64_t oracle_get_walkers(oracle_ctx *c, int64_t *states, int64_t *pops, double *dat, int64_t cap) {
    if (cap >= c->n) {
        if (states) memcpy(states, c->dets, sizeof(uint64_t) * c->nw * c->n);
        if (pops) memcpy(pops, c->pops, sizeof(int64_t) * c->R * c->n);
        if (dat) memcpy(dat, c->kii, sizeof(double) * c->n);
    }
    return c->n;
}

/* The start of a report (src/fciqmc.f90:283-291): clear the RDM once
 * accumulating; start accumulating after density_matrix_report reports once
 * every shift varies. */
static void report_start(oracle_ctx *c) {
    if (c->rep_cycles == 0 && c->rdm_enabled) {
        if (c->rdm_on) memset(c->rdm, 0, sizeof(double) * (size_t)(c->npairs * c->npairs));
        int all_vary = 1;
        for (int s = 0; s < c->R; s++) all_vary = all_vary && c->vary_shift[s];
        if (all_vary && c->reports_done + 1 > c->cfg.density_matrix_report) c->rdm_on = 1;
    }
}

int oracle_run_cycles(oracle_ctx *c, int32_t ncycles) {
    report_start(c);
    for (int k = 0; k < ncycles; k++) mc_cycle(c);
    return c->error_flags ? (c->error_flags & HGPU_FLAG_SPAWN_OVERFLOW ? HGPU_ERR_SPAWN_OVERFLOW
                                                                       : HGPU_ERR_MAIN_OVERFLOW)
                          : 0;
}

/* communicated_energy_estimators (src/energy_evaluation.F90:425-657) and
 * update_shift (:659-711), for one process: the damping term, then the
 * harmonic forcing toward target_particles (when shift_harmonic_forcing != 0). */
int oracle_end_report(oracle_ctx *c, hgpu_report *out) {
    int nc = c->rep_cycles > 0 ? c->rep_cycles : 1;
    memset(out, 0, sizeof(*out));
    if (c->rdm_on) {
        calc_rdm_energy(c, &c->rdm_energy, &c->rdm_trace);
        out->rdm_energy = c->rdm_energy;
        out->rdm_trace = c->rdm_trace;
    }
    c->reports_done++;
    double ntot[2];
    for (int s = 0; s < c->R; s++) {
        out->proj_energy[s] = c->acc_proj[s] / (double)nc;
        out->D0_population[s] = c->acc_d0[s] / (double)nc;
        ntot[s] = nparticles(c, s);
    }
    for (int s = 0; s < c->R; s++) {
        if (c->vary_shift[s]) {
            c->shift[s] = c->shift[s] - log(ntot[s] / c->nparticles_old[s]) * c->cfg.shift_damping /
                                            (1.0 * c->cfg.tau * (double)nc);
            if (c->cfg.shift_harmonic_forcing != 0.0 && c->cfg.target_particles > 0.0)
                c->shift[s] = c->shift[s] - log(ntot[s] / c->cfg.target_particles) * c->cfg.shift_harmonic_forcing /
                                                (1.0 * c->cfg.tau * (double)nc);
        }
    }
    for (int s = 0; s < c->R; s++) c->nparticles_old[s] = ntot[s];
    int all_vary_before = 1, all_vary = 1;
    for (int s = 0; s < c->R; s++) all_vary_before = all_vary_before && c->vary_shift[s];
    for (int s = 0; s < c->R; s++) {
        const double above = c->cfg.target_reference ? out->D0_population[s] : ntot[s];
        if (!c->vary_shift[s] && above > c->cfg.target_particles) {
            c->vary_shift[s] = 1;
            if (c->cfg.vary_shift_from_proje) c->shift[s] = out->proj_energy[s] / out->D0_population[s];
            else c->shift[s] = c->cfg.vary_shift_from;
        }
    }
    /* the space follows the shift (src/qmc_common.F90:1203-1204) */
    for (int s = 0; s < c->R; s++) all_vary = all_vary && c->vary_shift[s];
    if (!all_vary_before && all_vary && c->cfg.semi_stoch_space != 0 && c->cfg.semi_stoch_shift_iter != -1)
        c->ss_iter = c->cfg.semi_stoch_shift_iter + c->iter + 1;
    for (int s = 0; s < c->R; s++) {
        out->shift[s] = c->shift[s];
        out->nparticles[s] = ntot[s];
        out->vary_shift[s] = c->vary_shift[s];
    }
    out->iteration = c->iter;
    out->nstates = c->n;
    out->nspawn_events = c->last_nspawn_events;
    out->rspawn = c->acc_rspawn / (double)nc;
    out->nattempts = c->rep_attempts;
    out->nspawned = c->rep_spawned;
    out->error_flags = c->error_flags;
    out->nblooms = c->bloom_n;
    out->tot_bloom = (double)c->bloom_tot / (double)c->real_factor;
    out->max_bloom = (double)c->bloom_max / (double)c->real_factor;
    c->bloom_n = c->bloom_tot = 0; /* bloom_stats_init_report_loop */
    for (int s = 0; s < 2; s++) { c->acc_proj[s] = 0.0; c->acc_d0[s] = 0.0; }
    c->acc_rspawn = 0.0;
    c->rep_attempts = 0;
    c->rep_spawned = 0;
    c->rep_cycles = 0;
    return c->error_flags ? HGPU_ERR_SPAWN_OVERFLOW : 0;
}

int oracle_get_state(oracle_ctx *c, hgpu_state *out) {
    memset(out, 0, sizeof(*out));
    out->iteration = c->iter;
    for (int s = 0; s < 2; s++) {
        out->shift[s] = c->shift[s];
        out->vary_shift[s] = c->vary_shift[s];
        out->nparticles_old[s] = c->nparticles_old[s];
    }
    out->tau = c->cfg.tau;
    out->seed = c->cfg.seed;
    return 0;
}

int oracle_set_state(oracle_ctx *c, const hgpu_state *in) {
    c->iter = in->iteration;
    for (int s = 0; s < 2; s++) {
        c->shift[s] = in->shift[s];
        c->vary_shift[s] = in->vary_shift[s];
        c->nparticles_old[s] = in->nparticles_old[s];
    }
    ss_reschedule(c);
    return 0;
}

int oracle_eval_excitations(oracle_ctx *c, const int64_t *parents, const int64_t *parent_pops, int64_t n,
                            int64_t iteration, int32_t *orbs, double *pgen, double *hmatel, int32_t *allowed,
                            int64_t *nspawn) {
    for (int64_t i = 0; i < n; i++) {
        const uint64_t *f = (const uint64_t *)&parents[i * c->nw];
        det_info d;
        decode_any(c, f, &d);
        rstream rs;
        rs_init(&rs, (uint64_t)c->cfg.seed, P_SPAWN, 0, (uint64_t)i, 0, (uint64_t)iteration);
        attempt_t at;
        attempt(c, &rs, f, &d, parent_pops[i], &at, 1);
        orbs[4 * i + 0] = at.e.from[0];
        orbs[4 * i + 1] = at.e.nexcit == 2 ? at.e.from[1] : -1;
        orbs[4 * i + 2] = at.e.to[0];
        orbs[4 * i + 3] = at.e.nexcit == 2 ? at.e.to[1] : -1;
        pgen[i] = at.pgen;
        hmatel[i] = at.hmatel;
        allowed[i] = at.allowed;
        nspawn[i] = at.nspawn;
    }
    return 0;
}

int oracle_annihilate_fixed(oracle_ctx *c, const int64_t *sdata, int64_t n, int64_t iteration) {
    int el = c->nw + c->R + 1;
    if (n > c->scap) return HGPU_ERR_SPAWN_OVERFLOW;
    c->sn = 0;
    for (int64_t k = 0; k < n; k++) {
        const int64_t *e = &sdata[k * el];
        memcpy(&c->sdets[k * c->nw], e, sizeof(uint64_t) * c->nw);
        for (int s = 0; s < c->R; s++) c->spops[k * c->R + s] = e[c->nw + s];
        c->sflag[k] = c->cfg.initiator_approx ? e[c->nw + c->R] : 0;
        c->sord[k] = k;
    }
    c->sn = n;
    int64_t save = c->iter;
    c->iter = iteration;
    direct_annihilation(c);
    c->iter = save;
    return c->error_flags & HGPU_FLAG_MAIN_OVERFLOW ? HGPU_ERR_MAIN_OVERFLOW : 0;
}

double oracle_hmatel(oracle_ctx *c, const int64_t *f1, const int64_t *f2) {
    return hmatel_any(c, (const uint64_t *)f1, (const uint64_t *)f2);
}

double oracle_sc0(oracle_ctx *c, const int64_t *f) { return sc0(c, (const uint64_t *)f); }

double oracle_pattempt_parallel(oracle_ctx *c) { return c->spin_ij ? c->pattempt_parallel : -1.0; }

int64_t oracle_determ_space(oracle_ctx *c, int64_t *dets, int64_t n) {
    if (dets && n >= c->nd) memcpy(dets, c->ddets, sizeof(uint64_t) * (size_t)(c->nd * c->nw));
    return c->nd;
}

void oracle_pattempt(oracle_ctx *c, double *out) {
    out[0] = c->pattempt_single;
    out[1] = c->pattempt_double;
}

int64_t oracle_rdm(oracle_ctx *c, double *out, int64_t n) {
    if (!c->rdm_enabled) return 0;
    int64_t m = c->npairs * c->npairs;
    if (out && n >= m) memcpy(out, c->rdm, sizeof(double) * (size_t)m);
    return m;
}

void oracle_rdm_energy(oracle_ctx *c, double *energy, double *trace) {
    *energy = *trace = 0.0;
    if (c->rdm_enabled) calc_rdm_energy(c, energy, trace);
}

void oracle_rdm_from_list(oracle_ctx *c) {
    if (!c->rdm_enabled) return;
    c->rsn = 0;
    update_rdm_from_spawns(c);
}

double oracle_pgen(oracle_ctx *c, const int64_t *fi, const int32_t *orbs) {
    const uint64_t *f = (const uint64_t *)fi;
    det_info d;
    decode_any(c, f, &d);
    if (c->kind == HGPU_SYS_HUB_K) {
        int ij_sym = c->sym_table[kidx(orbs[0]) * c->nk + kidx(orbs[1])];
        if (c->cfg.excit_gen == HGPU_EXCIT_GEN_NO_RENORM)
            return 1.0 / (double)(c->nalpha * c->nbeta * c->nvirt_alpha);
        return calc_pgen_hub_k(c, ij_sym, f, &d);
    }
    int renorm = c->cfg.excit_gen == HGPU_EXCIT_GEN_RENORM || c->cfg.excit_gen == HGPU_EXCIT_GEN_RENORM_SPIN;
    if (orbs[1] < 0) {
        return c->pattempt_single *
               (renorm ? calc_pgen_single_mol(c, &d, orbs[2]) : calc_pgen_single_mol_no_renorm(c, orbs[2]));
    }
    int ij_sym = cross(c, c->orb_sym[orbs[0]], c->orb_sym[orbs[1]]);
    int spin = c->orb_ms[orbs[0]] + c->orb_ms[orbs[1]];
    double pij = 2.0 / (double)(c->nel * (c->nel - 1));
    if (c->spin_ij) pij = spin == 2 ? c->pgen_ij_aa : (spin == -2 ? c->pgen_ij_bb : c->pgen_ij_ab);
    if (renorm) return c->pattempt_double * pij * calc_pgen_double_mol(c, ij_sym, orbs[2], orbs[3], spin, &d);
    return c->pattempt_double * pij * calc_pgen_double_mol_no_renorm(c, orbs[2], orbs[3], spin);
}

int64_t oracle_total_attempts(oracle_ctx *c) { return c->total_attempts; }

/* ------------------------------------------------------------------------- */
/* Hash-partitioned calculation on many host cores                            */
/* ------------------------------------------------------------------------- */

/* HANDE runs one calculation over MPI ranks: every determinant belongs to the
 * rank given by a hash of its bit string (assign_particle_processor,
 * src/spawning.F90:770-838: modulo(MurmurHash2(f), nprocs) without load
 * balancing); each rank spawns from its own determinants into per-destination
 * blocks of its spawned list, the blocks are exchanged with one all-to-all per
 * cycle (src/spawn_data.F90:693,721), and each rank annihilates what it
 * received into its own part of the main list; the estimators are summed over
 * the ranks once per report (src/energy_evaluation.F90:191).  The replica RDM
 * spawns go to the owner of the child and every rank keeps an RDM of its own,
 * summed at the report end.  Here the ranks are threads, one oracle context
 * each, and the exchange is a copy through shared memory.  The random streams
 * of rank r are keyed by seed + 1000003 r, so ranks draw independent numbers. */

/* MurmurHash2, 32-bit (Austin Appleby's published algorithm, which the
 * reference vendors in lib/external/MurmurHash2.c), over the bytes of the
 * determinant's words. */
static uint32_t murmur2(const void *key, int len, uint32_t seed) {
    const uint32_t m = 0x5bd1e995u;
    uint32_t h = seed ^ (uint32_t)len;
    const unsigned char *data = (const unsigned char *)key;
    while (len >= 4) {
        uint32_t k = (uint32_t)data[0] | ((uint32_t)data[1] << 8) | ((uint32_t)data[2] << 16) |
                     ((uint32_t)data[3] << 24);
        k *= m;
        k ^= k >> 24;
        k *= m;
        h *= m;
        h ^= k;
        data += 4;
        len -= 4;
    }
    switch (len) {
        case 3: h ^= (uint32_t)data[2] << 16; /* fall through */
        case 2: h ^= (uint32_t)data[1] << 8;  /* fall through */
        case 1: h ^= (uint32_t)data[0]; h *= m;
    }
    h ^= h >> 13;
    h *= m;
    h ^= h >> 15;
    return h;
}

struct oracle_par {
    int P, nw, R;
    oracle_ctx **ctx;
    pthread_barrier_t bar;
    /* per rank: spawned entries ordered by destination rank, and the
     * destination offsets [P+1]; the same for the RDM spawns */
    uint64_t **sd;
    int64_t **sp, **sf, **off;
    uint64_t **rd;
    int64_t **rp, **roff;
    /* snapshot of every rank's list */
    int64_t *snap_n;
    uint64_t **snap_d;
    int64_t **snap_p;
    double **snap_k;
    int ncycles;
    int report_open; /* oracle_par_begin_report ran for the current report */
};

static int par_owner(const oracle_par *p, const uint64_t *f) {
    unsigned char b[8 * MAXW];
    for (int w = 0; w < p->nw; w++)
        for (int k = 0; k < 8; k++) b[8 * w + k] = (unsigned char)(f[w] >> (8 * k));
    const int32_t h = (int32_t)murmur2(b, 8 * p->nw, 7u);
    return (int)(((h % p->P) + p->P) % p->P); /* Fortran modulo */
}

/* rank r: its spawned (and RDM) entries into per-destination blocks */
static void par_bucket(oracle_par *p, int r) {
    oracle_ctx *c = p->ctx[r];
    const int nw = p->nw, R = p->R, P = p->P;
    int64_t *cnt = (int64_t *)calloc((size_t)(unsigned)P, sizeof(int64_t));
    int *dst = (int *)malloc(sizeof(int) * (size_t)(c->sn > 0 ? c->sn : 1));
    for (int64_t k = 0; k < c->sn; k++) cnt[dst[k] = par_owner(p, &c->sdets[k * nw])]++;
    p->off[r][0] = 0;
    for (int d = 0; d < P; d++) p->off[r][d + 1] = p->off[r][d] + cnt[d];
    for (int d = 0; d < P; d++) cnt[d] = p->off[r][d];
    for (int64_t k = 0; k < c->sn; k++) {
        const int64_t o = cnt[dst[k]]++;
        memcpy(&p->sd[r][o * nw], &c->sdets[k * nw], sizeof(uint64_t) * nw);
        memcpy(&p->sp[r][o * R], &c->spops[k * R], sizeof(int64_t) * R);
        p->sf[r][o] = c->sflag[k];
    }
    free(dst);
    if (c->rdm_enabled) {
        int *rdst = (int *)malloc(sizeof(int) * (size_t)(c->rsn > 0 ? c->rsn : 1));
        for (int d = 0; d < P; d++) cnt[d] = 0;
        for (int64_t k = 0; k < c->rsn; k++) cnt[rdst[k] = par_owner(p, &c->rsdets[k * 2 * nw + nw])]++;
        p->roff[r][0] = 0;
        for (int d = 0; d < P; d++) p->roff[r][d + 1] = p->roff[r][d] + cnt[d];
        for (int d = 0; d < P; d++) cnt[d] = p->roff[r][d];
        for (int64_t k = 0; k < c->rsn; k++) {
            const int64_t o = cnt[rdst[k]]++;
            memcpy(&p->rd[r][o * 2 * nw], &c->rsdets[k * 2 * nw], sizeof(uint64_t) * 2 * nw);
            memcpy(&p->rp[r][o * R], &c->rspops[k * R], sizeof(int64_t) * R);
        }
        free(rdst);
    }
    free(cnt);
}

/* rank d: the blocks every rank addressed to it, in rank order, become its
 * spawned list (the receive side of the all-to-all) */
static void par_gather(oracle_par *p, int d) {
    oracle_ctx *c = p->ctx[d];
    const int nw = p->nw, R = p->R;
    int64_t n = 0;
    for (int r = 0; r < p->P; r++) {
        const int64_t a = p->off[r][d], b = p->off[r][d + 1];
        if (n + (b - a) > c->scap) {
            c->error_flags |= HGPU_FLAG_SPAWN_OVERFLOW;
            break;
        }
        memcpy(&c->sdets[n * nw], &p->sd[r][a * nw], sizeof(uint64_t) * nw * (size_t)(b - a));
        memcpy(&c->spops[n * R], &p->sp[r][a * R], sizeof(int64_t) * R * (size_t)(b - a));
        for (int64_t k = a; k < b; k++, n++) {
            c->sflag[n] = p->sf[r][k];
            c->sord[n] = n;
        }
    }
    c->sn = n;
    if (c->rdm_enabled) {
        int64_t m = 0;
        for (int r = 0; r < p->P; r++) {
            const int64_t a = p->roff[r][d], b = p->roff[r][d + 1];
            if (m + (b - a) > c->scap) {
                c->error_flags |= HGPU_FLAG_SPAWN_OVERFLOW;
                break;
            }
            memcpy(&c->rsdets[m * 2 * nw], &p->rd[r][a * 2 * nw], sizeof(uint64_t) * 2 * nw * (size_t)(b - a));
            memcpy(&c->rspops[m * R], &p->rp[r][a * R], sizeof(int64_t) * R * (size_t)(b - a));
            m += b - a;
        }
        c->rsn = m;
    }
}

typedef struct {
    oracle_par *p;
    int r;
    void *(*body)(oracle_par *, int);
} par_arg;

static void *par_thread(void *arg) {
    par_arg *a = (par_arg *)arg;
    return a->body(a->p, a->r);
}

/* Run body(p, r) for every rank r on its own thread. */
static void par_each_rank(oracle_par *p, void *(*body)(oracle_par *, int)) {
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)(unsigned)p->P);
    par_arg *args = (par_arg *)malloc(sizeof(par_arg) * (size_t)(unsigned)p->P);
    for (int r = 0; r < p->P; r++) {
        args[r].p = p;
        args[r].r = r;
        args[r].body = body;
        pthread_create(&th[r], NULL, par_thread, &args[r]);
    }
    for (int r = 0; r < p->P; r++) pthread_join(th[r], NULL);
    free(th);
    free(args);
}

static void *par_report_start(oracle_par *p, int r) {
    report_start(p->ctx[r]);
    return NULL;
}

static void *par_rdm_energy(oracle_par *p, int r) {
    oracle_ctx *c = p->ctx[r];
    if (c->rdm_on) calc_rdm_energy(c, &c->rdm_energy, &c->rdm_trace);
    return NULL;
}

static void *par_cycles(oracle_par *p, int r) {
    oracle_ctx *c = p->ctx[r];
    for (int k = 0; k < p->ncycles; k++) {
        int64_t nacc;
        const int64_t ndeath = mc_cycle_spawn(c, &nacc);
        par_bucket(p, r);
        pthread_barrier_wait(&p->bar); /* every rank's blocks are ready */
        par_gather(p, r);
        mc_cycle_finish(c, ndeath, nacc);
        pthread_barrier_wait(&p->bar); /* every rank has read its blocks */
    }
    return NULL;
}

oracle_par *oracle_par_create(const hgpu_config *cfg, const hgpu_system *sys, int nthreads) {
    if (nthreads < 1) return NULL;
    oracle_par *p = (oracle_par *)calloc(1, sizeof(oracle_par));
    p->P = nthreads;
    p->nw = sys->nwords;
    p->R = cfg->nspaces > 0 ? cfg->nspaces : 1;
    p->ctx = (oracle_ctx **)calloc((size_t)nthreads, sizeof(oracle_ctx *));
#define PAR_ARRAYS(X) X(sd, uint64_t) X(sp, int64_t) X(sf, int64_t) X(off, int64_t) X(rd, uint64_t) \
    X(rp, int64_t) X(roff, int64_t) X(snap_d, uint64_t) X(snap_p, int64_t) X(snap_k, double)
#define PAR_ALLOC(name, T) p->name = (T **)calloc((size_t)nthreads, sizeof(T *));
    PAR_ARRAYS(PAR_ALLOC)
    p->snap_n = (int64_t *)calloc((size_t)nthreads, sizeof(int64_t));
    for (int r = 0; r < nthreads; r++) {
        hgpu_config c = *cfg;
        c.seed = cfg->seed + 1000003LL * r;
        p->ctx[r] = oracle_create(&c, sys);
        if (!p->ctx[r]) {
            oracle_par_destroy(p);
            return NULL;
        }
        const int64_t sc = p->ctx[r]->scap;
        p->sd[r] = (uint64_t *)malloc(sizeof(uint64_t) * p->nw * (size_t)sc);
        p->sp[r] = (int64_t *)malloc(sizeof(int64_t) * p->R * (size_t)sc);
        p->sf[r] = (int64_t *)malloc(sizeof(int64_t) * (size_t)sc);
        p->off[r] = (int64_t *)calloc((size_t)nthreads + 1, sizeof(int64_t));
        p->roff[r] = (int64_t *)calloc((size_t)nthreads + 1, sizeof(int64_t));
        if (cfg->density_matrices) {
            p->rd[r] = (uint64_t *)malloc(sizeof(uint64_t) * 2 * p->nw * (size_t)sc);
            p->rp[r] = (int64_t *)malloc(sizeof(int64_t) * p->R * (size_t)sc);
        }
    }
    pthread_barrier_init(&p->bar, NULL, (unsigned)nthreads);
    return p;
}

void oracle_par_destroy(oracle_par *p) {
    if (!p) return;
    for (int r = 0; r < p->P; r++) {
        if (p->ctx[r]) oracle_destroy(p->ctx[r]);
#define PAR_FREE(name, T) if (p->name) free(p->name[r]);
        PAR_ARRAYS(PAR_FREE)
    }
#define PAR_FREE2(name, T) free(p->name);
    PAR_ARRAYS(PAR_FREE2)
    free(p->snap_n);
    if (p->ctx[0]) pthread_barrier_destroy(&p->bar);
    free(p->ctx);
    free(p);
}

/* initial_distribution: the walkers on the reference, on its owner rank */
int oracle_par_initial_distribution(oracle_par *p) {
    const int owner = par_owner(p, p->ctx[0]->f0);
    for (int r = 0; r < p->P; r++) {
        oracle_ctx *c = p->ctx[r];
        oracle_initial_distribution(c);
        if (r != owner) c->n = 0;
    }
    /* N_w of the whole calculation */
    double tot[2] = {0.0, 0.0};
    for (int r = 0; r < p->P; r++)
        for (int s = 0; s < p->R; s++) tot[s] += nparticles(p->ctx[r], s);
    for (int r = 0; r < p->P; r++)
        for (int s = 0; s < p->R; s++) p->ctx[r]->nparticles_old[s] = tot[s];
    return 0;
}

/* The start of a report on every rank (each clears its own RDM once
 * accumulating); oracle_par_run_cycles does it when the caller has not. */
int oracle_par_begin_report(oracle_par *p) {
    if (!p->report_open) par_each_rank(p, par_report_start);
    p->report_open = 1;
    return 0;
}

int oracle_par_run_cycles(oracle_par *p, int32_t ncycles) {
    oracle_par_begin_report(p);
    p->ncycles = ncycles;
    par_each_rank(p, par_cycles);
    int flags = 0;
    for (int r = 0; r < p->P; r++) flags |= p->ctx[r]->error_flags;
    return flags ? (flags & HGPU_FLAG_SPAWN_OVERFLOW ? HGPU_ERR_SPAWN_OVERFLOW : HGPU_ERR_MAIN_OVERFLOW) : 0;
}

/* The report over all ranks: sums of the estimators, N_w and counters (the
 * estimator buffer's MPI_Allreduce), then update_shift once with the totals
 * and the same shift on every rank. */
int oracle_par_end_report(oracle_par *p, hgpu_report *out) {
    oracle_ctx *c0 = p->ctx[0];
    const int R = p->R;
    const int nc = c0->rep_cycles > 0 ? c0->rep_cycles : 1;
    memset(out, 0, sizeof(*out));
    double proj[2] = {0, 0}, d0[2] = {0, 0}, ntot[2] = {0, 0}, rspawn = 0.0;
    int64_t states = 0, events = 0;
    p->report_open = 0;
    if (c0->rdm_on) par_each_rank(p, par_rdm_energy);
    for (int r = 0; r < p->P; r++) {
        oracle_ctx *c = p->ctx[r];
        if (c->rdm_on) {
            out->rdm_energy += c->rdm_energy;
            out->rdm_trace += c->rdm_trace;
        }
        c->reports_done++;
        for (int s = 0; s < R; s++) {
            proj[s] += c->acc_proj[s];
            d0[s] += c->acc_d0[s];
            ntot[s] += nparticles(c, s);
        }
        rspawn += c->acc_rspawn;
        states += c->n;
        events += c->last_nspawn_events;
        out->nattempts += c->rep_attempts;
        out->nspawned += c->rep_spawned;
        out->error_flags |= c->error_flags;
        out->nblooms += c->bloom_n;
        out->tot_bloom += (double)c->bloom_tot / (double)c->real_factor;
        if ((double)c->bloom_max / (double)c->real_factor > out->max_bloom)
            out->max_bloom = (double)c->bloom_max / (double)c->real_factor;
    }
    for (int s = 0; s < R; s++) {
        out->proj_energy[s] = proj[s] / (double)nc;
        out->D0_population[s] = d0[s] / (double)nc;
    }
    double shift[2], old[2];
    int vary[2];
    for (int s = 0; s < 2; s++) {
        shift[s] = c0->shift[s];
        vary[s] = c0->vary_shift[s];
        old[s] = c0->nparticles_old[s];
    }
    for (int s = 0; s < R; s++)
        if (vary[s]) {
            shift[s] = shift[s] - log(ntot[s] / old[s]) * c0->cfg.shift_damping / (1.0 * c0->cfg.tau * (double)nc);
            if (c0->cfg.shift_harmonic_forcing != 0.0 && c0->cfg.target_particles > 0.0)
                shift[s] = shift[s] - log(ntot[s] / c0->cfg.target_particles) * c0->cfg.shift_harmonic_forcing /
                                          (1.0 * c0->cfg.tau * (double)nc);
        }
    for (int s = 0; s < R; s++) {
        const double above = c0->cfg.target_reference ? out->D0_population[s] : ntot[s];
        if (!vary[s] && above > c0->cfg.target_particles) {
            vary[s] = 1;
            shift[s] = c0->cfg.vary_shift_from_proje ? out->proj_energy[s] / out->D0_population[s]
                                                     : c0->cfg.vary_shift_from;
        }
        out->shift[s] = shift[s];
        out->nparticles[s] = ntot[s];
        out->vary_shift[s] = vary[s];
    }
    out->iteration = c0->iter;
    out->nstates = states;
    out->nspawn_events = events;
    out->rspawn = rspawn / (double)nc / (double)p->P;
    for (int r = 0; r < p->P; r++) {
        oracle_ctx *c = p->ctx[r];
        for (int s = 0; s < R; s++) {
            c->shift[s] = shift[s];
            c->vary_shift[s] = vary[s];
            c->nparticles_old[s] = ntot[s];
            c->acc_proj[s] = c->acc_d0[s] = 0.0;
        }
        c->acc_rspawn = 0.0;
        c->rep_attempts = c->rep_spawned = 0;
        c->rep_cycles = 0;
        c->bloom_n = c->bloom_tot = 0;
    }
    return out->error_flags ? HGPU_ERR_SPAWN_OVERFLOW : 0;
}

/* Save (restore = 0) or restore (1) every rank's walker list. */
int oracle_par_snapshot(oracle_par *p, int restore) {
    for (int r = 0; r < p->P; r++) {
        oracle_ctx *c = p->ctx[r];
        if (!restore) {
            free(p->snap_d[r]); free(p->snap_p[r]); free(p->snap_k[r]);
            const int64_t n = c->n > 0 ? c->n : 1;
            p->snap_d[r] = (uint64_t *)malloc(sizeof(uint64_t) * p->nw * (size_t)n);
            p->snap_p[r] = (int64_t *)malloc(sizeof(int64_t) * p->R * (size_t)n);
            p->snap_k[r] = (double *)malloc(sizeof(double) * (size_t)n);
            memcpy(p->snap_d[r], c->dets, sizeof(uint64_t) * p->nw * (size_t)c->n);
            memcpy(p->snap_p[r], c->pops, sizeof(int64_t) * p->R * (size_t)c->n);
            memcpy(p->snap_k[r], c->kii, sizeof(double) * (size_t)c->n);
            p->snap_n[r] = c->n;
        } else {
            if (!p->snap_d[r]) return HGPU_ERR_INVALID;
            c->n = p->snap_n[r];
            memcpy(c->dets, p->snap_d[r], sizeof(uint64_t) * p->nw * (size_t)c->n);
            memcpy(c->pops, p->snap_p[r], sizeof(int64_t) * p->R * (size_t)c->n);
            memcpy(c->kii, p->snap_k[r], sizeof(double) * (size_t)c->n);
        }
    }
    return 0;
}

/* The qmc_state scalars of every rank (iteration, shift, vary_shift, N_w of
 * the last report); the state of rank 0 is the calculation's. */
int oracle_par_set_state(oracle_par *p, const hgpu_state *in) {
    for (int r = 0; r < p->P; r++) oracle_set_state(p->ctx[r], in);
    return 0;
}

int oracle_par_get_state(oracle_par *p, hgpu_state *out) { return oracle_get_state(p->ctx[0], out); }

int64_t oracle_par_total_attempts(oracle_par *p) {
    int64_t t = 0;
    for (int r = 0; r < p->P; r++) t += p->ctx[r]->total_attempts;
    return t;
}

/* The whole calculation's walker list, merged over the ranks in HANDE's order
 * (the rank lists are each sorted); returns the number of states. */
int64_t oracle_par_get_walkers(oracle_par *p, int64_t *states, int64_t *pops, double *dat, int64_t cap) {
    int64_t n = 0;
    for (int r = 0; r < p->P; r++) n += p->ctx[r]->n;
    if (cap < n || !states) return n;
    int64_t *pos = (int64_t *)calloc((size_t)(unsigned)p->P, sizeof(int64_t));
    for (int64_t k = 0; k < n; k++) {
        int best = -1;
        for (int r = 0; r < p->P; r++) {
            oracle_ctx *c = p->ctx[r];
            if (pos[r] >= c->n) continue;
            if (best < 0 || det_cmp(&c->dets[pos[r] * p->nw], &p->ctx[best]->dets[pos[best] * p->nw], p->nw) > 0)
                best = r;
        }
        oracle_ctx *c = p->ctx[best];
        memcpy(&states[k * p->nw], &c->dets[pos[best] * p->nw], sizeof(uint64_t) * p->nw);
        if (pops) memcpy(&pops[k * p->R], &c->pops[pos[best] * p->R], sizeof(int64_t) * p->R);
        if (dat) dat[k] = c->kii[pos[best]];
        pos[best]++;
    }
    free(pos);
    return n;
}
