// hgpu_device.cuh -- device-side system description, RNG streams, determinant
// bit operations, excitation generators and Slater-Condon rules of the GB300
// FCIQMC engine.
//
// Orbitals are 0-based spin orbitals: p is bit p%64 of word p/64, even p alpha.
// All FP64 arithmetic is written in the operation order of the HANDE
// expressions it implements; the library is built with -fmad=false so no
// multiply-add is contracted and the results round exactly as written.
#pragma once

#include <cstdint>

#include "../../include/hande_gpu.h"
#include "hgpu_exact.h"
#include "hgpu_fixed.h"

namespace hgpu {

constexpr int kMaxWords = HGPU_MAX_WORDS;
// Upper bound on the redraws of a rejection loop.  Acceptance is at least
// 1/nbasis per draw, so the bound is never reached in a correct run; it only
// guarantees that a kernel always terminates (the attempt is then dropped).
constexpr int kMaxRedraw = 1 << 16;
constexpr int kMaxSym = 8;  // D2h subgroups: at most 8 irreps

// RNG stream purposes (counter word 3, bits 28..31).
enum Purpose : uint32_t { P_NATTEMPT = 1, P_SPAWN = 2, P_DEATH = 3, P_ROUND_MAIN = 4, P_ROUND_SPAWN = 5, P_DETERM = 6 };

// Everything the kernels need to know about the system and the calculation.
// Lives in device global memory; small tables are staged to shared memory by
// the kernels that gather from them.
struct alignas(16) DevSys {
    // exact diagonal energies (hgpu_fixed.h): E(D) = fx_const + sum_i h_i + sum_{i<j} pair_ij,
    // in units of 2^-fx_shift
    int64_t fx_const;          // Ecore (read_in) or nalpha*nbeta*U/N (hub_k)
    int64_t fx_E0;             // E(D_0)
    double fx_inv_scale;       // 2^-fx_shift
    const int64_t *fx_h1;      // [norb] h_pp
    const int64_t *fx_pair;    // [2][norb][norb]: [0] opposite spins (pp|qq), [1] same spin (pp|qq)-(pq|qp)
    const int64_t *fx_eps;     // [nbasis] hub_k single-particle energies
    int fx_shift;
    int pad_fx;
    // exact reciprocal tables (values of 1.0/(double)x, so results are unchanged)
    const double *inv;       // [inv_max+1]
    int inv_max;
    int pad_inv;
    double pgen_ij;          // 2/(nel(nel-1))
    const double *hub_pgen;  // [nvirt_alpha+1] 1/(nalpha nbeta (nvirt_alpha - forbidden)), renorm
    const double *hub_pspawn;  // [nvirt_alpha+1] real_factor tau |U/N| / hub_pgen
    const uint8_t *hub_allowed;  // [nvirt_alpha+1] 1/pgen > depsilon
    double hub_pgen_nr, hub_pspawn_nr;  // no_renorm: constant p_gen and p_spawn
    double d_nel, d_nelm1, d_nbasis, d_half_nbasis, d_nalpha, d_nbeta, d_nvirt_alpha, d_real_factor, d_cutoff;
    double d_nbss[16];
    int kind, nbasis, nel, nalpha, nbeta, nw;
    int nvirt_alpha, nvirt_beta, nvirt;
    int nspaces;
    int excit_gen;
    int initiator;
    int real_amplitudes;
    int precision;
    int64_t real_factor;
    int64_t cutoff;  // encoded spawn cutoff
    double tau;
    double pattempt_single, pattempt_double;
    uint64_t t_single;  // u < pattempt_single  <=>  k < t_single for u = k 2^-53: ceil(pattempt_single 2^53)
    const double *pg2;  // [class][n_aij][xa][xb] double-excitation p_gen (pgen_double), pg2_x = max orbitals
                        // per (irrep, spin) + 1; class 0 (and 1, 2: alpha-alpha, beta-beta pairs of the
                        // spin-resolved generators, whose class 0 is the opposite-spin pair)
    int pg2_x, pg2_n;
    // renorm_spin / no_renorm_spin: u < pattempt_parallel and u < nalpha/(nalpha+nbeta)
    // as k < t_parallel, k < t_alpha
    int spin_ij;
    int pad_spin;
    uint64_t t_parallel, t_alpha;
    double initiator_pop;
    int quadrature_initiator;  // two spaces share one initiator test (set_parent_flag)
    int pad_qi;
    double H00;
    uint64_t seed;
    uint64_t f0[kMaxWords];
    // hub_k
    int nk;
    double coulomb_k;
    const uint8_t *sym_table;  // nk*nk
    const uint8_t *inv_sym;    // nk
    const double *sp_eigv;     // nbasis
    // molecular
    int norb, nsym;
    double ecore;
    const double *h1;   // norb*norb
    const double *v2;   // packed (ia|jb)
    const float *h1f;   // FP32 copies for the mixed-precision spawning path
    const float *v2f;
    // per-irrep, per-spin orbital masks: symmask[(sym*2+ims)*nw + w]
    uint64_t symmask[kMaxSym * 2 * kMaxWords];
    int nbss[kMaxSym * 2];  // orbitals per (sym, ims): index sym*2+ims
    uint8_t orbsym[64 * kMaxWords];  // irrep of each spin orbital
    // heat-bath generator tables (hgpu_heat_bath.h); element type double, or
    // float in the mixed-precision mode
    const void *hb_i_w, *hb_ij_w, *hb_ija_w, *hb_ija_tot, *hb_ija_U, *hb_ijab_tot, *hb_ijab_U;
    const uint8_t *hb_ija_K, *hb_ijab_K;
    // uniform_power_pitzer / uniform_cauchy_schwarz: w(p, q) = sqrt|<pq|qp>| or
    // sqrt|<pq|pq>|, [nbasis][nbasis]
    const double *pp_w;
    // heat_bath_power_pitzer_ref: six weight / alias tables (hgpu_power_pitzer.h,
    // index PPN_*), row r entry k at r * ppn_stride[t] + k
    const double *ppn_w[6], *ppn_U[6], *ppn_tot[6];
    const uint8_t *ppn_K[6];
    int ppn_stride[6];
};

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of the published round function and Weyl key
// schedule.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t lo0 = 0xD2511F53u * c[0];
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
        uint32_t lo1 = 0xCD9E8D57u * c[2];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// One Philox block, out of line: every draw of a generator goes through this
// single copy of the ten rounds instead of an inlined copy per call site.
static __device__ __noinline__ uint4 philox_block(uint4 c, uint32_t k0, uint32_t k1) {
    uint32_t w[4] = {c.x, c.y, c.z, c.w};
    philox(w, k0, k1);
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// k * 2^-53 for k < 2^53, built from its bit pattern on the integer pipes
// (the value is exact, so this is the same number the conversion gives).
__device__ __forceinline__ double kdouble(uint64_t k) {
    if (k == 0) return 0.0;
    int msb = 63 - __clzll((long long)k);
    uint64_t man = (k << (52 - msb)) & ((1ull << 52) - 1);
    uint64_t bits = ((uint64_t)(msb - 53 + 1023) << 52) | man;
    return __longlong_as_double((long long)bits);
}

// The 53-bit integer k of the uniform u = k * 2^-53 drawn from two Philox words.
__device__ __forceinline__ uint64_t k53(uint32_t hi, uint32_t lo) { return (((uint64_t)hi << 32) | lo) >> 11; }

// (double)(x >> 11) * 2^-53 of the 64-bit word x = hi:lo.
__device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) { return kdouble(k53(hi, lo)); }

// Stream of uniforms in [0,1) for one (purpose, space, index, sub, iteration):
// counter = (index, sub, iteration, purpose<<28 | space<<26 | block).
struct RStream {
    uint32_t c0, c1, c2, c3;
    uint32_t k0, k1;
    uint32_t block;
    uint64_t bufk;
    bool have;

    __device__ __forceinline__ void init(uint64_t seed, uint32_t purpose, uint32_t space, uint64_t idx,
                                         uint64_t sub, uint64_t iter) {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        c0 = (uint32_t)idx;
        c1 = (uint32_t)sub;
        c2 = (uint32_t)iter;
        c3 = (purpose << 28) | (space << 26);
        block = 0;
        have = false;
    }
    // The next uniform as its integer k (u = k * 2^-53), for comparisons and
    // products that are exact in integer arithmetic.
    __device__ __forceinline__ uint64_t next_k() {
        if (have) {
            have = false;
            return bufk;
        }
        const uint4 c = philox_block(make_uint4(c0, c1, c2, c3 | block), k0, k1);
        block++;
        bufk = k53(c.z, c.w);
        have = true;
        return k53(c.x, c.y);
    }
    // get_rand_close_open
    __device__ __forceinline__ double next() { return kdouble(next_k()); }
};

// ---------------------------------------------------------------------------
// Determinant bit operations
// ---------------------------------------------------------------------------
template <int W>
struct Det {
    uint64_t w[W];
};

template <int W>
__device__ __forceinline__ bool tbit(const Det<W> &f, int p) {
    return (f.w[p >> 6] >> (p & 63)) & 1ull;
}

template <int W>
__device__ __forceinline__ int popc(const Det<W> &f) {
    int n = 0;
#pragma unroll
    for (int i = 0; i < W; i++) n += __popcll(f.w[i]);
    return n;
}

// Unsigned comparison with the last word most significant (bit_str_cmp).
template <int W>
__device__ __forceinline__ bool det_less(const Det<W> &a, const Det<W> &b) {
#pragma unroll
    for (int i = W - 1; i >= 0; i--) {
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i];
    }
    return false;
}

template <int W>
__device__ __forceinline__ bool det_eq(const Det<W> &a, const Det<W> &b) {
    bool e = true;
#pragma unroll
    for (int i = 0; i < W; i++) e = e && (a.w[i] == b.w[i]);
    return e;
}

// Position of the r-th (0-based) set bit of x; x has more than r set bits.
__device__ __forceinline__ int select64(uint64_t x, int r) {
    int base = 0;
    uint32_t lo = (uint32_t)x;
    int c = __popc(lo);
    uint32_t v;
    if (r >= c) {
        r -= c;
        v = (uint32_t)(x >> 32);
        base = 32;
    } else {
        v = lo;
    }
    uint32_t l16 = v & 0xFFFFu;
    c = __popc(l16);
    if (r >= c) {
        r -= c;
        v >>= 16;
        base += 16;
    }
    uint32_t l8 = v & 0xFFu;
    c = __popc(l8);
    if (r >= c) {
        r -= c;
        v >>= 8;
        base += 8;
    }
    // at most 8 candidate bits left
    v &= 0xFFu;
    for (;;) {
        int t = __ffs(v) - 1;
        if (r == 0) return base + t;
        v &= v - 1;
        r--;
    }
}

// r-th set bit of a W-word mask m (occupied-orbital list occ(r), etc.).
template <int W>
__device__ __forceinline__ int select_det(const uint64_t *m, int r) {
#pragma unroll
    for (int i = 0; i < W; i++) {
        int c = __popcll(m[i]);
        if (r < c) return 64 * i + select64(m[i], r);
        r -= c;
    }
    return -1;
}

constexpr uint64_t kAlpha = 0x5555555555555555ull;  // even bits
constexpr uint64_t kBeta = 0xAAAAAAAAAAAAAAAAull;

// Orbitals strictly above p (excit_mask(:, p), src/excitations.F90:25-70), word i.
__device__ __forceinline__ uint64_t above_mask(int p, int i) {
    int wp = p >> 6;
    if (i < wp) return 0ull;
    if (i > wp) return ~0ull;
    int b = p & 63;
    return b == 63 ? 0ull : (~0ull << (b + 1));
}

// find_excitation_permutation1 (src/excitations.F90:247-280).
template <int W>
__device__ __forceinline__ bool perm1(const Det<W> &f, int i, int a) {
    int perm = 0;
#pragma unroll
    for (int k = 0; k < W; k++) perm += __popcll(f.w[k] & (above_mask(i, k) ^ above_mask(a, k)));
    if (i > a) perm -= 1;
    return (perm & 1) != 0;
}

// find_excitation_permutation2 (src/excitations.F90:282-330).
template <int W>
__device__ __forceinline__ bool perm2(const Det<W> &f, int i, int j, int a, int b) {
    int perm = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        uint64_t ia = above_mask(i, k) ^ above_mask(a, k);
        uint64_t jb = above_mask(j, k) ^ above_mask(b, k);
        perm += __popcll((f.w[k] & ia) ^ (f.w[k] & jb));
    }
    if (i > a) perm += 1;
    if (i > b) perm += 1;
    if (j > b || j < a) perm += 1;
    return (perm & 1) != 0;
}

// get_excitation (src/excitations.F90:75-200) for D (f1) against the reference
// (f2): from = in f1 not in f2, to = in f2 not in f1, both ascending; perm is
// the parity of sum(shift - iel + iexcit) over the excited orbitals, which
// equals the parity computed below from the number of electrons of each
// determinant below each excited orbital.
struct Excit {
    int nexcit;
    int from[2], to[2];
    bool perm;
};

template <int W>
__device__ __forceinline__ Excit get_excitation(const Det<W> &f1, const Det<W> &f2, int nel) {
    Excit e;
    e.nexcit = 0;
    e.from[0] = e.from[1] = e.to[0] = e.to[1] = -1;
    e.perm = false;
    int diff = 0;
#pragma unroll
    for (int k = 0; k < W; k++) diff += __popcll(f1.w[k] ^ f2.w[k]);
    if (diff == 0) return e;
    e.nexcit = diff >> 1;
    if (e.nexcit > 2) return e;
    int shift = nel - e.nexcit;
    int n1 = 0, n2 = 0;
    int perm = 0;
    // Each excited orbital p in f1 only: iel1 = (# f1 electrons <= p), iexcit1 = its rank.
#pragma unroll
    for (int k = 0; k < W; k++) {
        uint64_t d1 = f1.w[k] & ~f2.w[k];
        uint64_t d2 = f2.w[k] & ~f1.w[k];
        while (d1) {
            int b = __ffsll((long long)d1) - 1;
            d1 &= d1 - 1;
            uint64_t below = b == 63 ? ~0ull : ((1ull << (b + 1)) - 1);
            int iel1 = 0;
#pragma unroll
            for (int q = 0; q < W; q++) iel1 += q < k ? __popcll(f1.w[q]) : (q == k ? __popcll(f1.w[q] & below) : 0);
            e.from[n1] = 64 * k + b;
            n1++;
            perm += shift - iel1 + n1;
        }
        while (d2) {
            int b = __ffsll((long long)d2) - 1;
            d2 &= d2 - 1;
            uint64_t below = b == 63 ? ~0ull : ((1ull << (b + 1)) - 1);
            int iel2 = 0;
#pragma unroll
            for (int q = 0; q < W; q++) iel2 += q < k ? __popcll(f2.w[q]) : (q == k ? __popcll(f2.w[q] & below) : 0);
            e.to[n2] = 64 * k + b;
            n2++;
            perm += shift - iel2 + n2;
        }
    }
    e.perm = (perm & 1) != 0;
    return e;
}

// ---------------------------------------------------------------------------
// Integrals
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t tri0(int64_t i, int64_t j) { return i * (i + 1) / 2 + j; }

// two_body_int_indx (src/molecular_integrals.F90:736-845), RHF, spin orbitals.
__device__ __forceinline__ int64_t v2_index(int i, int j, int a, int b) {
    int si = i >> 1, sj = j >> 1, sa = a >> 1, sb = b >> 1;
    int64_t ia = si >= sa ? tri0(si, sa) : tri0(sa, si);
    int64_t jb = sj >= sb ? tri0(sj, sb) : tri0(sb, sj);
    return ia >= jb ? tri0(ia, jb) : tri0(jb, ia);
}

template <typename Real>
struct Ints;

template <>
struct Ints<double> {
    __device__ __forceinline__ static double v2(const DevSys &s, int i, int j, int a, int b) {
        return __ldg(&s.v2[v2_index(i, j, a, b)]);
    }
    __device__ __forceinline__ static double h1(const DevSys &s, int i, int a) {
        return __ldg(&s.h1[(i >> 1) * s.norb + (a >> 1)]);
    }
};

template <>
struct Ints<float> {
    __device__ __forceinline__ static float v2(const DevSys &s, int i, int j, int a, int b) {
        return __ldg(&s.v2f[v2_index(i, j, a, b)]);
    }
    __device__ __forceinline__ static float h1(const DevSys &s, int i, int a) {
        return __ldg(&s.h1f[(i >> 1) * s.norb + (a >> 1)]);
    }
};

__device__ __forceinline__ int ms_of(int p) { return (p & 1) ? -1 : 1; }
__device__ __forceinline__ int ims_of(int p) { return (p & 1) ? 0 : 1; }  // 0 beta, 1 alpha

// Exact diagonal energy E(D) in units of 2^-fx_shift (hgpu_fixed.h): the terms of
// slater_condon0_mol (src/hamiltonian_molecular.f90:73-139) -- Ecore, h_ii,
// (ii|jj) and, for parallel spins, -(ij|ji) -- or of slater_condon0_hub_k
// (src/hamiltonian_hub_k.f90:91-132) -- nalpha*nbeta*U/N and the
// single-particle energies -- accumulated in 64-bit integers.
// The even bits of x (bits 0, 2, 4, ...) packed into the low 32 bits: the
// spatial orbitals of one spin of a determinant word.
__device__ __forceinline__ uint64_t unzip_even(uint64_t x) {
    x &= 0x5555555555555555ull;
    x = (x | (x >> 1)) & 0x3333333333333333ull;
    x = (x | (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x >> 4)) & 0x00FF00FF00FF00FFull;
    x = (x | (x >> 8)) & 0x0000FFFF0000FFFFull;
    x = (x | (x >> 16)) & 0x00000000FFFFFFFFull;
    return x;
}

// The tables (fx_h1, fx_pair, fx_eps) are passed explicitly so that a kernel can
// read them from a shared-memory copy (FxTabs).
struct FxTabs {
    const int64_t *h1, *pair, *eps;
};

__device__ __forceinline__ FxTabs fx_tabs(const DevSys &s) { return FxTabs{s.fx_h1, s.fx_pair, s.fx_eps}; }

// Words of the exact-diagonal tables: eps[nbasis] (hub_k) or h1[norb] + pair[2 norb^2].
__host__ __device__ __forceinline__ int fx_table_words(int kind, int nbasis, int norb) {
    return kind == HGPU_SYS_HUB_K ? nbasis : norb + 2 * norb * norb;
}

// Copies the exact-diagonal tables into dst (fx_table_words entries) with the
// whole block; the caller synchronises before use.
__device__ __forceinline__ FxTabs stage_fx(const DevSys &s, int64_t *dst) {
    if (s.kind == HGPU_SYS_HUB_K) {
        for (int k = threadIdx.x; k < s.nbasis; k += blockDim.x) dst[k] = s.fx_eps[k];
        return FxTabs{nullptr, nullptr, dst};
    }
    const int M = s.norb;
    for (int k = threadIdx.x; k < M; k += blockDim.x) dst[k] = s.fx_h1[k];
    for (int k = threadIdx.x; k < 2 * M * M; k += blockDim.x) dst[M + k] = s.fx_pair[k];
    return FxTabs{dst, dst + M, nullptr};
}

__device__ __forceinline__ int low_bit(uint32_t x) { return __ffs((int)x) - 1; }
__device__ __forceinline__ int low_bit(uint64_t x) { return __ffsll((long long)x) - 1; }

// One-electron and pair terms of the exact diagonal for alpha and beta
// spatial occupation masks.
template <typename Mask>
__device__ __forceinline__ int64_t fx_pair_sum(const FxTabs &tb, int M, Mask am, Mask bm) {
    int64_t e = 0;
    const int64_t *same_tab = tb.pair + (size_t)M * M;
    for (Mask x = am; x; x &= x - 1) {
        const int p = low_bit(x);
        e += tb.h1[p];
        const int64_t *opp = tb.pair + (size_t)p * M;
        const int64_t *same = same_tab + (size_t)p * M;
        for (Mask y = x & (x - 1); y; y &= y - 1) e += same[low_bit(y)];  // alpha partners above p
        for (Mask y = bm; y; y &= y - 1) e += opp[low_bit(y)];             // every beta partner
    }
    for (Mask x = bm; x; x &= x - 1) {
        const int p = low_bit(x);
        e += tb.h1[p];
        const int64_t *same = same_tab + (size_t)p * M;
        for (Mask y = x & (x - 1); y; y &= y - 1) e += same[low_bit(y)];  // beta partners above p
    }
    return e;
}

template <int W>
__device__ int64_t fx_energy(const DevSys &s, const Det<W> &f, const FxTabs &tb) {
    int64_t e = s.fx_const;
    if (s.kind == HGPU_SYS_HUB_K) {
#pragma unroll
        for (int k = 0; k < W; k++) {
            uint64_t x = f.w[k];
            while (x) {
                int p = 64 * k + __ffsll((long long)x) - 1;
                x &= x - 1;
                e += tb.eps[p];
            }
        }
        return e;
    }
    // Spin-resolved spatial occupations: every term is an integer, so the
    // pairs may be summed in any order -- alpha-alpha and beta-beta pairs from
    // the same-spin table, every alpha-beta pair (a doubly occupied orbital
    // included) from the opposite-spin table.  One determinant word holds at
    // most 32 spatial orbitals, whose masks are then 32-bit words.
    const int M = s.norb;
    uint64_t am = 0, bm = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        am |= unzip_even(f.w[k]) << (32 * k);
        bm |= unzip_even(f.w[k] >> 1) << (32 * k);
    }
    if (W == 1) return e + fx_pair_sum<uint32_t>(tb, M, (uint32_t)am, (uint32_t)bm);
    return e + fx_pair_sum<uint64_t>(tb, M, am, bm);
}

template <int W>
__device__ __forceinline__ int64_t fx_energy(const DevSys &s, const Det<W> &f) {
    return fx_energy<W>(s, f, fx_tabs(s));
}

// slater_condon0 (sc0_ptr): nearest double to the exact sum.
template <int W>
__device__ __forceinline__ double sc0(const DevSys &s, const Det<W> &f) {
    return fx_to_double(fx_energy<W>(s, f), s.fx_inv_scale);
}

// dat(1) of a new walker: K_ii = <D_i|H|D_i> - E_HF (src/annihilation.f90:855),
// the nearest double to the exact difference.
template <int W>
__device__ __forceinline__ double kii_of(const DevSys &s, const Det<W> &f, const FxTabs &tb) {
    return fx_to_double(fx_energy<W>(s, f, tb) - s.fx_E0, s.fx_inv_scale);
}

template <int W>
__device__ __forceinline__ double kii_of(const DevSys &s, const Det<W> &f) {
    return kii_of<W>(s, f, fx_tabs(s));
}

// slater_condon1_mol_excit (src/hamiltonian_molecular.f90:199-259).
// The integrals of four occupied orbitals at a time are loaded before any of
// them is added, so a determinant costs nel/4 memory round trips instead of
// nel; the additions stay in ascending orbital order, as the reference sums.
template <int W, typename Real>
__device__ Real sc1_mol(const DevSys &s, const Det<W> &f, int i, int a, bool perm) {
    constexpr int G = 4;
    Real h = Ints<Real>::h1(s, i, a);
#pragma unroll
    for (int k = 0; k < W; k++) {
        uint64_t x = f.w[k] & ~((k == (i >> 6)) ? (1ull << (i & 63)) : 0ull);  // q != i
        while (x) {
            int q[G];
            Real v[G], e[G];
#pragma unroll
            for (int u = 0; u < G; u++) {
                q[u] = x ? 64 * k + __ffsll((long long)x) - 1 : -1;
                x &= x - 1;
            }
#pragma unroll
            for (int u = 0; u < G; u++) {
                v[u] = (Real)0;
                e[u] = (Real)0;
                if (q[u] >= 0) {
                    v[u] = Ints<Real>::v2(s, i, q[u], a, q[u]);
                    if (((q[u] ^ i) & 1) == 0) e[u] = Ints<Real>::v2(s, i, q[u], q[u], a);
                }
            }
#pragma unroll
            for (int u = 0; u < G; u++) {
                if (q[u] >= 0) {
                    h = h + v[u];
                    if (((q[u] ^ i) & 1) == 0) h = h - e[u];
                }
            }
        }
    }
    if (perm) h = -h;
    return h;
}

// slater_condon2_mol_excit (src/hamiltonian_molecular.f90:300-346).
template <typename Real>
__device__ __forceinline__ Real sc2_mol(const DevSys &s, int i, int j, int a, int b, bool perm) {
    Real h = (Real)0;
    if (((i ^ a) & 1) == 0) h = Ints<Real>::v2(s, i, j, a, b);
    if (((i ^ b) & 1) == 0) h = h - Ints<Real>::v2(s, i, j, b, a);
    if (perm) h = -h;
    return h;
}

// ---------------------------------------------------------------------------
// Hubbard model in momentum space
// ---------------------------------------------------------------------------
struct HubTables {
    const uint8_t *sym;  // nk*nk (shared memory)
    const uint8_t *inv;  // nk
    int nk;
};

// get_two_e_int_hub_k (src/hubbard_k.f90:11-55) with momentum_conserved (:57-84).
__device__ __forceinline__ double two_e_int_hub_k(const DevSys &s, const HubTables &t, int p1, int p2, int p3,
                                                  int p4) {
    bool s12 = ((p1 ^ p2) & 1) == 0;
    bool s34 = ((p3 ^ p4) & 1) == 0;
    if (!s12 && (s12 == s34)) {
        int dk = t.sym[(p1 >> 1) * t.nk + (p2 >> 1)];
        dk = t.sym[dk * t.nk + t.inv[p3 >> 1]];
        if (dk == (p4 >> 1)) return ((p1 ^ p3) & 1) == 0 ? s.coulomb_k : -s.coulomb_k;
    }
    return 0.0;
}

// beta partner of alpha orbital a for total momentum ij_sym (find_ab_hub_k).
__device__ __forceinline__ int hub_partner(const HubTables &t, int ij_sym, int a) {
    return 2 * t.sym[ij_sym * t.nk + t.inv[a >> 1]] + 1;
}

// Result of one spawning attempt.
struct Attempt {
    int nexcit;
    int from[2], to[2];
    double pgen, hmatel;
    bool allowed;
    int64_t nspawn;
    int64_t nspawn_rdm;  // spawn_rdm's unweighted attempt (replica 2-RDM), 0 otherwise
};

// stochastic_round_spawned_particle (src/stoch_utils.f90:87-136).
// pspawn >= 0; the comparisons and the large-amplitude branch are evaluated in
// integer arithmetic with identical results (hgpu_exact.h).
__device__ __forceinline__ int64_t round_spawned(int64_t cutoff, double dcutoff, double pspawn, RStream &rs) {
    if (less_nonneg(dbits(pspawn), dbits(dcutoff))) return (pspawn > rs.next() * dcutoff) ? cutoff : 0;
    // nspawn = int(pspawn); if (pspawn - nspawn > rand) nspawn = nspawn + 1
    return round_up_frac(dbits(pspawn), rs.next_k());
}

__device__ __forceinline__ int64_t isign64(int64_t a, int64_t b) {
    int64_t m = a < 0 ? -a : a;
    return b >= 0 ? m : -m;
}

// set_child_sign (src/spawning.F90:680-709).
__device__ __forceinline__ int64_t child_sign(double hmatel, int64_t parent, int64_t nspawn) {
    return positive(dbits(hmatel)) ? -isign64(nspawn, parent) : isign64(nspawn, parent);  // hmatel > 0
}

// spawn_lattice_split_gen (src/spawning.F90:215-315) with gen_excit_init_hub_k /
// gen_excit_finalise_hub_k (src/excit_gen_hub_k.f90:29-156) or the no_renorm
// pair (:158-277).  complete: finish the excitation even when nothing spawns
// (parity evaluation only).
template <int W>
__device__ void attempt_hub_k(const DevSys &s, const HubTables &t, RStream &rs, const Det<W> &f, int64_t parent,
                              bool complete, Attempt &out) {
    out.nexcit = 2;
    out.to[0] = out.to[1] = -1;
    // occupied alpha / beta and unoccupied alpha masks
    uint64_t oa[W], ob[W], ua[W];
#pragma unroll
    for (int k = 0; k < W; k++) {
        uint64_t valid = (64 * (k + 1) <= s.nbasis) ? ~0ull : ((1ull << (s.nbasis - 64 * k)) - 1);
        oa[k] = f.w[k] & kAlpha;
        ob[k] = f.w[k] & kBeta;
        ua[k] = ~f.w[k] & kAlpha & valid;
    }
    // choose_ij_hub_k (src/excit_gen_hub_k.f90:469-532)
    int ind = floor_uab(rs.next_k(), s.nalpha, s.nbeta) + 1;  // int(rand * nalpha * nbeta) + 1
    // int((ind-1.0)/nbeta): exact for integers, so integer division gives it
    int ii = (ind - 1) / s.nbeta + 1;
    int jj = ind - (ii - 1) * s.nbeta;
    int i = select_det<W>(oa, ii - 1);
    int j = select_det<W>(ob, jj - 1);
    int ij_sym = t.sym[(i >> 1) * t.nk + (j >> 1)];
    out.from[0] = i;
    out.from[1] = j;
    bool renorm = s.excit_gen != HGPU_EXCIT_GEN_NO_RENORM;
    double pgen, abs_h;
    int a = -1, b = -1;
    int forbidden = 0;
    if (renorm) {
        // calc_pgen_hub_k (src/excit_gen_hub_k.f90:651-770)
#pragma unroll
        for (int k = 0; k < W; k++) {
            uint64_t x = ua[k];
            while (x) {
                int aa = 64 * k + __ffsll((long long)x) - 1;
                x &= x - 1;
                if (tbit<W>(f, hub_partner(t, ij_sym, aa))) forbidden++;
            }
        }
        // p_gen, the allowed test and p_spawn from tables of the same expressions
        pgen = s.hub_pgen[forbidden];
        out.allowed = s.hub_allowed[forbidden] != 0;
        abs_h = fabs(s.coulomb_k);
    } else {
        // find_ab_hub_k (src/excit_gen_hub_k.f90:579-649)
        int rr = floor_un(rs.next_k(), s.nvirt_alpha);  // int(rand * nvirt_alpha)
        a = select_det<W>(ua, rr);
        b = hub_partner(t, ij_sym, a);
        out.allowed = !tbit<W>(f, b);
        if (out.allowed) {
            pgen = s.hub_pgen_nr;
            abs_h = fabs(s.coulomb_k);
        } else {
            pgen = 1.0;
            abs_h = 0.0;
        }
    }
    out.pgen = pgen;
    double pspawn;
    if (renorm) pspawn = s.hub_pspawn[forbidden];
    else pspawn = out.allowed ? s.hub_pspawn_nr : 0.0;
    int64_t nspawn = round_spawned(s.cutoff, s.d_cutoff, pspawn, rs);
    if (nspawn != 0 || (complete && out.allowed)) {
        if (renorm) {
            // choose_ab_hub_k: redraw until b is unoccupied
            for (int it = 0;; it++) {
                int rr = floor_un(rs.next_k(), s.nvirt_alpha);
                a = select_det<W>(ua, rr);
                b = hub_partner(t, ij_sym, a);
                if (!tbit<W>(f, b)) break;
                if (it >= kMaxRedraw) {
                    out.nspawn = 0;
                    out.allowed = false;
                    return;
                }
            }
        }
        // slater_condon2_hub_k_excit (src/hamiltonian_hub_k.f90:163-234)
        int f0 = i < j ? i : j, f1 = i < j ? j : i;
        int t0 = a < b ? a : b, t1 = a < b ? b : a;
        out.from[0] = f0;
        out.from[1] = f1;
        out.to[0] = t0;
        out.to[1] = t1;
        double h = s.coulomb_k;
        if (perm2<W>(f, f0, f1, t0, t1)) h = -h;
        if (((f0 - t0) % 2) != 0) h = -h;
        out.hmatel = h;
        if (nspawn != 0) nspawn = child_sign(h, parent, nspawn);
    } else {
        out.to[0] = a;
        out.to[1] = b;
        out.hmatel = abs_h;
    }
    out.nspawn = nspawn;
}

// ---------------------------------------------------------------------------
// Molecular uniform generators (src/excit_gen_mol.f90)
// ---------------------------------------------------------------------------
// Per-determinant view: occupied mask and unoccupied counts per (sym, ims).
template <int W>
struct MolDet {
    Det<W> f;
    uint64_t valid[W];
    int symunocc[kMaxSym * 2];  // index sym*2+ims
};

template <int W>
__device__ __forceinline__ void mol_decode(const DevSys &s, const Det<W> &f, MolDet<W> &d) {
    d.f = f;
#pragma unroll
    for (int k = 0; k < W; k++)
        d.valid[k] = (64 * (k + 1) <= s.nbasis) ? ~0ull : ((1ull << (s.nbasis - 64 * k)) - 1);
    for (int q = 0; q < 2 * s.nsym; q++) {
        int n = 0;
#pragma unroll
        for (int k = 0; k < W; k++) n += __popcll(~f.w[k] & s.symmask[q * W + k] & d.valid[k]);
        d.symunocc[q] = n;
    }
}

#define SU(d, ims, sym) ((d).symunocc[(sym)*2 + (ims)])

// ind-th orbital (0-based) of irrep sym with spin ims (sym_spin_basis_fns).
template <int W>
__device__ __forceinline__ int ssbf(const DevSys &s, int ims, int sym, int ind) {
    return select_det<W>(&s.symmask[(sym * 2 + ims) * W], ind);
}

__device__ __forceinline__ int xsym(const DevSys &s, int a, int b) { return (a ^ b) & (s.nsym - 1); }

template <int W>
__device__ __forceinline__ int sym_of(const DevSys &s, int p) {
    return s.orbsym[p];
}

// int(rand * nbasis) or the spin-restricted int(rand * nbasis/2), u = k 2^-53.
template <int W>
__device__ __forceinline__ int pick_a(const DevSys &s, int spin, uint64_t ku) {
    if (spin == 0) return floor_un(ku, s.nbasis);
    int k = floor_un(ku, s.nbasis / 2);
    return spin == -2 ? 2 * k + 1 : 2 * k;
}

// p_gen of a double excitation, pattempt_double * 2/(nel(nel-1)) * (1/n_aij) *
// (1/xb + 1/xa) in the reference's rounding order, read from a table the host
// fills with exactly that expression (DevSys::pg2; symmetric in xa, xb).
__device__ __forceinline__ double pgen_double(const DevSys &s, int cls, int n_aij, int xa, int xb) {
    return __ldg(&s.pg2[(((size_t)cls * s.pg2_n + n_aij) * s.pg2_x + xa) * s.pg2_x + xb]);
}

// choose_ij_spin_mol (src/excit_gen_mol.f90:684-783): parallel spins with
// probability pattempt_parallel (alpha-alpha with probability nalpha/nel), else
// one alpha and one beta electron; false when the class has too few electrons.
// cls: 0 opposite spins, 1 alpha-alpha, 2 beta-beta (the p_gen table class).
template <int W>
__device__ __forceinline__ bool choose_ij_spin(const DevSys &s, RStream &rs, const Det<W> &f, int &i, int &j,
                                               int &cls) {
    Det<W> ma, mb;
#pragma unroll
    for (int w = 0; w < W; w++) {
        ma.w[w] = f.w[w] & kAlpha;
        mb.w[w] = f.w[w] & kBeta;
    }
    if (rs.next_k() < s.t_parallel) {
        const bool alpha = rs.next_k() < s.t_alpha;
        const int n = alpha ? s.nalpha : s.nbeta;
        if (n < 2) return false;
        // int(rand * real(n(n-1)) / 2): the product rounded once, halved exactly
        const int ind = floor_un(rs.next_k(), n * (n - 1)) / 2 + 1;
        int j_ind = (int)(1.5f + sqrtf((float)(2 * ind) - 1.75f));
        while (j_ind * (j_ind - 1) / 2 < ind) j_ind++;
        while ((j_ind - 1) * (j_ind - 2) / 2 >= ind) j_ind--;
        const int i_ind = ind - ((j_ind - 1) * (j_ind - 2)) / 2;
        const Det<W> &m = alpha ? ma : mb;
        i = select_det<W>(m.w, i_ind - 1);
        j = select_det<W>(m.w, j_ind - 1);
        cls = alpha ? 1 : 2;
    } else {
        if (s.nbeta < 1 || s.nalpha < 1) return false;
        const int i_ind = floor_un(rs.next_k(), s.nalpha) + 1;
        const int j_ind = floor_un(rs.next_k(), s.nbeta) + 1;
        i = select_det<W>(ma.w, i_ind - 1);
        j = select_det<W>(mb.w, j_ind - 1);
        if (j < i) {
            const int t = i;
            i = j;
            j = t;
        }
        cls = 0;
    }
    return true;
}

// choose_ij_mol (src/excit_gen_mol.f90:620-660): a uniform pair of occupied
// orbitals, i < j.
template <int W>
__device__ __forceinline__ void choose_ij_uniform(const DevSys &s, RStream &rs, const Det<W> &f, int &i, int &j) {
    const int ind = floor_uab_half(rs.next_k(), s.nel, s.nel - 1) + 1;  // int(rand * nel * (nel-1) / 2) + 1
    // int(1.5 + sqrt(2 ind - 1.75)) is exactly the j with
    // (j-1)(j-2)/2 < ind <= j(j-1)/2; found here in integer arithmetic
    int j_ind = (int)(1.5f + sqrtf((float)(2 * ind) - 1.75f));
    while (j_ind * (j_ind - 1) / 2 < ind) j_ind++;
    while ((j_ind - 1) * (j_ind - 2) / 2 >= ind) j_ind--;
    const int i_ind = ind - ((j_ind - 1) * (j_ind - 2)) / 2;
    i = select_det<W>(f.w, i_ind - 1);
    j = select_det<W>(f.w, j_ind - 1);
}

// attempt_to_spawn (src/spawning.F90:711-768).
__device__ __forceinline__ void attempt_to_spawn(const DevSys &s, RStream &rs, int64_t parent, double pgen, double h,
                                                 Attempt &out) {
    out.pgen = pgen;
    out.hmatel = h;
    double pspawn = s.tau * fabs(h) / pgen;
    pspawn = pspawn * s.d_real_factor;
    int64_t nspawn = round_spawned(s.cutoff, s.d_cutoff, pspawn, rs);
    if (nspawn > 0) nspawn = child_sign(h, parent, nspawn);
    out.nspawn = nspawn;
}

// spawn_rdm's second attempt (src/spawning.F90:664-671): attempt_to_spawn with
// tau = 1 and hmatel = -1, drawn after the spawn itself, for the replica
// sampling of the 2-RDM.
__device__ __forceinline__ void attempt_to_spawn_rdm(const DevSys &s, RStream &rs, int64_t parent, Attempt &out) {
    out.nspawn_rdm = 0;
    if (!out.allowed) return;
    double p = 1.0 * fabs(-1.0) / out.pgen;
    p = p * s.d_real_factor;
    int64_t n = round_spawned(s.cutoff, s.d_cutoff, p, rs);
    if (n > 0) n = child_sign(-1.0, parent, n);
    out.nspawn_rdm = n;
}

// gen_single_excit_mol / gen_single_excit_mol_no_renorm (src/excit_gen_mol.f90:384-519):
// one single excitation with its p_gen and matrix element.
template <int W, typename Real>
__device__ __forceinline__ void gen_single_mol(const DevSys &s, RStream &rs, const MolDet<W> &d, bool renorm,
                                               Attempt &out, double &pgen, Real &hm) {
    const Det<W> &f = d.f;
    out.nexcit = 1;
    int i = -1, a = -1;
    bool ok;
    if (renorm) {
        // choose_ia_mol (src/excit_gen_mol.f90:521-618)
        ok = false;
        for (int k = 0; k < s.nel; k++) {
            int p = select_det<W>(f.w, k);
            if (SU(d, ims_of(p), sym_of<W>(s, p)) != 0) {
                ok = true;
                break;
            }
        }
        if (ok) {
            int guard = 0;
            for (;;) {
                i = select_det<W>(f.w, floor_un(rs.next_k(), s.nel));  // int(rand * nel)
                int imsa = ims_of(i), isyma = sym_of<W>(s, i);
                if (SU(d, imsa, isyma) != 0) {
                    for (;;) {
                        int ind = floor_un(rs.next_k(), s.nbss[isyma * 2 + imsa]);  // int(nbss * rand)
                        a = ssbf<W>(s, imsa, isyma, ind);
                        if (!tbit<W>(f, a) || ++guard > kMaxRedraw) break;
                    }
                    break;
                }
                if (++guard > kMaxRedraw) break;
            }
            if (guard > kMaxRedraw) ok = false;
        }
    } else {
        // find_ia_mol (src/excit_gen_mol.f90:950-1016)
        i = select_det<W>(f.w, floor_un(rs.next_k(), s.nel));
        int imsa = ims_of(i), isyma = sym_of<W>(s, i);
        int nb = s.nbss[isyma * 2 + imsa];
        int ind = floor_un(rs.next_k(), nb);
        if (nb == 0) {
            ok = false;
        } else {
            a = ssbf<W>(s, imsa, isyma, ind);
            ok = !tbit<W>(f, a);
        }
    }
    out.allowed = ok;
    out.from[0] = i;
    out.to[0] = ok ? a : -1;
    if (ok) {
        double pg;
        if (renorm) {
            // calc_pgen_single_mol (src/excit_gen_mol.f90:1140-1200)
            int ni = s.nel;
            for (int k = 0; k < s.nel; k++) {
                int p = select_det<W>(f.w, k);
                if (SU(d, ims_of(p), sym_of<W>(s, p)) == 0) ni--;
            }
            pg = s.inv[ni * SU(d, ims_of(a), sym_of<W>(s, a))];
        } else {
            pg = s.inv[s.nel * s.nbss[sym_of<W>(s, a) * 2 + ims_of(a)]];
        }
        pgen = s.pattempt_single * pg;
        hm = sc1_mol<W, Real>(s, f, i, a, perm1<W>(f, i, a));
    } else {
        hm = (Real)0;
        pgen = 1.0;
    }
}

// gen_excit_mol / gen_excit_mol_no_renorm, double branch (src/excit_gen_mol.f90:16-101,
// :195-284): one double excitation with its p_gen and matrix element.
template <int W, typename Real>
__device__ __forceinline__ void gen_double_mol(const DevSys &s, RStream &rs, const MolDet<W> &d, bool renorm,
                                               Attempt &out, double &pgen, Real &hm) {
    const Det<W> &f = d.f;
    out.nexcit = 2;
    int i, j, cls = 0;
    if (s.spin_ij) {
        if (!choose_ij_spin<W>(s, rs, f, i, j, cls)) {
            out.from[0] = out.from[1] = -1;
            out.allowed = false;
            hm = (Real)0;
            pgen = 1.0;
            return;
        }
    } else {
        choose_ij_uniform<W>(s, rs, f, i, j);
    }
    int ij_sym = xsym(s, sym_of<W>(s, i), sym_of<W>(s, j));
    int ij_spin = ms_of(i) + ms_of(j);
    out.from[0] = i;
    out.from[1] = j;
    int a = -1, b = -1;
    bool ok = false;
    if (renorm) {
        // choose_ab_mol (src/excit_gen_mol.f90:802-948)
        int is = ij_spin == -2 ? 0 : 1;
        for (int isyma = 0; isyma < s.nsym; isyma++) {
            int isymb = xsym(s, isyma, ij_sym);
            if (ij_spin == 0) {
                if ((SU(d, 0, isyma) > 0 && SU(d, 1, isymb) > 0) || (SU(d, 1, isyma) > 0 && SU(d, 0, isymb) > 0)) {
                    ok = true;
                    break;
                }
            } else if (SU(d, is, isyma) > 0 &&
                       (SU(d, is, isymb) > 1 || (SU(d, is, isymb) == 1 && isyma != isymb))) {
                ok = true;
                break;
            }
        }
        if (ok) {
            int guard = 0;
            for (;;) {
                a = pick_a<W>(s, ij_spin, rs.next_k());
                if (!tbit<W>(f, a)) {
                    int imsb = (ij_spin - ms_of(a) + 3) / 2 - 1;
                    int syma = sym_of<W>(s, a);
                    int isymb = xsym(s, ij_sym, syma);
                    int nu = SU(d, imsb, isymb);
                    if (nu > 1 || (nu == 1 && (isymb != syma || ij_spin == 0))) {
                        for (;;) {
                            int k = floor_un(rs.next_k(), s.nbss[isymb * 2 + imsb]);
                            b = ssbf<W>(s, imsb, isymb, k);
                            if ((b != a && !tbit<W>(f, b)) || ++guard > kMaxRedraw) break;
                        }
                        break;
                    }
                }
                if (++guard > kMaxRedraw) break;
            }
            if (guard > kMaxRedraw) ok = false;
            if (a > b) {
                int tt = a;
                a = b;
                b = tt;
            }
        }
    } else {
        // find_ab_mol (src/excit_gen_mol.f90:1018-1138)
        for (int it = 0;; it++) {
            a = pick_a<W>(s, ij_spin, rs.next_k());
            if (!tbit<W>(f, a) || it >= kMaxRedraw) break;
        }
        int imsb = (ij_spin - ms_of(a) + 3) / 2 - 1;
        int syma = sym_of<W>(s, a);
        int isymb = xsym(s, ij_sym, syma);
        int nb = s.nbss[isymb * 2 + imsb];
        if (nb == 0) {
            ok = false;
        } else if (ij_spin != 0 && isymb == syma && nb == 1) {
            ok = false;
        } else {
            for (int it = 0;; it++) {
                int k = floor_un(rs.next_k(), s.nbss[isymb * 2 + imsb]);
                b = ssbf<W>(s, imsb, isymb, k);
                if (b != a || it >= kMaxRedraw) break;
            }
            ok = b != a && !tbit<W>(f, b);
            if (a > b) {
                int tt = a;
                a = b;
                b = tt;
            }
        }
    }
    out.allowed = ok;
    if (ok) {
        out.to[0] = a;
        out.to[1] = b;
        int imsa = ims_of(a), imsb = ims_of(b), syma = sym_of<W>(s, a), symb = sym_of<W>(s, b);
        if (renorm) {
            // calc_pgen_double_mol (src/excit_gen_mol.f90:1202-1327)
            int n_aij, xa, xb;
            if (ij_spin == 0) {
                n_aij = s.nvirt;
                for (int isyma = 0; isyma < s.nsym; isyma++) {
                    int isymb = xsym(s, isyma, ij_sym);
                    if (SU(d, 0, isymb) == 0) n_aij -= SU(d, 1, isyma);
                    if (SU(d, 1, isymb) == 0) n_aij -= SU(d, 0, isyma);
                }
                xa = SU(d, imsa, syma);
                xb = SU(d, imsb, symb);
            } else {
                int is = ij_spin == -2 ? 0 : 1;
                n_aij = ij_spin == -2 ? s.nvirt_beta : s.nvirt_alpha;
                for (int isyma = 0; isyma < s.nsym; isyma++) {
                    int isymb = xsym(s, isyma, ij_sym);
                    if (SU(d, is, isymb) == 0)
                        n_aij -= SU(d, is, isyma);
                    else if (isyma == isymb && SU(d, is, isymb) == 1)
                        n_aij -= SU(d, is, isyma);
                }
                int same = syma == symb ? 1 : 0;
                xa = SU(d, imsa, syma) - same;
                xb = SU(d, imsb, symb) - same;
            }
            // p_aijb = 1/xa, p_bija = 1/xb
            pgen = pgen_double(s, cls, n_aij, xa, xb);
        } else {
            // calc_pgen_double_mol_no_renorm (src/excit_gen_mol.f90:1368-1445)
            int n_aij = ij_spin == -2 ? s.nvirt_beta : (ij_spin == 0 ? s.nvirt : s.nvirt_alpha);
            int same = (syma == symb && imsa == imsb) ? 1 : 0;
            pgen = pgen_double(s, cls, n_aij, s.nbss[syma * 2 + imsa] - same, s.nbss[symb * 2 + imsb] - same);
        }
        hm = sc2_mol<Real>(s, i, j, a, b, perm2<W>(f, i, j, a, b));
    } else {
        hm = (Real)0;
        pgen = 1.0;
    }
}

template <int W>
__device__ void gen_pp_occ_double(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                                  double &hm);
template <int W>
__device__ void gen_ppn_single(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                               double &hm);
template <int W>
__device__ void gen_ppn_double(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                               double &hm);

template <int W, typename Real>
__device__ void attempt_mol(const DevSys &s, RStream &rs, const MolDet<W> &d, int64_t parent, Attempt &out) {
    out.from[0] = out.from[1] = out.to[0] = out.to[1] = -1;
    const bool pp = s.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC || s.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC ||
                    s.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
                    s.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ;
    bool renorm = s.excit_gen == HGPU_EXCIT_GEN_RENORM || s.excit_gen == HGPU_EXCIT_GEN_RENORM_SPIN || pp;
    double pgen;
    Real hm;
    if (s.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN) {
        double h;
        if (rs.next_k() < s.t_single) gen_ppn_single<W>(s, rs, d, out, pgen, h);
        else gen_ppn_double<W>(s, rs, d, out, pgen, h);
        hm = (Real)h;
    } else if (rs.next_k() < s.t_single) {
        gen_single_mol<W, Real>(s, rs, d, renorm, out, pgen, hm);  // rand < pattempt_single
    } else if (pp) {
        double h;
        gen_pp_occ_double<W>(s, rs, d, out, pgen, h);
        hm = (Real)h;
    } else {
        gen_double_mol<W, Real>(s, rs, d, renorm, out, pgen, hm);
    }
    attempt_to_spawn(s, rs, parent, pgen, (double)hm, out);
}

// ---------------------------------------------------------------------------
// Heat-bath generators (src/excit_gen_heat_bath_mol.F90), Real = double or float
// ---------------------------------------------------------------------------
constexpr int kHBMaxEl = 32;  // on-the-fly alias tables over the occupied orbitals

__device__ __forceinline__ double rabs(double x) { return fabs(x); }
__device__ __forceinline__ float rabs(float x) { return fabsf(x); }

// Typed view of the heat-bath tables (layout in hgpu_heat_bath.h).
template <typename Real>
struct HBView {
    const Real *i_w, *ij_w, *ija_w, *ija_tot, *ija_U, *ijab_tot, *ijab_U;
    const uint8_t *ija_K, *ijab_K;
    size_t nb;
    __device__ __forceinline__ explicit HBView(const DevSys &s)
        : i_w(static_cast<const Real *>(s.hb_i_w)), ij_w(static_cast<const Real *>(s.hb_ij_w)),
          ija_w(static_cast<const Real *>(s.hb_ija_w)), ija_tot(static_cast<const Real *>(s.hb_ija_tot)),
          ija_U(static_cast<const Real *>(s.hb_ija_U)), ijab_tot(static_cast<const Real *>(s.hb_ijab_tot)),
          ijab_U(static_cast<const Real *>(s.hb_ijab_U)), ija_K(s.hb_ija_K), ijab_K(s.hb_ijab_K),
          nb((size_t)s.nbasis) {}
    // ij_weights(j,i), hb_ija%weights(a,j,i), hb_ija%weights_tot(j,i), hb_ijab%weights_tot(a,j,i)
    __device__ __forceinline__ Real ij(int i, int j) const { return __ldg(&ij_w[i * nb + j]); }
    __device__ __forceinline__ Real ija(int i, int j, int a) const { return __ldg(&ija_w[(i * nb + j) * nb + a]); }
    __device__ __forceinline__ Real ija_t(int i, int j) const { return __ldg(&ija_tot[i * nb + j]); }
    __device__ __forceinline__ Real ijab_t(int i, int j, int a) const {
        return __ldg(&ijab_tot[(i * nb + j) * nb + a]);
    }
};

// h_ijab of init_excit_mol_heat_bath (src/excit_gen_heat_bath_mol.F90:131-152):
// |<ij|ab> - <ij|ba>| with i<j, a<b ordered, 0 for a disallowed excitation.  The
// same expression as the host table builder, so in FP64 it is the stored weight.
template <typename Real>
__device__ __forceinline__ Real hb_weight(const DevSys &s, int i, int j, int a, int b) {
    if (i == j || a == i || a == j || b == a || b == i || b == j) return (Real)0;
    int it = i < j ? i : j, jt = i < j ? j : i;
    int isymb = xsym(s, xsym(s, s.orbsym[it], s.orbsym[jt]), s.orbsym[a]);
    bool spin = (ms_of(it) == ms_of(a) && ms_of(jt) == ms_of(b)) || (ms_of(it) == ms_of(b) && ms_of(jt) == ms_of(a));
    if (!spin || s.orbsym[b] != isymb) return (Real)0;
    int at = a < b ? a : b, bt = a < b ? b : a;
    return rabs(sc2_mol<Real>(s, it, jt, at, bt, false));
}

// select_weighted_value (lib/local/alias.f90:62-98): generate_alias_tables
// (:100-184) over n <= CAP weights, then one draw.
template <typename Real, int CAP = kHBMaxEl>
__device__ __forceinline__ int hb_alias_select(RStream &rs, int n, const Real *w, Real tot) {
    Real U[CAP];
    uint8_t K[CAP], under[CAP], over[CAP];
    int nu = 0, no = 0;
    Real f = (Real)n / tot;
    for (int i = 0; i < n; i++) {
        Real u = w[i] * f;
        U[i] = u;
        if (u <= (Real)1) under[nu++] = (uint8_t)i;
        else over[no++] = (uint8_t)i;
        K[i] = (uint8_t)i;
    }
    while (no > 0 && nu > 0) {
        int ov = over[no - 1], un = under[nu - 1];
        K[un] = (uint8_t)ov;
        nu--;
        U[ov] = U[ov] - ((Real)1 - U[un]);
        if (U[ov] < (Real)1) {
            under[nu++] = over[no - 1];
            no--;
        }
    }
    double x = rs.next() * (double)n;
    int k = (int)x;
    x = x - (double)k;
    return x < (double)U[k] ? k : (int)K[k];
}

// select_weighted_value_precalc (lib/local/alias.f90:13-60) on a stored table.
template <typename Real>
__device__ __forceinline__ int hb_alias_draw(RStream &rs, int n, const Real *U, const uint8_t *K) {
    double x = rs.next() * (double)n;
    int k = (int)x;
    x = x - (double)k;
    return x < (double)__ldg(&U[k]) ? k : (int)__ldg(&K[k]);
}

// psingle of a single i -> a inside the heat-bath double branch
// (src/excit_gen_heat_bath_mol.F90:396-454): 0 if the single breaks spin or
// symmetry, |h_ia|/(W + |h_ia|) below W = hb_ijab%weights_tot, else 0.5.
template <int W, typename Real>
__device__ __forceinline__ Real hb_psingle(const DevSys &s, const Det<W> &f, int i, int a, Real wtot) {
    if (s.orbsym[a] != s.orbsym[i] || ms_of(a) != ms_of(i)) return (Real)0;
    Real h = rabs(sc1_mol<W, Real>(s, f, i, a, false));
    return h < wtot ? h / (wtot + h) : (Real)0.5;
}

// find_i_d_weights + select_ij_heat_bath (src/excit_gen_utils.f90:9-66, :142-167).
template <typename Real>
struct HBSel {
    uint8_t occ[kHBMaxEl];
    Real wi[kHBMaxEl], ijw[kHBMaxEl], jiw[kHBMaxEl];
    Real wi_tot, ij_tot, ji_tot;
    int i_ind, j_ind, i, j;
};

template <int W, typename Real>
__device__ __forceinline__ bool hb_select_ij(const DevSys &s, const HBView<Real> &hb, RStream &rs, const Det<W> &f,
                                             HBSel<Real> &q) {
    int n = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        uint64_t x = f.w[k];
        while (x && n < kHBMaxEl) {
            q.occ[n++] = (uint8_t)(64 * k + __ffsll((long long)x) - 1);
            x &= x - 1;
        }
    }
    const int nel = s.nel;
    q.wi_tot = (Real)0;
    for (int p = 0; p < nel; p++) {
        q.wi[p] = __ldg(&hb.i_w[q.occ[p]]);
        q.wi_tot = q.wi_tot + q.wi[p];
    }
    q.i_ind = hb_alias_select<Real>(rs, nel, q.wi, q.wi_tot);
    q.i = q.occ[q.i_ind];
    q.ij_tot = (Real)0;
    for (int p = 0; p < nel; p++) {
        q.ijw[p] = hb.ij(q.i, q.occ[p]);
        q.ij_tot = q.ij_tot + q.ijw[p];
    }
    q.j_ind = -1;
    q.j = -1;
    if (!(q.ij_tot > (Real)0)) return false;
    q.j_ind = hb_alias_select<Real>(rs, nel, q.ijw, q.ij_tot);
    q.j = q.occ[q.j_ind];
    q.ji_tot = (Real)0;
    for (int p = 0; p < nel; p++) {
        q.jiw[p] = hb.ij(q.j, q.occ[p]);
        q.ji_tot = q.ji_tot + q.jiw[p];
    }
    return true;
}

// ---------------------------------------------------------------------------
// uniform_ and heat_bath_power_pitzer / _cauchy_schwarz: the double
// excitations of gen_excit_mol_power_pitzer_occ
// (src/excit_gen_power_pitzer_mol.F90:1260-1547)
// ---------------------------------------------------------------------------

// create_weighted_excitation_list_mol (src/hamiltonian_molecular.f90:348-390):
// the weights w(p, q) of the set bits q of mask in ascending order (0 for
// q == skip) into w (when not null) and their sum in that order.
template <int W, int CAP>
__device__ __forceinline__ double pp_weights(const DevSys &s, int p, int skip, const uint64_t *mask, double *w) {
    const double *row = s.pp_w + (size_t)p * s.nbasis;
    double tot = 0.0;
    int n = 0;
#pragma unroll
    for (int k = 0; k < W; k++)
        for (uint64_t x = mask[k]; x; x &= x - 1) {
            const int q = 64 * k + __ffsll((long long)x) - 1;
            double v = 0.0;
            if (q != skip) {
                v = __ldg(&row[q]);
                tot = tot + v;
            }
            if (w != nullptr && n < CAP) w[n] = v;
            n++;
        }
    return tot;
}

// a from the determinant's unoccupied orbitals of i's spin, b from the orbitals
// of the spin and irrep that conserve both (a excluded), each through an alias
// table built for the attempt (select_weighted_value); for parallel spins p_gen
// adds the reverse order, b from i and a from j.  The weights of the reverse
// order are read from the table directly: ia_weights(b_ind_rev) = w(i, b) and
// ja_weights(a_ind_rev) = w(j, a), or 0 when a == b.
template <int W>
__device__ void gen_pp_occ_double(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                                  double &hm) {
    constexpr int CAP = 32 * W;  // orbitals of one spin
    const Det<W> &f = d.f;
    out.nexcit = 2;
    out.to[0] = out.to[1] = -1;
    out.allowed = false;
    hm = 0.0;
    pgen = 1.0;
    int i, j;
    double pgen_ij = s.pgen_ij;
    if (s.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ || s.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ) {
        // select_ij_heat_bath over ppm_i_d_weights / ppm_ij_d_weights
        HBView<double> hb(s);
        HBSel<double> q;
        const bool ok = hb_select_ij<W, double>(s, hb, rs, f, q);
        i = q.i;
        j = q.j;
        if (ok)
            pgen_ij = ((q.wi[q.i_ind] / q.wi_tot) * (q.ijw[q.j_ind] / q.ij_tot)) +
                      ((q.wi[q.j_ind] / q.wi_tot) * (q.jiw[q.i_ind] / q.ji_tot));
        if (j >= 0 && j < i) {
            const int t = j;
            j = i;
            i = t;
        }
        out.from[0] = i;
        out.from[1] = j;
        if (!ok) return;
    } else {
        choose_ij_uniform<W>(s, rs, f, i, j);
        out.from[0] = i;
        out.from[1] = j;
    }
    const int ij_sym = xsym(s, s.orbsym[i], s.orbsym[j]);
    const int ij_spin = ms_of(i) + ms_of(j);
    const uint64_t spin_mask = ms_of(i) > 0 ? kAlpha : kBeta;
    uint64_t um[W];
#pragma unroll
    for (int k = 0; k < W; k++) um[k] = ~f.w[k] & d.valid[k] & spin_mask;
    int nv = 0;
#pragma unroll
    for (int k = 0; k < W; k++) nv += __popcll(um[k]);
    if (nv == 0) return;
    double ia_w[CAP];
    const double ia_tot = pp_weights<W, CAP>(s, i, -1, um, ia_w);
    if (!(ia_tot > 0.0)) return;
    const int a_ind = hb_alias_select<double, CAP>(rs, nv, ia_w, ia_tot);
    const int a = select_det<W>(um, a_ind);
    const int isymb = xsym(s, ij_sym, s.orbsym[a]);
    const int imsb = (ij_spin - ms_of(a) + 1) / 2;  // 0 beta, 1 alpha
    const int nb = s.nbss[isymb * 2 + imsb];
    if (nb == 0) return;
    double jb_w[CAP];
    const double jb_tot = pp_weights<W, CAP>(s, j, a, &s.symmask[(isymb * 2 + imsb) * W], jb_w);
    if (!(jb_tot > 0.0)) return;
    const int b_ind = hb_alias_select<double, CAP>(rs, nb, jb_w, jb_tot);
    const int b = ssbf<W>(s, imsb, isymb, b_ind);
    if (tbit<W>(f, b)) return;
    double pg;
    if (ij_spin == 0) {
        pg = ia_w[a_ind] / ia_tot * jb_w[b_ind] / jb_tot;
    } else {
        const int isyma = xsym(s, ij_sym, isymb);
        const double ja_tot = pp_weights<W, CAP>(s, j, b, &s.symmask[(isyma * 2 + imsb) * W], nullptr);
        const double w_ib = __ldg(&s.pp_w[(size_t)i * s.nbasis + b]);
        const double w_ja = a == b ? 0.0 : __ldg(&s.pp_w[(size_t)j * s.nbasis + a]);
        pg = (ia_w[a_ind] * jb_w[b_ind]) / (ia_tot * jb_tot) + (w_ib * w_ja) / (ia_tot * ja_tot);
    }
    pgen = s.pattempt_double * pg * pgen_ij;
    out.allowed = true;
    out.to[0] = a < b ? a : b;
    out.to[1] = a < b ? b : a;
    hm = sc2_mol<double>(s, i, j, out.to[0], out.to[1], perm2<W>(f, i, j, out.to[0], out.to[1]));
}

// ---------------------------------------------------------------------------
// heat_bath_power_pitzer_ref (gen_excit_mol_power_pitzer_orderN,
// src/excit_gen_power_pitzer_mol.F90:941-1258)
// ---------------------------------------------------------------------------
constexpr int kPPN_IS = 0, kPPN_ID = 1, kPPN_IJD = 2, kPPN_IAS = 3, kPPN_IAD = 4, kPPN_JBD = 5;

// find_diff_ref_cdet (src/excit_gen_utils.f90:220-269): the reference's
// orbitals missing from the determinant (ascending) and the determinant's
// extra orbitals (ascending, then swapped forward so that each matches the
// spin of its hole, as the reference does).
struct RefMap {
    uint8_t hole[kHBMaxEl], part[kHBMaxEl];
    int nex;
};

template <int W>
__device__ __forceinline__ void ref_map_build(const DevSys &s, const Det<W> &f, RefMap &m) {
    int nh = 0, np = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        for (uint64_t x = s.f0[k] & ~f.w[k]; x && nh < kHBMaxEl; x &= x - 1)
            m.hole[nh++] = (uint8_t)(64 * k + __ffsll((long long)x) - 1);
        for (uint64_t x = f.w[k] & ~s.f0[k]; x && np < kHBMaxEl; x &= x - 1)
            m.part[np++] = (uint8_t)(64 * k + __ffsll((long long)x) - 1);
    }
    m.nex = nh < np ? nh : np;
    for (int ii = 0; ii < m.nex; ii++) {
        const int ms_ref = ms_of(m.hole[ii]);
        if (ms_ref != ms_of(m.part[ii])) {
            int jj = ii + 1;
            while (jj < m.nex && ms_ref != ms_of(m.part[jj])) jj++;
            if (jj < m.nex) {
                const uint8_t t = m.part[ii];
                m.part[ii] = m.part[jj];
                m.part[jj] = t;
            }
        }
    }
}

// ref_cdet_occ_list(pos): the determinant's orbital for position pos of the
// reference's occupied list.
template <int W>
__device__ __forceinline__ int ref_map(const DevSys &s, const RefMap &m, int pos) {
    const int orb = select_det<W>(s.f0, pos);
    for (int k = 0; k < m.nex; k++)
        if (m.hole[k] == orb) return m.part[k];
    return orb;
}

// Number of set bits of mask below bit p (the position of p in the ascending
// list the mask stands for).
template <int W>
__device__ __forceinline__ int rank_in_mask(const uint64_t *mask, int p) {
    int r = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        if (64 * k + 64 <= p) r += __popcll(mask[k]);
        else if (64 * k < p) r += __popcll(mask[k] & ((1ull << (p - 64 * k)) - 1));
    }
    return r;
}

__device__ __forceinline__ double ppn_w(const DevSys &s, int t, int r, int k) {
    return __ldg(&s.ppn_w[t][(size_t)r * s.ppn_stride[t] + k]);
}

__device__ __forceinline__ int ppn_draw(const DevSys &s, RStream &rs, int t, int r, int n) {
    const size_t off = (size_t)r * s.ppn_stride[t];
    return hb_alias_draw<double>(rs, n, s.ppn_U[t] + off, s.ppn_K[t] + off);
}

// Single excitation: i from the reference's list, a from i's (spin, irrep) table.
template <int W>
__device__ void gen_ppn_single(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                               double &hm) {
    const Det<W> &f = d.f;
    RefMap m;
    ref_map_build<W>(s, f, m);
    out.nexcit = 1;
    out.allowed = false;
    out.to[0] = -1;
    pgen = 1.0;
    hm = 0.0;
    const int i_ind = ppn_draw(s, rs, kPPN_IS, 0, s.nel);
    const int i = ref_map<W>(s, m, i_ind);
    out.from[0] = i;
    const int ims = (ms_of(i) + 1) / 2, sym = s.orbsym[i];
    const int na = s.nbss[sym * 2 + ims];
    if (na <= 0) return;
    const int a_ind = ppn_draw(s, rs, kPPN_IAS, i, na);
    const int a = ssbf<W>(s, ims, sym, a_ind);
    if (tbit<W>(f, a)) return;
    out.allowed = true;
    out.to[0] = a;
    pgen = (ppn_w(s, kPPN_IS, 0, i_ind) / __ldg(&s.ppn_tot[kPPN_IS][0])) *
           (ppn_w(s, kPPN_IAS, i, a_ind) / __ldg(&s.ppn_tot[kPPN_IAS][i]));
    pgen = s.pattempt_single * pgen;
    hm = sc1_mol<W, double>(s, f, i, a, perm1<W>(f, i, a));
}

// Double excitation: i, j positions of the reference's list mapped onto the
// determinant, a over all orbitals of i's spin, b over the (spin, irrep) that
// conserves both; p_gen adds the reverse order of a, b for parallel spins.
template <int W>
__device__ void gen_ppn_double(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                               double &hm) {
    const Det<W> &f = d.f;
    RefMap m;
    ref_map_build<W>(s, f, m);
    out.nexcit = 2;
    out.allowed = false;
    out.to[0] = out.to[1] = -1;
    pgen = 1.0;
    hm = 0.0;
    const int i_ind = ppn_draw(s, rs, kPPN_ID, 0, s.nel);
    int i = ref_map<W>(s, m, i_ind);
    const int j_ind = ppn_draw(s, rs, kPPN_IJD, i, s.nel);
    int j = ref_map<W>(s, m, j_ind);
    out.from[0] = i;
    out.from[1] = j;
    if (j == i) return;
    const double tot_id = __ldg(&s.ppn_tot[kPPN_ID][0]);
    double pg = (ppn_w(s, kPPN_ID, 0, i_ind) / tot_id) * (ppn_w(s, kPPN_IJD, i, j_ind) / __ldg(&s.ppn_tot[kPPN_IJD][i]));
    const int ij_spin = ms_of(i) + ms_of(j);
    pg = pg + ((ppn_w(s, kPPN_ID, 0, j_ind) / tot_id) * (ppn_w(s, kPPN_IJD, j, i_ind) / __ldg(&s.ppn_tot[kPPN_IJD][j])));
    if (j < i) {
        const int t = j;
        j = i;
        i = t;
    }
    out.from[0] = i;
    out.from[1] = j;
    const int a_ind = ppn_draw(s, rs, kPPN_IAD, i, s.nbasis / 2);
    const int a = 2 * a_ind + (ms_of(i) > 0 ? 0 : 1);
    if (tbit<W>(f, a)) return;
    const int ij_sym = xsym(s, s.orbsym[i], s.orbsym[j]);
    const int isymb = xsym(s, ij_sym, s.orbsym[a]);
    const int imsb = (ms_of(j) + 1) / 2;
    const int nbb = s.nbss[isymb * 2 + imsb];
    if (nbb == 0) return;
    const int rb = j * s.nsym + isymb;
    const int b_ind = ppn_draw(s, rs, kPPN_JBD, rb, nbb);
    const int b = ssbf<W>(s, imsb, isymb, b_ind);
    if (a == b || tbit<W>(f, b)) return;
    const double tot_a = __ldg(&s.ppn_tot[kPPN_IAD][i]), tot_b = __ldg(&s.ppn_tot[kPPN_JBD][rb]);
    if (ij_spin == 0) {
        pg = pg * (ppn_w(s, kPPN_IAD, i, a_ind) / tot_a * ppn_w(s, kPPN_JBD, rb, b_ind) / tot_b);
    } else {
        const int isyma = xsym(s, ij_sym, isymb);
        const int ra = j * s.nsym + isyma;
        const int a_rev = rank_in_mask<W>(&s.symmask[(isyma * 2 + imsb) * W], a);
        pg = pg * (ppn_w(s, kPPN_IAD, i, a_ind) / tot_a * ppn_w(s, kPPN_JBD, rb, b_ind) / tot_b +
                   ppn_w(s, kPPN_IAD, i, b >> 1) / tot_a * ppn_w(s, kPPN_JBD, ra, a_rev) /
                       __ldg(&s.ppn_tot[kPPN_JBD][ra]));
    }
    pgen = s.pattempt_double * pg;
    out.allowed = true;
    out.to[0] = a < b ? a : b;
    out.to[1] = a < b ? b : a;
    hm = sc2_mol<double>(s, i, j, out.to[0], out.to[1], perm2<W>(f, i, j, out.to[0], out.to[1]));
}

// gen_excit_mol_heat_bath (src/excit_gen_heat_bath_mol.F90:258-547).
template <int W, typename Real>
__device__ void gen_heat_bath(const DevSys &s, RStream &rs, const Det<W> &f, Attempt &out, double &pgen, Real &hm) {
    HBView<Real> hb(s);
    HBSel<Real> q;
    const int nb = s.nbasis;
    out.nexcit = 2;
    bool allowed = hb_select_ij<W, Real>(s, hb, rs, f, q);
    int i = q.i, j = q.j;
    out.from[0] = i;
    out.from[1] = j;
    if (!(allowed && rabs(hb.ija_t(i, j)) > (Real)0)) allowed = false;
    int a = -1, b = -1;
    bool dbl = true;
    Real psingle = (Real)0, hmod_ia = (Real)0;
    if (allowed) {
        size_t o3 = ((size_t)i * nb + j) * nb;
        a = hb_alias_draw<Real>(rs, nb, hb.ija_U + o3, hb.ija_K + o3);
        if (!tbit<W>(f, a)) {
            if (s.orbsym[a] == s.orbsym[i] && ms_of(a) == ms_of(i)) {
                hmod_ia = rabs(sc1_mol<W, Real>(s, f, i, a, perm1<W>(f, i, a)));
                double x = rs.next();
                Real wt = hb.ijab_t(i, j, a);
                psingle = hmod_ia < wt ? hmod_ia / (wt + hmod_ia) : (Real)0.5;
                dbl = !(x < (double)psingle);
            } else {
                dbl = true;
                psingle = (Real)0;
            }
        } else {
            allowed = false;
        }
    }
    Real pg = (Real)1, h = (Real)0;
    if (allowed) {
        if (dbl) {
            size_t o4 = (((size_t)i * nb + j) * nb + a) * nb;
            b = hb_alias_draw<Real>(rs, nb, hb.ijab_U + o4, hb.ijab_K + o4);
            if (!tbit<W>(f, b)) {
                const Real one = (Real)1;
                Real p_ij = (q.wi[q.i_ind] / q.wi_tot) * (q.ijw[q.j_ind] / q.ij_tot);
                Real p_ji = (q.wi[q.j_ind] / q.wi_tot) * (q.jiw[q.i_ind] / q.ji_tot);
                Real pgen_ija = p_ij * (hb.ija(i, j, a) / hb.ija_t(i, j)) * (one - psingle) *
                                (hb_weight<Real>(s, i, j, a, b) / hb.ijab_t(i, j, a));
                psingle = hb_psingle<W, Real>(s, f, i, b, hb.ijab_t(i, j, b));
                Real pgen_ijb = p_ij * (hb.ija(i, j, b) / hb.ija_t(i, j)) * (one - psingle) *
                                (hb_weight<Real>(s, i, j, b, a) / hb.ijab_t(i, j, b));
                psingle = hb_psingle<W, Real>(s, f, j, a, hb.ijab_t(j, i, a));
                Real pgen_jia = p_ji * (hb.ija(j, i, a) / hb.ija_t(j, i)) * (one - psingle) *
                                (hb_weight<Real>(s, j, i, a, b) / hb.ijab_t(j, i, a));
                psingle = hb_psingle<W, Real>(s, f, j, b, hb.ijab_t(j, i, b));
                Real pgen_jib = p_ji * (hb.ija(j, i, b) / hb.ija_t(j, i)) * (one - psingle) *
                                (hb_weight<Real>(s, j, i, b, a) / hb.ijab_t(j, i, b));
                pg = pgen_ija + pgen_ijb + pgen_jia + pgen_jib;
                int f0 = i < j ? i : j, f1 = i < j ? j : i, t0 = a < b ? a : b, t1 = a < b ? b : a;
                out.from[0] = f0;
                out.from[1] = f1;
                out.to[0] = t0;
                out.to[1] = t1;
                h = sc2_mol<Real>(s, f0, f1, t0, t1, perm2<W>(f, f0, f1, t0, t1));
            } else {
                allowed = false;
            }
        } else {
            out.nexcit = 1;
            out.from[1] = -1;
            out.to[0] = a;
            h = sc1_mol<W, Real>(s, f, i, a, perm1<W>(f, i, a));
            pg = (Real)0;
            for (int p = 0; p < s.nel; p++) {
                int oq = q.occ[p];
                // a q with no double excitation from (i,q) (weights_tot(q,i) = 0)
                // contributes 0 * (0/0) in the reference, a NaN p_gen; it adds 0 here
                if (i != oq && a != oq && hb.ija_t(i, oq) > (Real)0) {
                    Real wt = hb.ijab_t(i, oq, a);
                    Real psq = hmod_ia < wt ? hmod_ia / (wt + hmod_ia) : (Real)0.5;
                    pg = pg + psq * (q.ijw[p] / q.ij_tot) * (hb.ija(i, oq, a) / hb.ija_t(i, oq));
                }
            }
            pg = pg * (q.wi[q.i_ind] / q.wi_tot);
        }
    }
    out.allowed = allowed;
    pgen = allowed ? (double)pg : 1.0;
    hm = allowed ? h : (Real)0;
}

// gen_excit_mol_heat_bath_uniform, double branch (src/excit_gen_heat_bath_mol.F90:619-705).
template <int W, typename Real>
__device__ void gen_heat_bath_uniform_double(const DevSys &s, RStream &rs, const Det<W> &f, Attempt &out,
                                             double &pgen, Real &hm) {
    HBView<Real> hb(s);
    HBSel<Real> q;
    const int nb = s.nbasis;
    out.nexcit = 2;
    bool allowed = hb_select_ij<W, Real>(s, hb, rs, f, q);
    int i = q.i, j = q.j;
    if (!(allowed && rabs(hb.ija_t(i, j)) > (Real)0)) allowed = false;
    Real pij = (Real)0;
    if (q.j_ind >= 0)
        pij = ((q.wi[q.i_ind] / q.wi_tot) * (q.ijw[q.j_ind] / q.ij_tot)) +
              ((q.wi[q.j_ind] / q.wi_tot) * (q.jiw[q.i_ind] / q.ji_tot));
    if (j >= 0 && j < i) {
        int t = j;
        j = i;
        i = t;
    }
    out.from[0] = i;
    out.from[1] = j;
    int a = -1, b = -1;
    if (allowed) {
        size_t o3 = ((size_t)i * nb + j) * nb;
        a = hb_alias_draw<Real>(rs, nb, hb.ija_U + o3, hb.ija_K + o3);
        if (rabs(hb.ijab_t(i, j, a)) > (Real)0 && !tbit<W>(f, a)) {
            size_t o4 = (o3 + a) * nb;
            b = hb_alias_draw<Real>(rs, nb, hb.ijab_U + o4, hb.ijab_K + o4);
            allowed = !tbit<W>(f, b);
        } else {
            allowed = false;
        }
    }
    Real pg = (Real)1, h = (Real)0;
    if (allowed) {
        int t0 = a < b ? a : b, t1 = a < b ? b : a;
        out.to[0] = t0;
        out.to[1] = t1;
        h = sc2_mol<Real>(s, i, j, t0, t1, perm2<W>(f, i, j, t0, t1));
        pg = ((Real)1 - (Real)s.pattempt_single) * pij *
             (((hb.ija(i, j, a) / hb.ija_t(i, j)) * (hb_weight<Real>(s, i, j, a, b) / hb.ijab_t(i, j, a))) +
              ((hb.ija(i, j, b) / hb.ija_t(i, j)) * (hb_weight<Real>(s, i, j, b, a) / hb.ijab_t(i, j, b))));
    }
    out.allowed = allowed;
    pgen = (double)pg;
    hm = h;
}

// slater_condon1_mol (src/hamiltonian_molecular.f90:140-196) with perm = false:
// 0 unless i and a share spin and symmetry.
template <int W, typename Real>
__device__ __forceinline__ Real sc1_checked(const DevSys &s, const Det<W> &f, int i, int a) {
    if (s.orbsym[i] != s.orbsym[a] || ms_of(i) != ms_of(a)) return (Real)0;
    return sc1_mol<W, Real>(s, f, i, a, false);
}

// find_ia_single_weights (src/excit_gen_utils.f90:169-212) and
// gen_single_excit_heat_bath_exact (src/excit_gen_heat_bath_mol.F90:732-807):
// i chosen with weight sum_a |H_ia| over the unoccupied a, then a with weight
// |H_ia|.  The row of the chosen i is evaluated again rather than stored (the
// same values), so a thread holds O(nvirt) weights, not O(nel nvirt).
template <int W, typename Real>
__device__ void gen_single_hb_exact(const DevSys &s, RStream &rs, const MolDet<W> &d, Attempt &out, double &pgen,
                                    Real &hm) {
    const Det<W> &f = d.f;
    out.nexcit = 1;
    uint8_t occ[kHBMaxEl];
    Real wi[kHBMaxEl];
    int n = 0;
#pragma unroll
    for (int k = 0; k < W; k++)
        for (uint64_t x = f.w[k]; x && n < kHBMaxEl; x &= x - 1) occ[n++] = (uint8_t)(64 * k + __ffsll((long long)x) - 1);
    Real tot = (Real)0;
    for (int ii = 0; ii < s.nel; ii++) {
        Real w = (Real)0;
#pragma unroll
        for (int k = 0; k < W; k++)
            for (uint64_t x = ~f.w[k] & d.valid[k]; x; x &= x - 1)
                w = w + rabs(sc1_checked<W, Real>(s, f, occ[ii], 64 * k + __ffsll((long long)x) - 1));
        wi[ii] = w;
        tot = tot + w;
    }
    if (tot < (Real)1.0e-12) {
        out.allowed = false;
        pgen = 1.0;
        hm = (Real)0;
        return;
    }
    const int i_ind = hb_alias_select<Real>(rs, s.nel, wi, tot);
    const int i = occ[i_ind];
    constexpr int CAP = 64 * W;
    Real row[CAP];
    uint8_t unocc[CAP];
    int nv = 0;
#pragma unroll
    for (int k = 0; k < W; k++)
        for (uint64_t x = ~f.w[k] & d.valid[k]; x; x &= x - 1) {
            int a = 64 * k + __ffsll((long long)x) - 1;
            unocc[nv] = (uint8_t)a;
            row[nv++] = rabs(sc1_checked<W, Real>(s, f, i, a));
        }
    const int a_ind = hb_alias_select<Real, CAP>(rs, nv, row, wi[i_ind]);
    const int a = unocc[a_ind];
    out.allowed = true;
    out.from[0] = i;
    out.to[0] = a;
    pgen = (double)((Real)s.pattempt_single * (wi[i_ind] / tot) * (row[a_ind] / wi[i_ind]));
    hm = sc1_mol<W, Real>(s, f, i, a, perm1<W>(f, i, a));
}

// spawn_standard + attempt_to_spawn with a heat-bath generator (heat_bath;
// heat_bath_uniform, whose singles are gen_single_excit_mol's; heat_bath_single,
// whose singles are gen_single_excit_heat_bath_exact's).
template <int W, typename Real>
__device__ void attempt_heat_bath(const DevSys &s, RStream &rs, const MolDet<W> &d, int64_t parent, Attempt &out) {
    out.from[0] = out.from[1] = out.to[0] = out.to[1] = -1;
    double pgen;
    Real hm;
    if (s.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH)
        gen_heat_bath<W, Real>(s, rs, d.f, out, pgen, hm);
    else if (rs.next_k() >= s.t_single)  // rand >= pattempt_single: a double
        gen_heat_bath_uniform_double<W, Real>(s, rs, d.f, out, pgen, hm);
    else if (s.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE)
        gen_single_hb_exact<W, Real>(s, rs, d, out, pgen, hm);
    else
        gen_single_mol<W, Real>(s, rs, d, true, out, pgen, hm);
    attempt_to_spawn(s, rs, parent, pgen, (double)hm, out);
}

// Child determinant of an attempt (create_excited_det, src/excitations.F90:365-406).
template <int W>
__device__ __forceinline__ Det<W> excited(const Det<W> &f, const Attempt &a) {
    Det<W> c = f;
    for (int k = 0; k < a.nexcit; k++) {
        c.w[a.from[k] >> 6] &= ~(1ull << (a.from[k] & 63));
        c.w[a.to[k] >> 6] |= (1ull << (a.to[k] & 63));
    }
    return c;
}

// update_proj_energy_hub_k / update_proj_energy_mol
// (src/energy_evaluation.F90:795-849, :906-985): H_0i for D_i against D_0
// (0 when D_i is D_0 or not connected).
template <int W>
__device__ double proj_hmatel(const DevSys &s, const HubTables &t, const Det<W> &f, const Excit &e) {
    if (e.nexcit == 0 || e.nexcit > 2) return 0.0;
    if (s.kind == HGPU_SYS_HUB_K) {
        if (e.nexcit != 2) return 0.0;
        double h = two_e_int_hub_k(s, t, e.from[0], e.from[1], e.to[0], e.to[1]);
        return e.perm ? -h : h;
    }
    if (e.nexcit == 1) {
        if (ms_of(e.from[0]) == ms_of(e.to[0]) && sym_of<W>(s, e.from[0]) == sym_of<W>(s, e.to[0]))
            return sc1_mol<W, double>(s, f, e.from[0], e.to[0], e.perm);
        return 0.0;
    }
    int i = e.from[0], j = e.from[1], a = e.to[0], b = e.to[1];
    if (ms_of(i) + ms_of(j) == ms_of(a) + ms_of(b)) {
        if (xsym(s, sym_of<W>(s, i), sym_of<W>(s, j)) == xsym(s, sym_of<W>(s, a), sym_of<W>(s, b)))
            return sc2_mol<double>(s, i, j, a, b, e.perm);
    }
    return 0.0;
}

}  // namespace hgpu
