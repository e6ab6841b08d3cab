// hgpu_engine.cu -- host engine and C ABI (include/hande_gpu.h).
//
// One handle = one FCIQMC calculation resident on the current CUDA device: the
// system, the double-buffered main walker list, the spawned list and all
// scratch are allocated once at hgpu_create.  A Monte Carlo cycle is a fixed
// launch sequence on the handle's stream (hgpu_kernels.cu); it is captured as
// a CUDA graph per main-list buffer parity and replayed, so a report of
// ncycles cycles costs ncycles graph launches and one small readback.
#include <cuda_runtime.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <queue>
#include <vector>

#include "../../include/hande_gpu.h"
#include "hgpu_heat_bath.h"
#include "hgpu_power_pitzer.h"
#include "hgpu_kernels.cuh"

using namespace hgpu;

struct hgpu_handle {
    hgpu_config cfg;
    int W, R, kind;
    int sms;    // multiprocessors of the device
    int gkind;  // generator kind of the spawning kernels (hgpu_kernels.cuh: kKind*, or the system kind)
    int device;
    cudaStream_t stream;
    DevBuffers b;
    DevSys hsys;  // host copy of the device system struct
    int cur;      // buffer holding the current main list
    // replica 2-RDM: accumulating (spawn_rdm on), reports ended, a report in progress
    int rdm_on = 0;
    int reports_done = 0;
    bool report_open = false;
    cudaGraphExec_t graph[2];
    bool graph_ok[2];
    bool use_graphs;
    // report bookkeeping (host side, as qmc_state_t)
    double shift[HGPU_MAX_SPACES];
    int vary_shift[HGPU_MAX_SPACES];
    double nparticles_old[HGPU_MAX_SPACES];
    int64_t iter;
    int64_t ss_iter;  // iteration at whose start the deterministic space is built
    int64_t ss_gen = 0;  // number of deterministic spaces built or dropped so far
    int64_t launch_gen = 0;  // number of hgpu_set_launch calls (batch graphs follow it)
    // hub_k momentum tables on the host (the 'ci' deterministic space)
    std::vector<int> h_symtab, h_invsym;
    cudaEvent_t ev0, ev1;
    double report_ms;
    std::vector<void *> allocs;
    // device staging for parity entry points
    void *scratch;
    size_t scratch_bytes;
    // walker-list snapshot (hgpu_snapshot)
    uint64_t *snap_dets;
    int64_t *snap_pops;
    double *snap_kii;
    int64_t snap_n;
    int64_t snap_abs[HGPU_MAX_SPACES];
    int64_t snap_ss_gen = -1;  // ss_gen when the snapshot was taken
};

#define CK(x)                                                \
    do {                                                     \
        cudaError_t e_ = (x);                                \
        if (e_ != cudaSuccess) {                             \
            last_error_text(cudaGetErrorString(e_), #x);     \
            return HGPU_ERR_CUDA;                            \
        }                                                    \
    } while (0)

static char g_last_error[512];
static void last_error_text(const char *what, const char *where) {
    snprintf(g_last_error, sizeof(g_last_error), "%s (%s)", what, where);
}

template <typename T>
static int dalloc(hgpu_handle *h, T **p, size_t n) {
    if (n == 0) n = 1;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) {
        last_error_text(cudaGetErrorString(e), "cudaMalloc");
        *p = nullptr;
        return HGPU_ERR_OOM;
    }
    h->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return HGPU_OK;
}

extern "C" {

int32_t hgpu_version(void) { return 100; }

const char *hgpu_error_string(int32_t status) {
    switch (status) {
        case HGPU_OK: return "ok";
        case HGPU_ERR_INVALID: return "invalid argument";
        case HGPU_ERR_OOM: return "out of device memory";
        case HGPU_ERR_SPAWN_OVERFLOW: return "spawned walker list full";
        case HGPU_ERR_MAIN_OVERFLOW: return "main walker list full";
        case HGPU_ERR_TIMEOUT: return "device wait timed out";
        case HGPU_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA error";
        case HGPU_ERR_NO_DEVICE: return "no CUDA device";
        case HGPU_ERR_UNSUPPORTED: return "unsupported option";
        default: return "unknown status";
    }
}

int32_t hgpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // extern "C"

static int64_t capacity_entries(int64_t v, size_t bytes_per_entry, int64_t fallback) {
    // qmc_in%walker_length: > 0 entries, < 0 megabytes (src/qmc.F90:1462-1465)
    if (v > 0) return v;
    if (v < 0) return (int64_t)((double)(-v) * 1048576.0 / (double)bytes_per_entry);
    return fallback;
}

// Exact-diagonal tables (hgpu_fixed.h) and E(D) on the host, same definition
// as the device's fx_energy.
struct FxTables {
    int shift;
    int64_t cst;
    std::vector<int64_t> h1, pair, eps;
};

static void build_fx(const hgpu_system *sys, FxTables &t) {
    if (sys->kind == HGPU_SYS_HUB_K) {
        double c0 = (double)(sys->nalpha * sys->nbeta) * sys->coulomb_k;
        int64_t B = fx_ceil_abs(c0);
        for (int p = 0; p < sys->nbasis; p++) B += fx_ceil_abs(sys->sp_eigv[p]);
        t.shift = fx_scale_for_bound(B);
        t.cst = fx_from_double(c0, t.shift);
        t.eps.resize(sys->nbasis);
        for (int p = 0; p < sys->nbasis; p++) t.eps[p] = fx_from_double(sys->sp_eigv[p], t.shift);
        return;
    }
    int M = sys->norb;
    auto tri0 = [](int64_t i, int64_t j) { return i * (i + 1) / 2 + j; };
    auto v2 = [&](int p, int q, int r, int s) {  // (pq|rs), spatial
        int64_t pq = p >= q ? tri0(p, q) : tri0(q, p);
        int64_t rs = r >= s ? tri0(r, s) : tri0(s, r);
        return sys->v2[pq >= rs ? tri0(pq, rs) : tri0(rs, pq)];
    };
    // bound over every term of every determinant: spin orbitals i < j
    int nb = sys->nbasis;
    int64_t B = fx_ceil_abs(sys->ecore);
    for (int i = 0; i < nb; i++) {
        B += fx_ceil_abs(sys->h1[(i >> 1) * M + (i >> 1)]);
        for (int j = i + 1; j < nb; j++) {
            B += fx_ceil_abs(v2(i >> 1, i >> 1, j >> 1, j >> 1));
            if (((i ^ j) & 1) == 0) B += fx_ceil_abs(v2(i >> 1, j >> 1, j >> 1, i >> 1));
        }
    }
    t.shift = fx_scale_for_bound(B);
    t.cst = fx_from_double(sys->ecore, t.shift);
    t.h1.resize(M);
    t.pair.resize((size_t)2 * M * M);
    for (int p = 0; p < M; p++) {
        t.h1[p] = fx_from_double(sys->h1[p * M + p], t.shift);
        for (int q = 0; q < M; q++) {
            int64_t J = fx_from_double(v2(p, p, q, q), t.shift);  // <ij|ij> = (ii|jj)
            int64_t K = fx_from_double(v2(p, q, q, p), t.shift);  // <ij|ji> = (ij|ji)
            t.pair[(size_t)p * M + q] = J;
            t.pair[(size_t)M * M + (size_t)p * M + q] = J - K;
        }
    }
}

static int64_t host_energy(const hgpu_system *sys, const FxTables &t, const uint64_t *f) {
    int64_t e = t.cst;
    std::vector<int> occ;
    for (int p = 0; p < sys->nbasis; p++)
        if ((f[p >> 6] >> (p & 63)) & 1ull) occ.push_back(p);
    if (sys->kind == HGPU_SYS_HUB_K) {
        for (int p : occ) e += t.eps[p];
        return e;
    }
    int M = sys->norb;
    for (size_t a = 0; a < occ.size(); a++) {
        int i = occ[a];
        e += t.h1[i >> 1];
        for (size_t c = a + 1; c < occ.size(); c++) {
            int j = occ[c];
            e += t.pair[(((i ^ j) & 1) == 0 ? (size_t)M * M : 0) + (size_t)(i >> 1) * M + (j >> 1)];
        }
    }
    return e;
}

template <typename T>
static int upload(hgpu_handle *h, const T *src, size_t n, const T **out) {
    T *d;
    int rc = dalloc(h, &d, n);
    if (rc) return rc;
    CK(cudaMemcpy(d, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    *out = d;
    return HGPU_OK;
}

// Heat-bath tables (hgpu_heat_bath.h) in the precision of the spawning path.
template <typename Real>
static int upload_heat_bath(hgpu_handle *h, const HeatBathTables &t, DevSys &s) {
    auto put = [&](const std::vector<double> &v, const void **out) -> int {
        std::vector<Real> r(v.size());
        for (size_t k = 0; k < v.size(); k++) r[k] = (Real)v[k];
        const Real *d;
        int rc = upload(h, r.data(), r.size(), &d);
        *out = d;
        return rc;
    };
    int rc;
    if ((rc = put(t.i_w, &s.hb_i_w))) return rc;
    if ((rc = put(t.ij_w, &s.hb_ij_w))) return rc;
    if ((rc = put(t.ija_w, &s.hb_ija_w))) return rc;
    if ((rc = put(t.ija_tot, &s.hb_ija_tot))) return rc;
    if ((rc = put(t.ija_U, &s.hb_ija_U))) return rc;
    if ((rc = put(t.ijab_tot, &s.hb_ijab_tot))) return rc;
    if ((rc = put(t.ijab_U, &s.hb_ijab_U))) return rc;
    if ((rc = upload(h, t.ija_K.data(), t.ija_K.size(), &s.hb_ija_K))) return rc;
    if ((rc = upload(h, t.ijab_K.data(), t.ijab_K.size(), &s.hb_ijab_K))) return rc;
    return HGPU_OK;
}

static int build_heat_bath(hgpu_handle *h, const hgpu_system *sys, DevSys &s) {
    HeatBathTables t;
    if (!HeatBathBuilder(sys).build(t, h->cfg.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH)) return HGPU_ERR_OOM;
    if (t.bias && h->cfg.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH) {
        // init_excit_mol_heat_bath stops the calculation here (src/excit_gen_heat_bath_mol.F90:185-197)
        last_error_text("Not all possible single excitations can be accounted for. Use another excitation generator.",
                        "heat bath");
        return HGPU_ERR_INVALID;
    }
    if (h->cfg.precision == HGPU_PREC_MIXED) return upload_heat_bath<float>(h, t, s);
    return upload_heat_bath<double>(h, t, s);
}

// find_single_double_prob, read_in branch (src/qmc_common.F90:152-260): the
// numbers of symmetry- and spin-allowed single and double excitations of the
// reference determinant, each divided by their sum.
static void single_double_prob(const hgpu_system *sys, const uint64_t *ref, double &psingle, double &pdouble) {
    const int nsym = sys->nsym_pg;
    std::vector<int64_t> virt((size_t)2 * nsym);
    std::vector<int> occ;
    for (int p = 0; p < sys->nbasis; p++)
        if ((ref[p >> 6] >> (p & 63)) & 1u) occ.push_back(p);
    for (int k = 0; k < 2 * nsym; k++) virt[k] = sys->nbasis_sym_spin[k];
    auto slot = [&](int p) { return (size_t)((sys->orb_ms[p] + 1) / 2) * nsym + sys->orb_sym[p]; };
    for (int p : occ) virt[slot(p)]--;
    int64_t nsingles = 0, ndoubles = 0;
    for (int p : occ) nsingles += virt[slot(p)];
    const size_t n = occ.size();
    for (size_t i = 0; i < n; i++) {
        const int m1 = (sys->orb_ms[occ[i]] + 1) / 2;
        for (size_t j = i + 1; j < n; j++) {
            const int m2 = (sys->orb_ms[occ[j]] + 1) / 2;
            const int ij = sys->orb_sym[occ[i]] ^ sys->orb_sym[occ[j]];
            for (int sa = 0; sa < nsym; sa++) {
                const int sb = (sa ^ ij) & (nsym - 1);
                const int64_t va = virt[(size_t)m1 * nsym + sa], vb = virt[(size_t)m2 * nsym + sb];
                if (sa == sb) {
                    ndoubles += m1 == m2 ? (va * (vb - 1)) / 2 : va * vb;
                } else if (sa < sb) {
                    ndoubles += va * vb;
                    if (m1 != m2) ndoubles += virt[(size_t)m2 * nsym + sa] * virt[(size_t)m1 * nsym + sb];
                }
            }
        }
    }
    psingle = (double)nsingles / (double)(nsingles + ndoubles);
    pdouble = (double)ndoubles / (double)(nsingles + ndoubles);
}

static int build_system(hgpu_handle *h, const hgpu_system *sys) {
    DevSys &s = h->hsys;
    memset(&s, 0, sizeof(s));
    const hgpu_config &c = h->cfg;
    s.kind = sys->kind;
    s.nbasis = sys->nbasis;
    s.nel = sys->nel;
    s.nalpha = sys->nalpha;
    s.nbeta = sys->nbeta;
    s.nw = sys->nwords;
    s.nvirt_alpha = sys->nbasis / 2 - sys->nalpha;
    s.nvirt_beta = sys->nbasis / 2 - sys->nbeta;
    s.nvirt = sys->nbasis - sys->nel;
    s.nspaces = h->R;
    s.excit_gen = c.excit_gen;
    s.initiator = c.initiator_approx ? 1 : 0;
    s.real_amplitudes = c.real_amplitudes ? 1 : 0;
    s.precision = c.precision;
    s.real_factor = c.real_amplitudes ? ((int64_t)1 << 31) : 1;
    s.cutoff = c.real_amplitudes ? (int64_t)std::ceil(c.spawn_cutoff * (double)s.real_factor) : 0;
    s.tau = c.tau;
    // init_excit_gen (src/qmc.F90:951-972)
    if (c.pattempt_single < 0 || c.pattempt_double < 0) {
        if (sys->kind == HGPU_SYS_HUB_K) {
            s.pattempt_single = 0.0;
            s.pattempt_double = 1.0;
        } else {
            single_double_prob(sys, c.ref_det, s.pattempt_single, s.pattempt_double);
        }
    } else {
        s.pattempt_single = c.pattempt_single / (c.pattempt_single + c.pattempt_double);
        s.pattempt_double = 1.0 - c.pattempt_single;
    }
    s.t_single = (uint64_t)std::ceil(std::ldexp(s.pattempt_single, 53));
    s.initiator_pop = c.initiator_pop;
    s.quadrature_initiator = c.quadrature_initiator != 0 && h->R == 2;
    s.seed = (uint64_t)c.seed;
    for (int w = 0; w < kMaxWords; w++) s.f0[w] = w < s.nw ? c.ref_det[w] : 0;
    FxTables fx;
    build_fx(sys, fx);
    s.fx_shift = fx.shift;
    s.fx_inv_scale = std::ldexp(1.0, -fx.shift);
    s.fx_const = fx.cst;
    s.fx_E0 = host_energy(sys, fx, s.f0);
    s.H00 = fx_to_double(s.fx_E0, s.fx_inv_scale);
    int rc;
    if (sys->kind == HGPU_SYS_HUB_K) {
        if ((rc = upload(h, fx.eps.data(), fx.eps.size(), &s.fx_eps))) return rc;
    } else {
        if ((rc = upload(h, fx.h1.data(), fx.h1.size(), &s.fx_h1))) return rc;
        if ((rc = upload(h, fx.pair.data(), fx.pair.size(), &s.fx_pair))) return rc;
    }
    // reciprocal table 1/x (x = 0..inv_max) and the FP64 constants of the generators
    s.inv_max = 2 * sys->nbasis * (sys->nel + 1) + 16;
    {
        std::vector<double> inv((size_t)s.inv_max + 1);
        for (int x = 0; x <= s.inv_max; x++) inv[x] = 1.0 / (double)x;
        if ((rc = upload(h, inv.data(), inv.size(), &s.inv))) return rc;
    }
    s.pgen_ij = 2.0 / (double)(s.nel * (s.nel - 1));
    s.d_nel = (double)s.nel;
    s.d_nelm1 = (double)(s.nel - 1);
    s.d_nbasis = (double)s.nbasis;
    s.d_half_nbasis = (double)(s.nbasis / 2);
    s.d_nalpha = (double)s.nalpha;
    s.d_nbeta = (double)s.nbeta;
    s.d_nvirt_alpha = (double)s.nvirt_alpha;
    s.d_real_factor = (double)s.real_factor;
    s.d_cutoff = (double)s.cutoff;
    if (sys->kind == HGPU_SYS_HUB_K) {
        int nv = s.nvirt_alpha;
        std::vector<double> pg(nv + 1), ps(nv + 1);
        std::vector<uint8_t> al(nv + 1);
        double abs_h = std::fabs(sys->coulomb_k);
        for (int f = 0; f <= nv; f++) {
            // calc_pgen_hub_k and spawn_lattice_split_gen's p_spawn, per forbidden count
            pg[f] = 1.0 / (double)(s.nalpha * s.nbeta * (nv - f));
            al[f] = 1.0 / pg[f] > 1.0e-12 ? 1 : 0;
            ps[f] = (double)s.real_factor * c.tau * abs_h / pg[f];
        }
        if ((rc = upload(h, pg.data(), pg.size(), &s.hub_pgen))) return rc;
        if ((rc = upload(h, ps.data(), ps.size(), &s.hub_pspawn))) return rc;
        if ((rc = upload(h, al.data(), al.size(), &s.hub_allowed))) return rc;
        s.hub_pgen_nr = 1.0 / (double)(s.nalpha * s.nbeta * nv);
        s.hub_pspawn_nr = (double)s.real_factor * c.tau * abs_h / s.hub_pgen_nr;
    }
    double *sp;
    if ((rc = dalloc(h, &sp, sys->nbasis))) return rc;
    CK(cudaMemcpy(sp, sys->sp_eigv, sizeof(double) * sys->nbasis, cudaMemcpyHostToDevice));
    s.sp_eigv = sp;
    if (sys->kind == HGPU_SYS_HUB_K) {
        int nk = sys->nkpoints;
        if (nk > 255) return HGPU_ERR_UNSUPPORTED;
        s.nk = nk;
        s.coulomb_k = sys->coulomb_k;
        std::vector<uint8_t> st(nk * nk), inv(nk);
        for (int i = 0; i < nk * nk; i++) st[i] = (uint8_t)sys->sym_table[i];
        for (int i = 0; i < nk; i++) inv[i] = (uint8_t)sys->inv_sym[i];
        uint8_t *dst, *dinv;
        if ((rc = dalloc(h, &dst, nk * nk))) return rc;
        if ((rc = dalloc(h, &dinv, nk))) return rc;
        CK(cudaMemcpy(dst, st.data(), nk * nk, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dinv, inv.data(), nk, cudaMemcpyHostToDevice));
        s.sym_table = dst;
        s.inv_sym = dinv;
        s.nsym = 1;
        h->b.nk = nk;
        h->h_symtab.assign(sys->sym_table, sys->sym_table + nk * nk);
        h->h_invsym.assign(sys->inv_sym, sys->inv_sym + nk);
    } else if (sys->kind == HGPU_SYS_READ_IN) {
        if (sys->nsym_pg > kMaxSym || sys->nsym_pg < 1) return HGPU_ERR_UNSUPPORTED;
        s.norb = sys->norb;
        s.nsym = sys->nsym_pg;
        s.ecore = sys->ecore;
        int M = sys->norb;
        double *dh1, *dv2;
        float *fh1, *fv2;
        if ((rc = dalloc(h, &dh1, (size_t)M * M))) return rc;
        if ((rc = dalloc(h, &dv2, (size_t)sys->nv2))) return rc;
        CK(cudaMemcpy(dh1, sys->h1, sizeof(double) * M * M, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dv2, sys->v2, sizeof(double) * sys->nv2, cudaMemcpyHostToDevice));
        s.h1 = dh1;
        s.v2 = dv2;
        if (c.precision == HGPU_PREC_MIXED) {
            std::vector<float> t1(M * M), t2(sys->nv2);
            for (int i = 0; i < M * M; i++) t1[i] = (float)sys->h1[i];
            for (int64_t i = 0; i < sys->nv2; i++) t2[i] = (float)sys->v2[i];
            if ((rc = dalloc(h, &fh1, (size_t)M * M))) return rc;
            if ((rc = dalloc(h, &fv2, (size_t)sys->nv2))) return rc;
            CK(cudaMemcpy(fh1, t1.data(), sizeof(float) * M * M, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(fv2, t2.data(), sizeof(float) * sys->nv2, cudaMemcpyHostToDevice));
            s.h1f = fh1;
            s.v2f = fv2;
        }
        for (int p = 0; p < sys->nbasis; p++) {
            int sym = sys->orb_sym[p];
            int ims = (p & 1) ? 0 : 1;
            if (sym < 0 || sym >= s.nsym) return HGPU_ERR_INVALID;
            s.symmask[(sym * 2 + ims) * s.nw + (p >> 6)] |= 1ull << (p & 63);
            s.nbss[sym * 2 + ims]++;
            s.orbsym[p] = (uint8_t)sym;
        }
        for (int k = 0; k < 2 * kMaxSym; k++) s.d_nbss[k] = (double)s.nbss[k];
        h->b.nk = 0;
        // renorm_spin / no_renorm_spin: pattempt_parallel (src/qmc.F90:974-988)
        // and the pgen_ij of each spin class in choose_ij_spin_mol's rounding
        // order (src/excit_gen_mol.f90:684-783)
        double pgen_ij_cls[3] = {s.pgen_ij, 0.0, 0.0};
        int ncls = 1;
        s.spin_ij = c.excit_gen == HGPU_EXCIT_GEN_RENORM_SPIN || c.excit_gen == HGPU_EXCIT_GEN_NO_RENORM_SPIN;
        if (s.spin_ij) {
            const double pp = c.pattempt_parallel < 0.0 ? HeatBathBuilder(sys).parallel_spin_prob() : c.pattempt_parallel;
            const double na = (double)s.nalpha, nb = (double)s.nbeta;
            pgen_ij_cls[0] = (1.0 - pp) * (1.0 / (double)(s.nalpha * s.nbeta));
            pgen_ij_cls[1] = s.nalpha >= 2 ? pp * (na / (na + nb)) * 2.0 * (1.0 / na) * (1.0 / (na - 1.0)) : 0.0;
            pgen_ij_cls[2] = s.nbeta >= 2 ? pp * (nb / (na + nb)) * 2.0 * (1.0 / nb) * (1.0 / (nb - 1.0)) : 0.0;
            s.t_parallel = (uint64_t)std::ceil(std::ldexp(pp, 53));
            s.t_alpha = (uint64_t)std::ceil(std::ldexp(na / (na + nb), 53));
            ncls = 3;
        }
        {
            // double-excitation p_gen table: pattempt_double * pgen_ij * (inv[n] * (inv[xb] + inv[xa])),
            // each product and sum rounded as the generator writes it, for each pgen_ij class
            int X = 1;
            for (int k = 0; k < 2 * kMaxSym; k++) X = std::max(X, s.nbss[k] + 1);
            int Nn = s.nvirt + 1;
            std::vector<double> tab((size_t)ncls * Nn * X * X);
            for (int cls = 0; cls < ncls; cls++) {
                double c0 = s.pattempt_double * pgen_ij_cls[cls];
                for (int n = 0; n < Nn; n++)
                    for (int xa = 0; xa < X; xa++)
                        for (int xb = 0; xb < X; xb++) {
                            double pb = 1.0 / (double)xb, pa = 1.0 / (double)xa;
                            double pg = (1.0 / (double)n) * (pb + pa);
                            tab[(((size_t)cls * Nn + n) * X + xa) * X + xb] = c0 * pg;
                        }
            }
            if ((rc = upload(h, tab.data(), tab.size(), &s.pg2))) return rc;
            s.pg2_x = X;
            s.pg2_n = Nn;
        }
        if (c.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH || c.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM ||
            c.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE) {
            if ((rc = build_heat_bath(h, sys, s))) return rc;
        }
        const bool pp_ij = c.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
                           c.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ;
        if (pp_ij) {
            // ppm_i_d_weights, ppm_ij_d_weights: read by the heat-bath choice of i, j
            std::vector<double> iw, ijw;
            HeatBathBuilder(sys).pair_weights(iw, ijw);
            const double *p;
            if ((rc = upload(h, iw.data(), iw.size(), &p))) return rc;
            s.hb_i_w = p;
            if ((rc = upload(h, ijw.data(), ijw.size(), &p))) return rc;
            s.hb_ij_w = p;
        }
        if (c.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN) {
            PPNTables t;
            PowerPitzerRefBuilder(sys, c.ref_det, c.power_pitzer_min_weight).build(t);
            for (int k = 0; k < PPN_NTAB; k++) {
                const double *p;
                const uint8_t *q;
                if ((rc = upload(h, t.w[k].data(), t.w[k].size(), &p))) return rc;
                s.ppn_w[k] = p;
                if ((rc = upload(h, t.U[k].data(), t.U[k].size(), &p))) return rc;
                s.ppn_U[k] = p;
                if ((rc = upload(h, t.tot[k].data(), t.tot[k].size(), &p))) return rc;
                s.ppn_tot[k] = p;
                if ((rc = upload(h, t.K[k].data(), t.K[k].size(), &q))) return rc;
                s.ppn_K[k] = q;
                s.ppn_stride[k] = t.stride[k];
            }
        }
        if (pp_ij || c.excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC ||
            c.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC) {
            // the weights of gen_excit_mol_power_pitzer_occ: sqrt|<pq|qp>| for equal
            // spins, else 0 (get_two_body_int_ex_mol_real), or sqrt|<pq|pq>|
            // (get_two_body_int_cou_mol_real), src/hamiltonian_molecular.f90:392-434
            const int nb = sys->nbasis;
            const bool cs = c.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC ||
                            c.excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ;
            auto tri0 = [](int64_t x, int64_t y) { return x >= y ? x * (x + 1) / 2 + y : y * (y + 1) / 2 + x; };
            std::vector<double> w((size_t)nb * nb);
            for (int p = 0; p < nb; p++)
                for (int q = 0; q < nb; q++) {
                    const int64_t sp = p >> 1, sq = q >> 1;
                    double v = 0.0;
                    if (cs) v = sys->v2[tri0(tri0(sp, sp), tri0(sq, sq))];                   // (pp|qq)
                    else if (sys->orb_ms[p] == sys->orb_ms[q]) v = sys->v2[tri0(tri0(sp, sq), tri0(sq, sp))];  // (pq|qp)
                    w[(size_t)p * nb + q] = std::sqrt(std::fabs(v));
                }
            if ((rc = upload(h, w.data(), w.size(), &s.pp_w))) return rc;
        }
    } else {
        return HGPU_ERR_INVALID;
    }
    DevSys *d;
    if ((rc = dalloc(h, &d, 1))) return rc;
    CK(cudaMemcpy(d, &s, sizeof(DevSys), cudaMemcpyHostToDevice));
    h->b.sys = d;
    return HGPU_OK;
}

// Table of the spin-resolved rank of a determinant with na alpha and nb beta
// electrons among M spatial orbitals (hgpu_sort.cuh, det_rank):
// T[(ka (nb + 1) + kb) * 2M + p] = C((p + 1) / 2, ka) C(p / 2, kb) when that
// table fits the shared memory of k_sort_hist (one load per electron), else
// C(n, k) for k <= max(na, nb), n <= M (two loads and a product per electron;
// mode 3 when the rank needs more than 64 bits: 128-bit products, two key
// words).  Returns the bits of the largest rank, or 0 when it needs more than
// 128 bits (then the sort keys are the determinant words).
static int rank_bits(int M, int na, int nb, std::vector<uint64_t> &table, int &rows, int &cols, int &mode) {
    typedef unsigned __int128 u128;
    const u128 cap = ~(uint64_t)0;
    const int kmax = std::max(na, nb);
    if (na > M || nb > M || na < 0 || nb < 0) return 0;
    std::vector<u128> c((size_t)(kmax + 1) * (M + 1), 0);
    auto C = [&](int n, int k) -> u128 & { return c[(size_t)k * (M + 1) + n]; };
    for (int n = 0; n <= M; n++) {
        C(n, 0) = 1;
        for (int k = 1; k <= kmax && k <= n; k++) {
            u128 v = C(n - 1, k - 1) + (k <= n - 1 ? C(n - 1, k) : 0);
            C(n, k) = v > cap ? cap : v;
        }
    }
    const u128 ca = C(M, na), cb = C(M, nb);
    if (ca >= cap || cb >= cap || ca == 0 || cb == 0) return 0;
    const u128 all = ~(u128)0;
    if (ca > all / cb) return 0;
    const u128 total = ca * cb;
    const size_t limit = 32768 / sizeof(uint64_t);  // shared-memory table of k_sort_hist
    const int nbasis = 2 * M;
    if (total >= cap) {
        // 128-bit ranks: binomials up to C(M, max(na, nb)) < 2^64
        if ((size_t)(kmax + 1) * (M + 1) > limit) return 0;
        mode = 3;
        rows = kmax + 1;
        cols = M + 1;
        table.assign((size_t)rows * cols, 0);
        for (size_t k = 0; k < table.size(); k++) table[k] = (uint64_t)c[k];
        const u128 maxrank = total - 1;
        int bits = 64;
        while (bits < 128 && (maxrank >> bits) != 0) bits++;
        return bits;
    }
    if ((size_t)(na + 1) * (nb + 1) * nbasis <= limit) {
        mode = 1;
        rows = (na + 1) * (nb + 1);
        cols = nbasis;
        table.assign((size_t)rows * cols, 0);
        for (int ka = 0; ka <= na; ka++)
            for (int kb = 0; kb <= nb; kb++)
                for (int p = 0; p < nbasis; p++)
                    table[(size_t)(ka * (nb + 1) + kb) * cols + p] =
                        (uint64_t)(C((p + 1) / 2, ka) * C(p / 2, kb));  // <= total: no overflow
    } else if ((size_t)(kmax + 1) * (M + 1) <= limit) {
        mode = 2;
        rows = kmax + 1;
        cols = M + 1;
        table.assign((size_t)rows * cols, 0);
        for (size_t k = 0; k < table.size(); k++) table[k] = (uint64_t)c[k];
    } else {
        return 0;
    }
    uint64_t maxrank = (uint64_t)total - 1;
    int bits = 1;
    while (bits < 64 && (maxrank >> bits) != 0) bits++;
    return bits;
}

static int alloc_lists(hgpu_handle *h) {
    int W = h->W, R = h->R, rc;
    DevBuffers &b = h->b;
    size_t main_entry = 8 * W + 8 * R + 8;
    b.cap = capacity_entries(h->cfg.walker_length, main_entry, 1 << 20);
    b.scap = capacity_entries(h->cfg.spawned_walker_length, 8 * (W + R + 1), 1 << 20);
    if (b.cap >= ((int64_t)1 << 32) || b.scap >= ((int64_t)1 << 31)) return HGPU_ERR_UNSUPPORTED;
    for (int k = 0; k < 2; k++) {
        if ((rc = dalloc(h, &b.dets[k], (size_t)b.cap * W))) return rc;
        if ((rc = dalloc(h, &b.pops[k], (size_t)b.cap * R))) return rc;
        if ((rc = dalloc(h, &b.kii[k], (size_t)b.cap))) return rc;
    }
    if ((rc = dalloc(h, &b.natt, (size_t)b.cap * R))) return rc;
    if ((rc = dalloc(h, &b.aoff, (size_t)b.cap * R))) return rc;
    if ((rc = dalloc(h, &b.pinfo, (size_t)b.cap))) return rc;
    if ((rc = dalloc(h, &b.sdets, (size_t)b.scap * W))) return rc;
    if ((rc = dalloc(h, &b.spops, (size_t)b.scap * R))) return rc;
    b.sflag = nullptr;
    if (h->cfg.initiator_approx)
        if ((rc = dalloc(h, &b.sflag, (size_t)b.scap))) return rc;
    // the singles queue of the generators that classify their attempts (a
    // tenth of the attempts with the default p_single; singles past its
    // capacity run in the spawning kernel itself)
    b.sq = nullptr;
    b.sq_cap = 0;
    const int gk = h->gkind;
    if (gk == HGPU_SYS_READ_IN || gk == kKindReadInNoRenorm || gk == kKindHeatBathUniform ||
        gk == kKindPowerPitzerOcc || gk == kKindPowerPitzerRef) {
        b.sq_cap = b.scap / 4 > (1 << 16) ? b.scap / 4 : (1 << 16);
        if ((rc = dalloc(h, &b.sq, (size_t)b.sq_cap))) return rc;
    }
    for (int k = 0; k < 2; k++) {
        if ((rc = dalloc(h, &b.keys[k], (size_t)b.scap * W))) return rc;  // key_words <= W
        if ((rc = dalloc(h, &b.idx[k], (size_t)b.scap))) return rc;
    }
    // sort: ranks (when the spin-resolved rank fits 64 bits) or determinant words
    {
        std::vector<uint64_t> binom;
        int rows = 0, cols = 0, mode = 0;
        int bits = rank_bits(h->hsys.nbasis / 2, h->hsys.nalpha, h->hsys.nbeta, binom, rows, cols, mode);
        b.use_rank = bits > 0 ? mode : 0;
        b.key32 = b.use_rank && bits <= 32 ? 1 : 0;
        if (b.use_rank == 3 && W < 2) return HGPU_ERR_UNSUPPORTED;  // two key words need two-word buffers
        b.binom_rows = rows;
        b.binom_cols = cols;
        b.sort_na = h->hsys.nalpha;
        b.sort_nb = h->hsys.nbeta;
        b.key_words = b.use_rank ? (b.use_rank == 3 ? 2 : 1) : W;
        int key_bits = b.use_rank ? bits : h->hsys.nbasis;
        b.sort_passes = (key_bits + kRadixBits - 1) / kRadixBits;
        if (b.sort_passes < 1) b.sort_passes = 1;
        if (b.sort_passes > kMaxPasses) return HGPU_ERR_UNSUPPORTED;
        // passes whose digit has at most 5 significant bits (the top of the key)
        b.sort_few_from = b.sort_passes;
        for (int p = 0; p < kMaxPasses; p++) {
            int bits = key_bits - p * kRadixBits;
            b.sort_few_values[p] = bits >= kRadixBits ? kRadix : (bits > 0 ? 1 << bits : 1);
            if (p < b.sort_passes && bits <= 5 && b.sort_few_from == b.sort_passes) b.sort_few_from = p;
        }
        // packed records (key bits and entry index in one or two words) when
        // they fit the W-word key buffers
        b.sort_key_bits = key_bits;
        b.sort_ibits = 1;
        while (b.sort_ibits < 32 && ((int64_t)1 << b.sort_ibits) < b.scap) b.sort_ibits++;
        b.sort_packed = 0;
        if (b.use_rank && key_bits + b.sort_ibits <= 64 * W) b.sort_packed = key_bits + b.sort_ibits <= 64 ? 1 : 2;
        b.binom = nullptr;
        if (b.use_rank) {
            if ((rc = upload(h, binom.data(), binom.size(), &b.binom))) return rc;
            const int words = b.sort_packed ? b.sort_packed : b.key_words;
            if ((rc = dalloc(h, &b.skeys, (size_t)b.scap * words))) return rc;
        }
    }
    if ((rc = dalloc(h, &b.ghist, (size_t)kMaxPasses * kRadix))) return rc;
    if ((rc = dalloc(h, &b.gofs, (size_t)kMaxPasses * kRadix))) return rc;
    CK(cudaMemset(b.ghist, 0, sizeof(uint32_t) * kMaxPasses * kRadix));
    {
        size_t tiles = (size_t)b.scap / OSConf<uint64_t, 2>::tile + 2;
        if ((rc = dalloc(h, &b.lookback, tiles * kRadix))) return rc;
        CK(cudaMemset(b.lookback, 0, sizeof(uint64_t) * tiles * kRadix));
        if ((rc = dalloc(h, &b.os_epoch, 1))) return rc;
        CK(cudaMemset(b.os_epoch, 0, sizeof(uint32_t)));
    }
    {
        // tiles of the annihilation over the merged main and spawned lists
        size_t tiles = ((size_t)b.cap + (size_t)b.scap) / kAnnTileMin + 2;
        if ((rc = dalloc(h, &b.msplit, 3 * (tiles + 1)))) return rc;
        if ((rc = dalloc(h, &b.seg_status, tiles))) return rc;
        CK(cudaMemset(b.seg_status, 0, sizeof(uint64_t) * tiles));
        if ((rc = dalloc(h, &b.seg_epoch, 1))) return rc;
        CK(cudaMemset(b.seg_epoch, 0, sizeof(uint32_t)));
    }
    // replica 2-RDM (density_matrices): the RDM, the cycle's RDM spawns, row sums
    b.rdm = nullptr;
    b.npairs = 0;
    if (h->cfg.density_matrices) {
        if (b.cap >= (int64_t)0xFFFFFFFF) return HGPU_ERR_UNSUPPORTED;  // 32-bit hash-table entries
        b.npairs = (int64_t)h->hsys.nbasis * (h->hsys.nbasis - 1) / 2;
        if ((rc = dalloc(h, &b.rdm, (size_t)(b.npairs * b.npairs)))) return rc;
        CK(cudaMemset(b.rdm, 0, sizeof(double) * (size_t)(b.npairs * b.npairs)));
        if ((rc = dalloc(h, &b.rdm_schild, (size_t)b.scap * W))) return rc;
        if ((rc = dalloc(h, &b.rdm_sparent, (size_t)b.scap))) return rc;
        if ((rc = dalloc(h, &b.rdm_spops, (size_t)b.scap))) return rc;
        if ((rc = dalloc(h, &b.rdm_sspace, (size_t)b.scap))) return rc;
        if ((rc = dalloc(h, &b.rdm_rows, (size_t)(2 * b.npairs)))) return rc;
        int64_t hs = 16;
        while (hs < b.cap + b.cap / 2) hs <<= 1;
        b.rdm_hash_mask = hs - 1;
        int ibits = 1;  // smallest with 2^ibits > cap: no entry equals the empty marker
        while (ibits < 32 && ((int64_t)1 << ibits) <= b.cap) ibits++;
        b.rdm_hash_tagmask = ibits >= 32 ? 0u : ~((1u << ibits) - 1u);
        CK(cudaStreamCreateWithFlags(&b.rdm_aux, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&b.rdm_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b.rdm_join, cudaEventDisableTiming));
        if ((rc = dalloc(h, &b.rdm_hash, (size_t)hs))) return rc;
    }
    if ((rc = dalloc(h, &b.scan_part, (size_t)kMaxBlocks * 2))) return rc;
    if ((rc = dalloc(h, &b.part_d, (size_t)kMaxBlocks * 4))) return rc;
    if ((rc = dalloc(h, &b.part_i, (size_t)kMaxBlocks * 4))) return rc;
    // Grids: sized to the lists, up to a few resident blocks per SM (every kernel
    // loops over its work, so a grid only bounds the parallelism): a small
    // calculation, one of many in a batch, does not launch thousands of idle blocks
    {
        auto clampi = [](int64_t v, int lo, int hi) { return (int)std::max<int64_t>(lo, std::min<int64_t>(hi, v)); };
        const int sms = h->sms;
        b.grid = clampi(b.cap / 4096, 8, std::min(4 * sms, kMaxBlocks));
        b.spawn_grid = clampi(b.scap / 1024, 8, 8 * sms);
        b.sort_grid = clampi(b.scap / OSConf<uint64_t, 1>::tile + 1, 4, 4 * sms);  // 256 threads, <= 48 KB shared memory
        b.splits_grid = clampi(((b.cap + b.scap) / kAnnTileMin + 3 + 7) / 8, 1, 4 * sms);  // a warp per cut
        b.spawn_chunk = 256;
    }
    b.ss_combined = h->cfg.semi_stoch_combined;
    if ((rc = dalloc(h, &b.state, 1))) return rc;
    CK(cudaMemset(b.state, 0, sizeof(DevState)));
    CK(cudaMemset(b.part_i, 0, sizeof(int64_t) * kMaxBlocks * 4));
    CK(cudaMemset(b.part_d, 0, sizeof(double) * kMaxBlocks * 4));
    return HGPU_OK;
}

static void invalidate_graphs(hgpu_handle *h) {
    for (int k = 0; k < 2; k++) {
        if (h->graph_ok[k]) cudaGraphExecDestroy(h->graph[k]);
        h->graph_ok[k] = false;
    }
}

// Free one allocation made by dalloc (and forget it).
static void dfree(hgpu_handle *h, const void *p) {
    if (!p) return;
    auto it = std::find(h->allocs.begin(), h->allocs.end(), const_cast<void *>(p));
    if (it == h->allocs.end()) return;
    h->allocs.erase(it);
    cudaFree(const_cast<void *>(p));
}

// Drop the deterministic space: its determinants, Hamiltonian columns and
// per-cycle vectors are freed and no state is deterministic any more.
static void ss_drop(hgpu_handle *h) {
    DevBuffers &b = h->b;
    dfree(h, b.ddets);
    dfree(h, b.dcol_ptr);
    dfree(h, b.dcol_i);
    dfree(h, b.dcol_h);
    dfree(h, b.dvec);
    dfree(h, b.dind);
    b.ddets = nullptr;
    b.dcol_ptr = nullptr;
    b.dcol_i = nullptr;
    b.dcol_h = nullptr;
    b.dvec = nullptr;
    b.dind = nullptr;
    b.nd = 0;
    h->ss_gen++;
}

// A main list that did not come from this calculation's own cycles (an upload,
// a restore, a restart) need not hold the deterministic states, which HANDE
// keeps in psip_list at all times: the space is dropped and built again at the
// next iteration from the new list, as a restarted calculation does --
// semi_stoch_iter = max(start_iter, mc_cycles_done + 1), or mc_cycles_done + 1
// when every shift already varies and shift_start_iteration is set
// (src/fciqmc.f90:229-235).
static void ss_reschedule(hgpu_handle *h) {
    if (h->cfg.semi_stoch_space == 0) return;
    bool all_vary = true;
    for (int s = 0; s < h->R; s++) all_vary = all_vary && h->vary_shift[s];
    h->ss_iter = std::max<int64_t>(h->cfg.semi_stoch_start_iter, h->iter + 1);
    if (all_vary && h->cfg.semi_stoch_shift_iter != -1) h->ss_iter = h->iter + 1;
    if (h->b.nd > 0 || h->b.ddets) {
        ss_drop(h);
        invalidate_graphs(h);
    }
}

static int read_state(hgpu_handle *h, DevState *st) {
    CK(cudaMemcpyAsync(st, h->b.state, sizeof(DevState), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HGPU_OK;
}

static int write_state(hgpu_handle *h, const DevState *st) {
    CK(cudaMemcpyAsync(h->b.state, st, sizeof(DevState), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HGPU_OK;
}

extern "C" {

int32_t hgpu_create(const hgpu_config *cfg, const hgpu_system *sys, hgpu_handle **out) {
    if (!cfg || !sys || !out) return HGPU_ERR_INVALID;
    *out = nullptr;
    if (sys->nwords < 1 || sys->nwords > HGPU_MAX_WORDS || sys->nbasis > 64 * sys->nwords ||
        sys->nbasis <= 64 * (sys->nwords - 1))
        return HGPU_ERR_INVALID;
    if (sys->nel < 2 || sys->nalpha + sys->nbeta != sys->nel) return HGPU_ERR_INVALID;
    if (cfg->nspaces < 1 || cfg->nspaces > HGPU_MAX_SPACES) return HGPU_ERR_INVALID;
    if (!(cfg->tau > 0.0)) return HGPU_ERR_INVALID;
    if (sys->kind == HGPU_SYS_HUB_K) {
        if (cfg->excit_gen != HGPU_EXCIT_GEN_RENORM && cfg->excit_gen != HGPU_EXCIT_GEN_NO_RENORM)
            return HGPU_ERR_UNSUPPORTED;
    } else if (sys->kind == HGPU_SYS_READ_IN) {
        bool hb = cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH || cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM ||
                  cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE;
        const bool pp_ij = cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
                           cfg->excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ;
        const bool ppn = cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN;
        const bool pp = pp_ij || ppn || cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC ||
                        cfg->excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC;
        if (cfg->excit_gen != HGPU_EXCIT_GEN_RENORM && cfg->excit_gen != HGPU_EXCIT_GEN_NO_RENORM &&
            cfg->excit_gen != HGPU_EXCIT_GEN_RENORM_SPIN && cfg->excit_gen != HGPU_EXCIT_GEN_NO_RENORM_SPIN && !hb &&
            !pp)
            return HGPU_ERR_UNSUPPORTED;
        if ((hb || pp_ij || ppn) && sys->nel > kHBMaxEl) return HGPU_ERR_UNSUPPORTED;
        if (pp && cfg->precision != HGPU_PREC_FP64) return HGPU_ERR_UNSUPPORTED;  // FP64 generator only
    } else {
        return HGPU_ERR_INVALID;
    }
    // src/check_input.F90:182-184
    if (!(cfg->power_pitzer_min_weight >= 0.0 && cfg->power_pitzer_min_weight <= 1.0)) return HGPU_ERR_INVALID;
    // semi-stochastic: a 'high' space (read_in: read_determ_space needs HDF5), not
    // combined with the replica RDM
    if (cfg->semi_stoch_space != 0 && cfg->semi_stoch_space != 1 && cfg->semi_stoch_space != 4)
        return HGPU_ERR_UNSUPPORTED;
    if (cfg->semi_stoch_space != 0 && cfg->density_matrices) return HGPU_ERR_UNSUPPORTED;
    if (cfg->semi_stoch_combined != 0 && cfg->semi_stoch_combined != 1) return HGPU_ERR_INVALID;
    if ((cfg->semi_stoch_space == 1 && cfg->semi_stoch_size < 1) ||
        (cfg->semi_stoch_space == 4 && cfg->semi_stoch_ci_level < 0))
        return HGPU_ERR_INVALID;
    // density_matrices: replica sampling of molecular systems (two spaces)
    if (cfg->density_matrices && (sys->kind != HGPU_SYS_READ_IN || cfg->nspaces != 2)) return HGPU_ERR_INVALID;
    // pattempt_parallel only with the spin-resolved generators, at most 1
    // (src/check_input.F90:212-218)
    {
        const bool spin_gen = sys->kind == HGPU_SYS_READ_IN && (cfg->excit_gen == HGPU_EXCIT_GEN_RENORM_SPIN ||
                                                                 cfg->excit_gen == HGPU_EXCIT_GEN_NO_RENORM_SPIN);
        if (cfg->pattempt_parallel > 0.0 && (!spin_gen || cfg->pattempt_parallel > 1.0)) return HGPU_ERR_INVALID;
    }
    int ndev = hgpu_device_count();
    if (ndev <= 0) return HGPU_ERR_NO_DEVICE;
    hgpu_handle *h = new (std::nothrow) hgpu_handle();
    if (!h) return HGPU_ERR_OOM;
    h->cfg = *cfg;
    h->W = sys->nwords;
    h->R = cfg->nspaces;
    h->kind = sys->kind;
    h->gkind = sys->kind;
    if (sys->kind == HGPU_SYS_READ_IN) {
        if (cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH) h->gkind = kKindHeatBath;
        else if (cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_UNIFORM ||
                 cfg->excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE)
            h->gkind = kKindHeatBathUniform;  // the singles differ at run time
        else if (cfg->excit_gen == HGPU_EXCIT_GEN_NO_RENORM || cfg->excit_gen == HGPU_EXCIT_GEN_NO_RENORM_SPIN)
            h->gkind = kKindReadInNoRenorm;
        else if (cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC ||
                 cfg->excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC ||
                 cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_OCC_IJ ||
                 cfg->excit_gen == HGPU_EXCIT_GEN_CAUCHY_SCHWARZ_OCC_IJ)
            h->gkind = kKindPowerPitzerOcc;
        else if (cfg->excit_gen == HGPU_EXCIT_GEN_POWER_PITZER_ORDERN)
            h->gkind = kKindPowerPitzerRef;
    }
    h->use_graphs = getenv("HGPU_NO_GRAPH") == nullptr;
    // semi_stoch_iter = max(start_iter, mc_cycles_done + 1) (src/fciqmc.f90:229)
    h->ss_iter = INT64_MAX;
    if (cfg->semi_stoch_space != 0) h->ss_iter = cfg->semi_stoch_start_iter > 1 ? cfg->semi_stoch_start_iter : 1;
    cudaGetDevice(&h->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    if (sms <= 0) sms = 148;
    h->sms = sms;
    int rc = HGPU_OK;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) rc = HGPU_ERR_CUDA;
    if (!rc) rc = build_system(h, sys);
    if (!rc) {
        // exact-diagonal tables above 32 KB (molecules beyond ~45 orbitals) stay in
        // global memory, where the L1 cache holds them, so that they do not cost
        // the annihilation kernel resident blocks
        const size_t fx = sizeof(int64_t) * (size_t)fx_table_words(sys->kind, sys->nbasis, sys->norb);
        h->b.fx_smem_bytes = fx <= 32768 ? fx : 0;
        if (set_kernel_attributes(h->b)) {
            last_error_text(cudaGetErrorString(cudaGetLastError()), "cudaFuncSetAttribute");
            rc = HGPU_ERR_CUDA;
        }
    }
    if (!rc) rc = alloc_lists(h);
    if (!rc) {
        cudaEventCreate(&h->ev0);
        cudaEventCreate(&h->ev1);
        for (int s = 0; s < HGPU_MAX_SPACES; s++) h->shift[s] = cfg->initial_shift;
    }
    if (rc) {
        hgpu_destroy(h);
        return rc;
    }
    *out = h;
    return HGPU_OK;
}

int32_t hgpu_destroy(hgpu_handle *h) {
    if (!h) return HGPU_ERR_INVALID;
    if (h->stream) cudaStreamSynchronize(h->stream);
    invalidate_graphs(h);
    for (void *p : h->allocs) cudaFree(p);
    if (h->scratch) cudaFree(h->scratch);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->b.rdm_fork) cudaEventDestroy(h->b.rdm_fork);
    if (h->b.rdm_join) cudaEventDestroy(h->b.rdm_join);
    if (h->b.rdm_aux) cudaStreamDestroy(h->b.rdm_aux);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return HGPU_OK;
}

// Host pages that the CPU has not touched for a while were copied by the GPU
// at a fraction of the link's rate: on the GB300's C2C link a 4.6 GB list went up
// in 57-140 ms instead of 22 ms, and an 8.7 GB list came down in up to 187 ms
// instead of 45, the difference varying from one call to the next as the
// operating system ages the pages.  One CPU access per page just before the
// copy -- a read of a source page, a write of a destination page (a byte the
// copy overwrites) -- removes it, for about 0.4 ms per GB with 64 KB pages.
static size_t host_page_size() {
    static const size_t page = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    return page;
}

static void touch_host_pages(const void *p, size_t bytes) {
    const size_t page = host_page_size();
    const volatile unsigned char *c = static_cast<const volatile unsigned char *>(p);
    unsigned char sink = 0;
    for (size_t off = 0; off < bytes; off += page) sink ^= c[off];
    if (bytes) sink ^= c[bytes - 1];
    (void)sink;
}

static void touch_host_pages_for_write(void *p, size_t bytes) {
    const size_t page = host_page_size();
    volatile unsigned char *c = static_cast<volatile unsigned char *>(p);
    for (size_t off = 0; off < bytes; off += page) c[off] = 0;
    if (bytes) c[bytes - 1] = 0;
}

static int set_list(hgpu_handle *h, const int64_t *states, const int64_t *pops, const double *dat, int64_t n,
                    bool compute_kii) {
    if (n < 0 || n > h->b.cap) return HGPU_ERR_INVALID;
    int W = h->W, R = h->R;
    ss_reschedule(h);
    h->cur = 0;
    if (n > 0) {
        touch_host_pages(states, sizeof(uint64_t) * W * n);
        CK(cudaMemcpyAsync(h->b.dets[0], states, sizeof(uint64_t) * W * n, cudaMemcpyHostToDevice, h->stream));
        touch_host_pages(pops, sizeof(int64_t) * R * n);
        CK(cudaMemcpyAsync(h->b.pops[0], pops, sizeof(int64_t) * R * n, cudaMemcpyHostToDevice, h->stream));
        if (dat && !compute_kii) {
            touch_host_pages(dat, sizeof(double) * n);
            CK(cudaMemcpyAsync(h->b.kii[0], dat, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
        }
        else
            launch_eval_diagonal(h->b, W, h->b.dets[0], n, h->b.kii[0], h->stream);
    }
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    st.n_main = n;
    st.abs_pop[0] = st.abs_pop[1] = 0;
    // the cycles read the shift from the device state: publish the current one
    for (int s = 0; s < HGPU_MAX_SPACES; s++) st.shift[s] = h->shift[s];
    if ((rc = write_state(h, &st))) return rc;
    launch_abs_pop(h->b, R, 0, h->stream);
    if ((rc = read_state(h, &st))) return rc;
    for (int s = 0; s < R; s++) h->nparticles_old[s] = (double)st.abs_pop[s] / (double)h->hsys.real_factor;
    return HGPU_OK;
}

int32_t hgpu_initial_distribution(hgpu_handle *h) {
    if (!h) return HGPU_ERR_INVALID;
    int64_t st[HGPU_MAX_WORDS], po[HGPU_MAX_SPACES];
    for (int w = 0; w < h->W; w++) st[w] = (int64_t)h->hsys.f0[w];
    for (int s = 0; s < h->R; s++) po[s] = (int64_t)llround(h->cfg.D0_population) * h->hsys.real_factor;
    double kii = 0.0;
    DevState ds;
    int rc = read_state(h, &ds);
    if (rc) return rc;
    memset(&ds, 0, sizeof(ds));
    for (int s = 0; s < HGPU_MAX_SPACES; s++) {
        h->shift[s] = h->cfg.initial_shift;
        h->vary_shift[s] = 0;
        ds.shift[s] = h->cfg.initial_shift;
    }
    h->iter = 0;
    if ((rc = write_state(h, &ds))) return rc;
    return set_list(h, st, po, &kii, 1, false);
}

int32_t hgpu_upload_walkers(hgpu_handle *h, const int64_t *states, const int64_t *pops, const double *dat,
                            int64_t n) {
    if (!h || (n > 0 && (!states || !pops))) return HGPU_ERR_INVALID;
    return set_list(h, states, pops, dat, n, dat == nullptr);
}

int32_t hgpu_rdm_download(hgpu_handle *h, double *rdm, int64_t capacity, int64_t *n_out) {
    if (!h || !n_out) return HGPU_ERR_INVALID;
    *n_out = h->b.rdm ? h->b.npairs * h->b.npairs : 0;
    if (!h->b.rdm || !rdm) return HGPU_OK;  // a query of the size
    if (capacity < *n_out) return HGPU_ERR_INVALID;
    CK(cudaMemcpyAsync(rdm, h->b.rdm, sizeof(double) * (size_t)*n_out, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HGPU_OK;
}

int32_t hgpu_download_walkers(hgpu_handle *h, int64_t *states, int64_t *pops, double *dat, int64_t capacity,
                              int64_t *n_out) {
    if (!h || !n_out) return HGPU_ERR_INVALID;
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    *n_out = st.n_main;
    if (capacity < st.n_main) return HGPU_ERR_INVALID;
    int64_t n = st.n_main;
    if (n > 0) {
        if (states) {
            touch_host_pages_for_write(states, sizeof(uint64_t) * h->W * n);
            CK(cudaMemcpyAsync(states, h->b.dets[h->cur], sizeof(uint64_t) * h->W * n, cudaMemcpyDeviceToHost,
                               h->stream));
        }
        if (pops) {
            touch_host_pages_for_write(pops, sizeof(int64_t) * h->R * n);
            CK(cudaMemcpyAsync(pops, h->b.pops[h->cur], sizeof(int64_t) * h->R * n, cudaMemcpyDeviceToHost, h->stream));
        }
        if (dat) {
            touch_host_pages_for_write(dat, sizeof(double) * n);
            CK(cudaMemcpyAsync(dat, h->b.kii[h->cur], sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
    }
    return HGPU_OK;
}

// init_semi_stoch_t (src/semi_stoch.F90:134-377) for a 'high' space, at the
// start of the cycle that builds it: find_most_populated_dets (:1318-1385;
// the first smallest entry is replaced, so a min-heap of (population, slot)
// gives the same set), the space sorted into the main list's order, its
// absent determinants added with zero population (add_determ_dets_to_psip_list,
// :728-793), then the Hamiltonian by column on the device.
static int ss_init(hgpu_handle *h) {
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    const int W = h->W, R = h->R;
    const int64_t n = st.n_main;
    std::vector<uint64_t> dets((size_t)n * W);
    std::vector<int64_t> pops((size_t)n * R);
    if (n > 0) {
        CK(cudaMemcpyAsync(dets.data(), h->b.dets[h->cur], sizeof(uint64_t) * W * n, cudaMemcpyDeviceToHost,
                           h->stream));
        CK(cudaMemcpyAsync(pops.data(), h->b.pops[h->cur], sizeof(int64_t) * R * n, cudaMemcpyDeviceToHost,
                           h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    auto less = [&](const uint64_t *a, const uint64_t *b) {
        for (int w = W - 1; w >= 0; w--)
            if (a[w] != b[w]) return a[w] < b[w];
        return false;
    };
    std::vector<uint64_t> dd;
    int64_t K = 0;
    // a space built before (a rebuild after a restart) is freed first
    ss_drop(h);
    invalidate_graphs(h);
    if (h->cfg.semi_stoch_space == 4) {
        // create_ci_determ_space (src/semi_stoch.F90:1763-1805): every
        // determinant of the reference's spin and symmetry within ci_level
        // excitations of it
        const uint64_t *f0 = h->hsys.f0;
        std::vector<int> occ, virt;
        for (int p = 0; p < h->hsys.nbasis; p++) {
            if ((f0[p >> 6] >> (p & 63)) & 1u) occ.push_back(p);
            else virt.push_back(p);
        }
        // spin orbitals alternate alpha (even) and beta (odd).  The symmetry
        // change of the holes and particles so far: molecular irreps combine by
        // XOR (identity 0), Hubbard crystal momenta by sym_table (a hole adds
        // -k, a particle +k; identity the Gamma point, k + (-k))
        auto alpha = [](int p) { return (p & 1) == 0 ? 1 : 0; };
        const bool hubk = h->kind == HGPU_SYS_HUB_K;
        const uint8_t *sym = h->hsys.orbsym;
        const int nk = hubk ? (int)h->h_invsym.size() : 0;
        const int ident = hubk ? h->h_symtab[h->h_invsym[0]] : 0;  // k_0 + (-k_0) = Gamma
        auto with = [&](int sy, int p, bool hole) {
            if (!hubk) return sy ^ (int)sym[p];
            const int k = p >> 1;  // the k-point of spin orbital p
            return h->h_symtab[sy * nk + (hole ? h->h_invsym[k] : k)];
        };
        std::vector<uint64_t> f(f0, f0 + W);
        std::function<void(size_t, int, int, int)> parts = [&](size_t v, int k, int na, int sy) {
            if (k == 0) {
                if (na == 0 && sy == ident) dd.insert(dd.end(), f.begin(), f.end());
                return;
            }
            for (size_t q = v; q + k <= virt.size(); q++) {
                const int p = virt[q], a = alpha(p);
                if (na - a < 0) continue;
                f[p >> 6] |= 1ull << (p & 63);
                parts(q + 1, k - 1, na - a, with(sy, p, false));
                f[p >> 6] &= ~(1ull << (p & 63));
            }
        };
        std::function<void(size_t, int, int, int, int)> holes = [&](size_t o, int k, int kk, int na, int sy) {
            if (k == 0) {
                parts(0, kk, na, sy);
                return;
            }
            for (size_t q = o; q + k <= occ.size(); q++) {
                const int p = occ[q];
                f[p >> 6] &= ~(1ull << (p & 63));
                holes(q + 1, k - 1, kk, na + alpha(p), with(sy, p, true));
                f[p >> 6] |= 1ull << (p & 63);
            }
        };
        for (int k = 0; k <= h->cfg.semi_stoch_ci_level && k <= (int)occ.size() && k <= (int)virt.size(); k++)
            holes(0, k, k, 0, ident);
        K = (int64_t)(dd.size() / W);
        std::vector<int64_t> order(K);
        for (int64_t k = 0; k < K; k++) order[k] = k;
        std::sort(order.begin(), order.end(),
                  [&](int64_t x, int64_t y) { return less(&dd[(size_t)x * W], &dd[(size_t)y * W]); });
        std::vector<uint64_t> sorted((size_t)K * W);
        for (int64_t k = 0; k < K; k++)
            for (int w = 0; w < W; w++) sorted[(size_t)k * W + w] = dd[(size_t)order[k] * W + w];
        dd.swap(sorted);
    } else {
        K = std::min<int64_t>(h->cfg.semi_stoch_size, n);
        auto tot = [&](int64_t i) {
            int64_t p = 0;
            for (int s = 0; s < R; s++) p += std::llabs(pops[(size_t)i * R + s]);
            return p;
        };
        std::vector<int64_t> slot_of(K > 0 ? K : 0);
        std::priority_queue<std::pair<int64_t, int64_t>, std::vector<std::pair<int64_t, int64_t>>,
                            std::greater<std::pair<int64_t, int64_t>>>
            heap;
        for (int64_t i = 0; i < K; i++) {
            slot_of[i] = i;
            heap.push({tot(i), i});
        }
        for (int64_t i = K; i < n && K > 0; i++) {
            const int64_t p = tot(i);
            if (p > heap.top().first) {
                const int64_t sl = heap.top().second;
                heap.pop();
                slot_of[sl] = i;
                heap.push({p, sl});
            }
        }
        // the main list is sorted, so the selected entries in index order are
        // the space in main-list order
        std::sort(slot_of.begin(), slot_of.end());
        dd.resize((size_t)(K > 0 ? K : 0) * W);
        for (int64_t k = 0; k < K; k++)
            for (int w = 0; w < W; w++) dd[(size_t)k * W + w] = dets[(size_t)slot_of[k] * W + w];
    }
    if (K < 1) return HGPU_OK;
    uint64_t *ddets;
    if ((rc = dalloc(h, &ddets, (size_t)K * W))) return rc;
    CK(cudaMemcpy(ddets, dd.data(), sizeof(uint64_t) * K * W, cudaMemcpyHostToDevice));
    h->b.ddets = ddets;
    h->b.nd = K;
    // the Hamiltonian by column: count, offsets, fill
    int64_t *counts;
    if ((rc = dalloc(h, &counts, (size_t)K))) return rc;
    launch_determ_columns(h->b, W, h->kind, false, counts, nullptr, nullptr, h->stream);
    std::vector<int64_t> cnt(K), ptr(K + 1);
    CK(cudaMemcpyAsync(cnt.data(), counts, sizeof(int64_t) * K, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    dfree(h, counts);
    ptr[0] = 0;
    for (int64_t k = 0; k < K; k++) ptr[k + 1] = ptr[k] + cnt[k];
    int64_t *dptr;
    int32_t *ci;
    double *ch, *dvec;
    int64_t *dind;
    if ((rc = dalloc(h, &dptr, (size_t)K + 1)) || (rc = dalloc(h, &ci, (size_t)ptr[K])) ||
        (rc = dalloc(h, &ch, (size_t)ptr[K])) || (rc = dalloc(h, &dvec, (size_t)K * R)) ||
        (rc = dalloc(h, &dind, (size_t)K)))
        return rc;
    CK(cudaMemcpy(dptr, ptr.data(), sizeof(int64_t) * (K + 1), cudaMemcpyHostToDevice));
    h->b.dcol_ptr = dptr;
    launch_determ_columns(h->b, W, h->kind, true, nullptr, ci, ch, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    h->b.dcol_i = ci;
    h->b.dcol_h = ch;
    h->b.dvec = dvec;
    h->b.dind = dind;
    h->ss_gen++;
    // absent determinants join the main list with zero population
    std::vector<uint64_t> nd_;
    std::vector<int64_t> np_;
    nd_.reserve((size_t)(n + K) * W);
    np_.reserve((size_t)(n + K) * R);
    int64_t added = 0;
    {
        int64_t i = 0, k = 0;
        while (i < n || k < K) {
            const uint64_t *dm = i < n ? &dets[(size_t)i * W] : nullptr;
            const uint64_t *dk = k < K ? &dd[(size_t)k * W] : nullptr;
            if (dk && (!dm || less(dk, dm))) {
                nd_.insert(nd_.end(), dk, dk + W);
                for (int s = 0; s < R; s++) np_.push_back(0);
                added++;
                k++;
            } else {
                nd_.insert(nd_.end(), dm, dm + W);
                for (int s = 0; s < R; s++) np_.push_back(pops[(size_t)i * R + s]);
                if (dk && !less(dm, dk)) k++;  // present in both
                i++;
            }
        }
    }
    if (added > 0) {
        const int64_t m = n + added;
        if (m > h->b.cap) return HGPU_ERR_MAIN_OVERFLOW;
        CK(cudaMemcpyAsync(h->b.dets[h->cur], nd_.data(), sizeof(uint64_t) * W * m, cudaMemcpyHostToDevice,
                           h->stream));
        CK(cudaMemcpyAsync(h->b.pops[h->cur], np_.data(), sizeof(int64_t) * R * m, cudaMemcpyHostToDevice,
                           h->stream));
        launch_eval_diagonal(h->b, W, h->b.dets[h->cur], m, h->b.kii[h->cur], h->stream);
        st.n_main = m;
        if ((rc = write_state(h, &st))) return rc;
    }
    invalidate_graphs(h);
    return HGPU_OK;
}

static int launch_one_cycle(hgpu_handle *h) {
    int cur = h->cur;
    if (h->use_graphs) {
        if (!h->graph_ok[cur]) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            launch_cycle(h->b, h->W, h->R, h->gkind, h->cfg.precision, cur, h->stream);
            CK(cudaStreamEndCapture(h->stream, &g));
            cudaError_t e = cudaGraphInstantiate(&h->graph[cur], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                last_error_text(cudaGetErrorString(e), "cudaGraphInstantiate");
                return HGPU_ERR_CUDA;
            }
            h->graph_ok[cur] = true;
        }
        CK(cudaGraphLaunch(h->graph[cur], h->stream));
    } else {
        launch_cycle(h->b, h->W, h->R, h->gkind, h->cfg.precision, cur, h->stream);
        CK(cudaGetLastError());
    }
    h->cur = 1 - cur;
    return HGPU_OK;
}

// The start of a report with density_matrices (src/fciqmc.f90:283-291): the RDM
// is cleared once accumulating, and accumulating starts in the first report
// after density_matrix_report in which every shift varies.
static int begin_report(hgpu_handle *h) {
    if (h->report_open) return HGPU_OK;
    h->report_open = true;
    if (!h->b.rdm) return HGPU_OK;
    if (h->rdm_on)
        CK(cudaMemsetAsync(h->b.rdm, 0, sizeof(double) * (size_t)(h->b.npairs * h->b.npairs), h->stream));
    bool all_vary = true;
    for (int s = 0; s < h->R; s++) all_vary = all_vary && h->vary_shift[s];
    if (!h->rdm_on && all_vary && h->reports_done + 1 > h->cfg.density_matrix_report) {
        h->rdm_on = 1;
        CK(cudaMemcpyAsync(&h->b.state->rdm_on, &h->rdm_on, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    return HGPU_OK;
}

int32_t hgpu_run_cycles(hgpu_handle *h, int32_t ncycles) {
    if (!h || ncycles < 0) return HGPU_ERR_INVALID;
    {
        int rc = begin_report(h);
        if (rc) return rc;
    }
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int k = 0; k < ncycles; k++) {
        int rc;
        if (h->ss_iter == h->iter + k + 1 && (rc = ss_init(h))) return rc;
        rc = launch_one_cycle(h);
        if (rc) return rc;
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->report_ms += ms;
    h->iter += ncycles;
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    if (st.error_flags & HGPU_FLAG_SPAWN_OVERFLOW) return HGPU_ERR_SPAWN_OVERFLOW;
    if (st.error_flags & HGPU_FLAG_MAIN_OVERFLOW) return HGPU_ERR_MAIN_OVERFLOW;
    if (st.error_flags & HGPU_FLAG_TIMEOUT) return HGPU_ERR_TIMEOUT;
    return HGPU_OK;
}

// ---------------------------------------------------------------------------
// Batches of handles: one graph launch per cycle for all of them
// ---------------------------------------------------------------------------
struct hgpu_batch {
    std::vector<hgpu_handle *> hs;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    std::vector<int> parity[2];  // buffer parity of every handle each graph was built for
    std::vector<int64_t> gens;   // launch shapes (launch_gen) the graphs were built with
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void batch_free_graphs(hgpu_batch *b) {
    for (int k = 0; k < 2; k++) {
        if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
        b->exec[k] = nullptr;
        b->parity[k].clear();
    }
}

// One graph whose independent branches are the handles' cycles at the given
// buffer parities (each captured on its handle's stream, then added as a child
// graph, which the graph copies).
static int batch_build(hgpu_batch *b, int slot, const std::vector<int> &par) {
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    for (size_t i = 0; i < b->hs.size(); i++) {
        hgpu_handle *h = b->hs[i];
        cudaGraph_t hg;
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            launch_cycle(h->b, h->W, h->R, h->gkind, h->cfg.precision, par[i], h->stream);
            e = cudaStreamEndCapture(h->stream, &hg);
        }
        cudaGraphNode_t node;
        if (e == cudaSuccess) {
            e = cudaGraphAddChildGraphNode(&node, g, nullptr, 0, hg);
            cudaGraphDestroy(hg);
        }
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            last_error_text(cudaGetErrorString(e), "batch graph");
            return HGPU_ERR_CUDA;
        }
    }
    cudaError_t e = cudaGraphInstantiate(&b->exec[slot], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->exec[slot] = nullptr;
        last_error_text(cudaGetErrorString(e), "cudaGraphInstantiate");
        return HGPU_ERR_CUDA;
    }
    b->parity[slot] = par;
    return HGPU_OK;
}

int32_t hgpu_batch_create(hgpu_handle *const *handles, int32_t n, hgpu_batch **out) {
    if (!handles || n < 1 || !out) return HGPU_ERR_INVALID;
    *out = nullptr;
    int dev = -1;
    cudaGetDevice(&dev);
    std::vector<hgpu_handle *> hs(handles, handles + n);
    for (int i = 0; i < n; i++) {
        if (!hs[i] || hs[i]->device != dev) return HGPU_ERR_INVALID;
        if (hs[i]->cfg.semi_stoch_space != 0) return HGPU_ERR_UNSUPPORTED;  // its space is built between cycles
        for (int j = 0; j < i; j++)
            if (hs[j] == hs[i]) return HGPU_ERR_INVALID;
    }
    hgpu_batch *b = new (std::nothrow) hgpu_batch();
    if (!b) return HGPU_ERR_OOM;
    b->hs = hs;
    b->device = dev;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
        hgpu_batch_destroy(b);
        return HGPU_ERR_CUDA;
    }
    *out = b;
    return HGPU_OK;
}

int32_t hgpu_batch_run_cycles(hgpu_batch *b, int32_t ncycles) {
    if (!b || ncycles < 0) return HGPU_ERR_INVALID;
    std::vector<int> par(b->hs.size()), flip(b->hs.size());
    for (size_t i = 0; i < b->hs.size(); i++) {
        int rc = begin_report(b->hs[i]);
        if (rc) return rc;
        par[i] = b->hs[i]->cur;
        flip[i] = 1 - par[i];
        CK(cudaStreamSynchronize(b->hs[i]->stream));  // earlier per-handle work
    }
    std::vector<int64_t> gens(b->hs.size());
    for (size_t i = 0; i < b->hs.size(); i++) gens[i] = b->hs[i]->launch_gen;
    if (gens != b->gens) {
        batch_free_graphs(b);
        b->gens = gens;
    }
    int slot;
    if (b->exec[0] && b->parity[0] == par) {
        slot = 0;
    } else if (b->exec[1] && b->parity[1] == par) {
        slot = 1;
    } else {
        batch_free_graphs(b);
        int rc = batch_build(b, 0, par);
        if (!rc) rc = batch_build(b, 1, flip);
        if (rc) return rc;
        slot = 0;
    }
    CK(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k < ncycles; k++) {
        CK(cudaGraphLaunch(b->exec[slot], b->stream));
        slot ^= 1;
    }
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    int first = HGPU_OK;
    for (hgpu_handle *h : b->hs) {
        h->cur ^= ncycles & 1;
        h->iter += ncycles;
        h->report_ms += ms;
        DevState st;
        int rc = read_state(h, &st);
        if (!rc && (st.error_flags & HGPU_FLAG_SPAWN_OVERFLOW)) rc = HGPU_ERR_SPAWN_OVERFLOW;
        if (!rc && (st.error_flags & HGPU_FLAG_MAIN_OVERFLOW)) rc = HGPU_ERR_MAIN_OVERFLOW;
        if (!rc && (st.error_flags & HGPU_FLAG_TIMEOUT)) rc = HGPU_ERR_TIMEOUT;
        if (rc && !first) first = rc;
    }
    return first;
}

int32_t hgpu_get_launch(hgpu_handle *h, hgpu_launch *out) {
    if (!h || !out) return HGPU_ERR_INVALID;
    out->spawn_chunk = h->b.spawn_chunk;
    out->spawn_blocks = h->b.spawn_grid;
    out->stream_blocks = h->b.grid;
    out->sort_blocks = h->b.sort_grid;
    return HGPU_OK;
}

int32_t hgpu_set_launch(hgpu_handle *h, const hgpu_launch *in) {
    if (!h || !in) return HGPU_ERR_INVALID;
    if (in->spawn_chunk < 32 || in->spawn_chunk > kSpawnChunk || in->spawn_chunk % 32 != 0 || in->spawn_blocks < 1 ||
        in->stream_blocks < 1 || in->stream_blocks > kMaxBlocks || in->sort_blocks < 1)
        return HGPU_ERR_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    h->b.spawn_chunk = in->spawn_chunk;
    h->b.spawn_grid = in->spawn_blocks;
    h->b.grid = in->stream_blocks;
    h->b.sort_grid = in->sort_blocks;
    invalidate_graphs(h);
    h->launch_gen++;
    return HGPU_OK;
}

int32_t hgpu_batch_destroy(hgpu_batch *b) {
    if (!b) return HGPU_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_free_graphs(b);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return HGPU_OK;
}

int32_t hgpu_end_report(hgpu_handle *h, hgpu_report *out) {
    if (!h || !out) return HGPU_ERR_INVALID;
    // calc_rdm_energy of the report's RDM (src/fciqmc.f90:409-411)
    if (h->rdm_on) launch_rdm_energy(h->b, h->W, h->stream);
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    if (h->rdm_on) {
        out->rdm_energy = st.rdm_energy;
        out->rdm_trace = st.rdm_trace;
    }
    h->reports_done++;
    h->report_open = false;
    int R = h->R;
    int nc = st.rep_cycles > 0 ? st.rep_cycles : 1;
    double ntot[HGPU_MAX_SPACES] = {0, 0};
    for (int s = 0; s < R; s++) {
        out->proj_energy[s] = (st.acc_proj[s] + st.acc_proj_c[s]) / (double)nc;
        out->D0_population[s] = (st.acc_d0[s] + st.acc_d0_c[s]) / (double)nc;
        ntot[s] = (double)st.abs_pop[s] / (double)h->hsys.real_factor;
    }
    // update_shift (src/energy_evaluation.F90:659-711): the damping term, then the
    // harmonic forcing toward target_particles
    for (int s = 0; s < R; s++)
        if (h->vary_shift[s]) {
            h->shift[s] = h->shift[s] - std::log(ntot[s] / h->nparticles_old[s]) * h->cfg.shift_damping /
                                            (1.0 * h->cfg.tau * (double)nc);
            if (h->cfg.shift_harmonic_forcing != 0.0 && h->cfg.target_particles > 0.0)
                h->shift[s] = h->shift[s] - std::log(ntot[s] / h->cfg.target_particles) *
                                                h->cfg.shift_harmonic_forcing / (1.0 * h->cfg.tau * (double)nc);
        }
    for (int s = 0; s < R; s++) h->nparticles_old[s] = ntot[s];
    bool all_vary_before = true, all_vary = true;
    for (int s = 0; s < R; s++) all_vary_before = all_vary_before && h->vary_shift[s];
    for (int s = 0; s < R; s++) {
        const double above = h->cfg.target_reference ? out->D0_population[s] : ntot[s];
        if (!h->vary_shift[s] && above > h->cfg.target_particles) {
            h->vary_shift[s] = 1;
            h->shift[s] = h->cfg.vary_shift_from_proje ? out->proj_energy[s] / out->D0_population[s]
                                                       : h->cfg.vary_shift_from;
        }
    }
    // the deterministic space follows the shift (src/qmc_common.F90:1203-1204)
    for (int s = 0; s < R; s++) all_vary = all_vary && h->vary_shift[s];
    if (!all_vary_before && all_vary && h->cfg.semi_stoch_space != 0 && h->cfg.semi_stoch_shift_iter != -1)
        h->ss_iter = h->cfg.semi_stoch_shift_iter + st.iter + 1;
    for (int s = 0; s < R; s++) {
        out->shift[s] = h->shift[s];
        out->nparticles[s] = ntot[s];
        out->vary_shift[s] = h->vary_shift[s];
    }
    out->iteration = st.iter;
    out->nstates = st.n_main;
    out->nspawn_events = st.last_nspawn_events;
    out->rspawn = st.acc_rspawn / (double)nc;
    out->nattempts = st.acc_attempts;
    out->nspawned = st.acc_spawned;
    out->error_flags = st.error_flags;
    out->device_ms = h->report_ms;
    h->report_ms = 0.0;
    out->nblooms = st.bloom_n;
    out->tot_bloom = (double)st.bloom_tot / (double)h->hsys.real_factor;
    out->max_bloom = (double)st.bloom_max / (double)h->hsys.real_factor;
    // reset the report accumulators, publish the new shift
    for (int s = 0; s < HGPU_MAX_SPACES; s++) {
        st.shift[s] = h->shift[s];
        st.acc_proj[s] = st.acc_proj_c[s] = st.acc_d0[s] = st.acc_d0_c[s] = 0.0;
    }
    st.acc_rspawn = 0.0;
    st.acc_attempts = st.acc_spawned = 0;
    st.rep_cycles = 0;
    st.bloom_n = st.bloom_tot = 0;  // bloom_stats_init_report_loop
    if ((rc = write_state(h, &st))) return rc;
    if (out->error_flags & HGPU_FLAG_SPAWN_OVERFLOW) return HGPU_ERR_SPAWN_OVERFLOW;
    if (out->error_flags & HGPU_FLAG_MAIN_OVERFLOW) return HGPU_ERR_MAIN_OVERFLOW;
    if (out->error_flags & HGPU_FLAG_TIMEOUT) return HGPU_ERR_TIMEOUT;
    return HGPU_OK;
}

int32_t hgpu_run_report(hgpu_handle *h, hgpu_report *out) {
    if (!h) return HGPU_ERR_INVALID;
    int rc = hgpu_run_cycles(h, h->cfg.ncycles);
    if (rc && rc != HGPU_ERR_SPAWN_OVERFLOW && rc != HGPU_ERR_MAIN_OVERFLOW) return rc;
    return hgpu_end_report(h, out);
}

int32_t hgpu_get_state(hgpu_handle *h, hgpu_state *out) {
    if (!h || !out) return HGPU_ERR_INVALID;
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->iteration = st.iter;
    for (int s = 0; s < HGPU_MAX_SPACES; s++) {
        out->shift[s] = h->shift[s];
        out->vary_shift[s] = h->vary_shift[s];
        out->nparticles_old[s] = h->nparticles_old[s];
    }
    out->tau = h->cfg.tau;
    out->seed = h->cfg.seed;
    return HGPU_OK;
}

int32_t hgpu_set_state(hgpu_handle *h, const hgpu_state *in) {
    if (!h || !in) return HGPU_ERR_INVALID;
    DevState st;
    int rc = read_state(h, &st);
    if (rc) return rc;
    st.iter = in->iteration;
    for (int s = 0; s < HGPU_MAX_SPACES; s++) {
        h->shift[s] = in->shift[s];
        h->vary_shift[s] = in->vary_shift[s];
        h->nparticles_old[s] = in->nparticles_old[s];
        st.shift[s] = in->shift[s];
    }
    h->iter = in->iteration;
    // a restarted calculation builds its deterministic space again:
    // semi_stoch_iter = max(start_iter, mc_cycles_done + 1), or mc_cycles_done + 1
    // when every shift already varies and shift_start_iteration is set
    // (src/fciqmc.f90:229-235)
    ss_reschedule(h);
    return write_state(h, &st);
}

// Checkpoint layout: magic, version, nwords, nspaces, n, hgpu_state, then
// states (nwords*n int64), pops (nspaces*n int64), dat (n double).
static const char kMagic[8] = {'H', 'G', 'P', 'U', 'C', 'K', 'P', 'T'};

int32_t hgpu_checkpoint(hgpu_handle *h, const char *path) {
    if (!h || !path) return HGPU_ERR_INVALID;
    int64_t n = 0;
    int rc = hgpu_download_walkers(h, nullptr, nullptr, nullptr, 0, &n);
    if (rc && rc != HGPU_ERR_INVALID) return rc;
    std::vector<int64_t> st((size_t)(n * h->W + 1)), po((size_t)(n * h->R + 1));
    std::vector<double> da((size_t)(n + 1));
    if ((rc = hgpu_download_walkers(h, st.data(), po.data(), da.data(), n, &n))) return rc;
    hgpu_state s;
    if ((rc = hgpu_get_state(h, &s))) return rc;
    FILE *fp = fopen(path, "wb");
    if (!fp) return HGPU_ERR_INVALID;
    int32_t hdr[4] = {1, h->W, h->R, 0};
    bool ok = fwrite(kMagic, 1, 8, fp) == 8 && fwrite(hdr, sizeof(hdr), 1, fp) == 1 &&
              fwrite(&n, sizeof(n), 1, fp) == 1 && fwrite(&s, sizeof(s), 1, fp) == 1 &&
              fwrite(st.data(), sizeof(int64_t), (size_t)(n * h->W), fp) == (size_t)(n * h->W) &&
              fwrite(po.data(), sizeof(int64_t), (size_t)(n * h->R), fp) == (size_t)(n * h->R) &&
              fwrite(da.data(), sizeof(double), (size_t)n, fp) == (size_t)n;
    ok = (fclose(fp) == 0) && ok;
    return ok ? HGPU_OK : HGPU_ERR_INVALID;
}

int32_t hgpu_restore(hgpu_handle *h, const char *path) {
    if (!h || !path) return HGPU_ERR_INVALID;
    FILE *fp = fopen(path, "rb");
    if (!fp) return HGPU_ERR_INVALID;
    char magic[8];
    int32_t hdr[4];
    int64_t n = -1;
    hgpu_state s;
    bool ok = fread(magic, 1, 8, fp) == 8 && memcmp(magic, kMagic, 8) == 0 && fread(hdr, sizeof(hdr), 1, fp) == 1 &&
              hdr[0] == 1 && hdr[1] == h->W && hdr[2] == h->R && fread(&n, sizeof(n), 1, fp) == 1 && n >= 0 &&
              n <= h->b.cap && fread(&s, sizeof(s), 1, fp) == 1;
    std::vector<int64_t> st, po;
    std::vector<double> da;
    if (ok) {
        st.resize((size_t)(n * h->W + 1));
        po.resize((size_t)(n * h->R + 1));
        da.resize((size_t)(n + 1));
        ok = fread(st.data(), sizeof(int64_t), (size_t)(n * h->W), fp) == (size_t)(n * h->W) &&
             fread(po.data(), sizeof(int64_t), (size_t)(n * h->R), fp) == (size_t)(n * h->R) &&
             fread(da.data(), sizeof(double), (size_t)n, fp) == (size_t)n;
        // nothing may follow
        char extra;
        ok = ok && fread(&extra, 1, 1, fp) == 0;
    }
    fclose(fp);
    if (!ok) return HGPU_ERR_INVALID;
    int rc = set_list(h, st.data(), po.data(), da.data(), n, false);
    if (rc) return rc;
    return hgpu_set_state(h, &s);
}

static int ensure_scratch(hgpu_handle *h, size_t bytes) {
    if (h->scratch_bytes >= bytes) return HGPU_OK;
    if (h->scratch) cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
    CK(cudaMalloc(&h->scratch, bytes));
    h->scratch_bytes = bytes;
    return HGPU_OK;
}

int32_t hgpu_eval_excitations(hgpu_handle *h, const int64_t *parents, const int64_t *parent_pops, int64_t n,
                              int64_t iteration, int32_t *orbs, double *pgen, double *hmatel, int32_t *allowed,
                              int64_t *nspawn) {
    if (!h || n < 0 || (n > 0 && (!parents || !parent_pops || !orbs || !pgen || !hmatel || !allowed || !nspawn)))
        return HGPU_ERR_INVALID;
    if (n == 0) return HGPU_OK;
    size_t off_par = 0, off_pp = off_par + sizeof(int64_t) * h->W * n, off_or = off_pp + sizeof(int64_t) * n;
    size_t off_pg = off_or + sizeof(int32_t) * 4 * n, off_hm = off_pg + sizeof(double) * n;
    size_t off_al = off_hm + sizeof(double) * n, off_ns = off_al + sizeof(int32_t) * n + 8;
    off_ns = (off_ns + 7) & ~(size_t)7;
    size_t total = off_ns + sizeof(int64_t) * n;
    int rc = ensure_scratch(h, total);
    if (rc) return rc;
    char *base = static_cast<char *>(h->scratch);
    CK(cudaMemcpyAsync(base + off_par, parents, sizeof(int64_t) * h->W * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(base + off_pp, parent_pops, sizeof(int64_t) * n, cudaMemcpyHostToDevice, h->stream));
    launch_eval_excitations(h->b, h->W, h->gkind, h->cfg.precision, (const uint64_t *)(base + off_par),
                            (const int64_t *)(base + off_pp), n, iteration, (int32_t *)(base + off_or),
                            (double *)(base + off_pg), (double *)(base + off_hm), (int32_t *)(base + off_al),
                            (int64_t *)(base + off_ns), h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(orbs, base + off_or, sizeof(int32_t) * 4 * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(pgen, base + off_pg, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hmatel, base + off_hm, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(allowed, base + off_al, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(nspawn, base + off_ns, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HGPU_OK;
}

int32_t hgpu_annihilate_fixed(hgpu_handle *h, const int64_t *sdata, int64_t n, int64_t iteration) {
    if (!h || n < 0 || (n > 0 && !sdata)) return HGPU_ERR_INVALID;
    if (n > h->b.scap) return HGPU_ERR_SPAWN_OVERFLOW;
    int el = h->W + h->R + 1;
    int rc = ensure_scratch(h, sizeof(int64_t) * el * (n > 0 ? n : 1));
    if (rc) return rc;
    if (n > 0) CK(cudaMemcpyAsync(h->scratch, sdata, sizeof(int64_t) * el * n, cudaMemcpyHostToDevice, h->stream));
    DevState st;
    if ((rc = read_state(h, &st))) return rc;
    int64_t save = st.iter;
    st.iter = iteration;
    st.error_flags = 0;
    if ((rc = write_state(h, &st))) return rc;
    launch_load_fixed_spawns(h->b, h->W, h->R, (const int64_t *)h->scratch, n, h->stream);
    launch_annihilation(h->b, h->W, h->R, h->kind, h->cur, h->stream);
    CK(cudaGetLastError());
    h->cur = 1 - h->cur;
    if ((rc = read_state(h, &st))) return rc;
    st.iter = save;
    int flags = st.error_flags;
    if ((rc = write_state(h, &st))) return rc;
    return (flags & HGPU_FLAG_MAIN_OVERFLOW) ? HGPU_ERR_MAIN_OVERFLOW : HGPU_OK;
}

int32_t hgpu_snapshot(hgpu_handle *h, int32_t restore) {
    if (!h) return HGPU_ERR_INVALID;
    int W = h->W, R = h->R, rc;
    DevState st;
    if ((rc = read_state(h, &st))) return rc;
    if (!restore) {
        if (!h->snap_dets) {
            if ((rc = dalloc(h, &h->snap_dets, (size_t)h->b.cap * W))) return rc;
            if ((rc = dalloc(h, &h->snap_pops, (size_t)h->b.cap * R))) return rc;
            if ((rc = dalloc(h, &h->snap_kii, (size_t)h->b.cap))) return rc;
        }
        int64_t n = st.n_main;
        CK(cudaMemcpyAsync(h->snap_dets, h->b.dets[h->cur], sizeof(uint64_t) * W * n, cudaMemcpyDeviceToDevice,
                           h->stream));
        CK(cudaMemcpyAsync(h->snap_pops, h->b.pops[h->cur], sizeof(int64_t) * R * n, cudaMemcpyDeviceToDevice,
                           h->stream));
        CK(cudaMemcpyAsync(h->snap_kii, h->b.kii[h->cur], sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        h->snap_n = n;
        for (int s = 0; s < HGPU_MAX_SPACES; s++) h->snap_abs[s] = st.abs_pop[s];
        h->snap_ss_gen = h->ss_gen;
        return HGPU_OK;
    }
    if (!h->snap_dets) return HGPU_ERR_INVALID;
    // a list saved under another deterministic space (or none) does not hold
    // the current space's states: the space is built again from it
    if (h->snap_ss_gen != h->ss_gen) ss_reschedule(h);
    int64_t n = h->snap_n;
    CK(cudaMemcpyAsync(h->b.dets[h->cur], h->snap_dets, sizeof(uint64_t) * W * n, cudaMemcpyDeviceToDevice,
                       h->stream));
    CK(cudaMemcpyAsync(h->b.pops[h->cur], h->snap_pops, sizeof(int64_t) * R * n, cudaMemcpyDeviceToDevice,
                       h->stream));
    CK(cudaMemcpyAsync(h->b.kii[h->cur], h->snap_kii, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    st.n_main = n;
    for (int s = 0; s < HGPU_MAX_SPACES; s++) st.abs_pop[s] = h->snap_abs[s];
    return write_state(h, &st);
}

int32_t hgpu_profile_cycle(hgpu_handle *h, double *phase_ms, int32_t nphase, int64_t *counts) {
    if (!h || !phase_ms || nphase < 1) return HGPU_ERR_INVALID;
    PhaseMarks pm;
    for (int k = 0; k < kNumMarks; k++) CK(cudaEventCreate(&pm.ev[k]));
    DevState before;
    int rc = read_state(h, &before);
    if (rc) return rc;
    launch_cycle(h->b, h->W, h->R, h->gkind, h->cfg.precision, h->cur, h->stream, &pm);
    CK(cudaGetLastError());
    h->cur = 1 - h->cur;
    h->iter += 1;
    CK(cudaEventSynchronize(pm.ev[kNumMarks - 1]));
    for (int k = 0; k < nphase && k < kNumMarks - 1; k++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pm.ev[k], pm.ev[k + 1]);
        phase_ms[k] = ms;
    }
    for (int k = 0; k < kNumMarks; k++) cudaEventDestroy(pm.ev[k]);
    DevState st;
    if ((rc = read_state(h, &st))) return rc;
    if (counts) {
        // N before, A, S, U, N after, launches in the cycle
        counts[0] = before.n_main;
        counts[1] = st.n_attempts;
        counts[2] = st.n_spawn;
        counts[3] = st.n_uniq;
        counts[4] = st.n_main;
        counts[5] = launches_per_cycle(h->b);
        counts[6] = h->b.sort_passes;
        // bytes the radix passes read and write per spawned entry, all passes:
        // packed records (16 bytes while the key and the index need two words,
        // then 8, the last pass writing the 4-byte index) or key and index
        const DevBuffers &b = h->b;
        int64_t moved = 0;
        for (int p = 0; p < b.sort_passes; p++) {
            if (b.sort_packed) {
                const int in = b.sort_key_bits - kRadixBits * p + b.sort_ibits > 64 ? 16 : 8;
                const bool last = p == b.sort_passes - 1;
                const int out = last ? 4 : (b.sort_key_bits - kRadixBits * (p + 1) + b.sort_ibits > 64 ? 16 : 8);
                moved += in + out;
            } else {
                moved += 2 * ((b.key32 ? 4 : 8 * b.key_words) + 4);
            }
        }
        counts[7] = moved;
    }
    return HGPU_OK;
}

int32_t hgpu_eval_diagonal(hgpu_handle *h, const int64_t *dets, int64_t n, double *kii) {
    if (!h || n < 0 || (n > 0 && (!dets || !kii))) return HGPU_ERR_INVALID;
    if (n == 0) return HGPU_OK;
    size_t bytes = sizeof(int64_t) * h->W * n + sizeof(double) * n;
    int rc = ensure_scratch(h, bytes);
    if (rc) return rc;
    char *base = static_cast<char *>(h->scratch);
    CK(cudaMemcpyAsync(base, dets, sizeof(int64_t) * h->W * n, cudaMemcpyHostToDevice, h->stream));
    double *dk = (double *)(base + sizeof(int64_t) * h->W * n);
    launch_eval_diagonal(h->b, h->W, (const uint64_t *)base, n, dk, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(kii, dk, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HGPU_OK;
}

}  // extern "C"
