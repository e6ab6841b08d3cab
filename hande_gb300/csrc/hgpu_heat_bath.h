// hgpu_heat_bath.h -- host construction of the heat-bath excitation generator
// tables (init_excit_mol_heat_bath, src/excit_gen_heat_bath_mol.F90:14-243).
//
// Weights of Holmes, Changlani and Umrigar (JCTC 12, 1561 (2016)) as HANDE
// defines them: h_ijab = |<ij||ab>| over all spin orbitals with spin and
// symmetry conserved, S_i = sum_jab h_ijab, D_ij = sum_ab h_ijab, and per
// (i,j) and (i,j,a) Walker alias tables over a and b.  The sums run in the
// reference's serial loop order, so every weight is the same double the
// reference computes.  The nb^4 weights themselves are not kept: the device
// recomputes h_ijab (two integral lookups) where p_gen needs it, with the same
// expression; only the alias tables (U, K) of b are nb^4 in size.
//
// Layout, 0-based, i slowest (Fortran's first index fastest):
//   i_w[i], ij_w[i*nb + j] = ij_weights(j,i),
//   ija_w / ija_U / ija_K [(i*nb + j)*nb + a] = hb_ija%{weights,aliasU,aliasK}(a,j,i),
//   ija_tot[i*nb + j] = hb_ija%weights_tot(j,i),
//   ijab_tot[(i*nb + j)*nb + a] = hb_ijab%weights_tot(a,j,i),
//   ijab_U / ijab_K [((i*nb + j)*nb + a)*nb + b] = hb_ijab%{aliasU,aliasK}(b,a,j,i).
// Alias tables the reference leaves unset (zero total weight) are U = 0, K = self.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/hande_gpu.h"

namespace hgpu {

struct HeatBathTables {
    int nb = 0;
    std::vector<double> i_w, ij_w, ija_w, ija_tot, ija_U, ijab_tot, ijab_U;
    std::vector<uint8_t> ija_K, ijab_K;
    bool bias = false;  // a valid single i -> a has no j (original heat bath stops here)
};

// generate_alias_tables (lib/local/alias.f90:100-184), 0-based, n <= 128.
template <typename Real>
inline void hb_alias_build(int n, const Real *w, Real tot, Real *U, uint8_t *K) {
    int under[128], over[128], nu = 0, no = 0;
    Real f = (Real)n / tot;
    for (int i = 0; i < n; i++) {
        U[i] = w[i] * f;
        if (U[i] <= (Real)1) under[nu++] = i;
        else over[no++] = i;
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
}

class HeatBathBuilder {
  public:
    HeatBathBuilder(const hgpu_system *sys) : sys_(sys), nb_(sys->nbasis) {}

    // |<ij|ab> - <ij|ba>| of init_excit_mol_heat_bath's inner loop, 0 when the
    // excitation is not allowed (src/excit_gen_heat_bath_mol.F90:131-152).
    double weight(int i, int j, int a, int b) const {
        if (i == j || a == i || a == j || b == a || b == i || b == j) return 0.0;
        int it = j < i ? j : i, jt = j < i ? i : j;
        const int32_t *sym = sys_->orb_sym, *ms = sys_->orb_ms;
        int isymb = xsym(xsym(sym[it], sym[jt]), sym[a]);
        if (!(((ms[it] == ms[a]) && (ms[jt] == ms[b])) || ((ms[it] == ms[b]) && (ms[jt] == ms[a])))) return 0.0;
        if (sym[b] != isymb) return 0.0;
        int at = b < a ? b : a, bt = b < a ? a : b;
        return std::fabs(sc2(it, jt, at, bt));
    }

    // Fills t; returns false only on allocation failure.
    bool build(HeatBathTables &t, bool original) const {
        const int nb = nb_;
        const size_t n2 = (size_t)nb * nb, n3 = n2 * nb, n4 = n3 * nb;
        t.nb = nb;
        try {
            t.i_w.assign(nb, 0.0);
            t.ij_w.assign(n2, 0.0);
            t.ija_w.assign(n3, 0.0);
            t.ija_tot.assign(n2, 0.0);
            t.ija_U.assign(n3, 0.0);
            t.ija_K.resize(n3);
            t.ijab_tot.assign(n3, 0.0);
            t.ijab_U.assign(n4, 0.0);
            t.ijab_K.resize(n4);
        } catch (...) {
            return false;
        }
        std::vector<char> bias(nb, 0);
        unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
        std::vector<std::thread> pool;
        for (unsigned w = 0; w < nt; w++) {
            pool.emplace_back([&, w]() {
                std::vector<double> row(nb);
                std::vector<int> j_nonzero(nb);
                for (int i = (int)w; i < nb; i += (int)nt) {
                    std::fill(j_nonzero.begin(), j_nonzero.end(), 0);
                    double i_weight = 0.0;
                    for (int j = 0; j < nb; j++) {
                        double ij_weight = 0.0;
                        size_t o2 = (size_t)i * nb + j;
                        if (i != j) {
                            double ija_weights_tot = 0.0, i_weight_extra = 0.0;
                            for (int a = 0; a < nb; a++) {
                                double ija_weight = 0.0, tot = 0.0;
                                size_t o3 = o2 * nb + a;
                                if (a != i && a != j) {
                                    // a disallowed (b) contributes +0.0, which leaves
                                    // every running sum unchanged, as the reference's skip does
                                    for (int b = 0; b < nb; b++) {
                                        double h = weight(i, j, a, b);
                                        i_weight_extra = i_weight_extra + h;
                                        ij_weight = ij_weight + h;
                                        ija_weight = ija_weight + h;
                                        double ijab_weight = 0.0 + h;
                                        row[b] = ijab_weight;
                                        tot = tot + ijab_weight;
                                    }
                                } else {
                                    std::fill(row.begin(), row.end(), 0.0);
                                }
                                t.ijab_tot[o3] = tot;
                                uint8_t *K = &t.ijab_K[o3 * nb];
                                double *U = &t.ijab_U[o3 * nb];
                                for (int b = 0; b < nb; b++) K[b] = (uint8_t)b;
                                if (std::fabs(tot) > 0.0) hb_alias_build<double>(nb, row.data(), tot, U, K);
                                t.ija_w[o3] = ija_weight;
                                ija_weights_tot = ija_weights_tot + ija_weight;
                                if (ija_weight > 1.0e-12) j_nonzero[a]++;
                            }
                            i_weight = i_weight + i_weight_extra;
                            t.ija_tot[o2] = 0.0 + ija_weights_tot;
                        } else {
                            for (int a = 0; a < nb; a++) {
                                size_t o3 = o2 * nb + a;
                                for (int b = 0; b < nb; b++) t.ijab_K[o3 * nb + b] = (uint8_t)b;
                            }
                        }
                        t.ij_w[o2] = ij_weight;
                        uint8_t *K = &t.ija_K[o2 * nb];
                        for (int a = 0; a < nb; a++) K[a] = (uint8_t)a;
                        if (std::fabs(t.ija_tot[o2]) > 0.0)
                            hb_alias_build<double>(nb, &t.ija_w[o2 * nb], t.ija_tot[o2], &t.ija_U[o2 * nb], K);
                    }
                    t.i_w[i] = i_weight;
                    for (int a = 0; a < nb && original; a++) {
                        if (j_nonzero[a] < nb - sys_->nel && i != a && sys_->orb_sym[a] == sys_->orb_sym[i] &&
                            sys_->orb_ms[a] == sys_->orb_ms[i])
                            bias[i] = 1;
                    }
                }
            });
        }
        for (auto &th : pool) th.join();
        t.bias = std::any_of(bias.begin(), bias.end(), [](char c) { return c != 0; });
        return true;
    }

    // init_excit_mol_power_pitzer_orderM_ij (src/excit_gen_power_pitzer_mol.F90:574-648)
    // with init_double_weights_ab (src/excit_gen_utils.f90:68-138): ij_w[i*nb + j]
    // is the sum of |<ij||ab>| over the allowed ordered (a, b), a-major, and
    // i_w[i] the sum of row i in j order; one thread per i.
    void pair_weights(std::vector<double> &i_w, std::vector<double> &ij_w) const {
        const int nb = nb_;
        i_w.assign(nb, 0.0);
        ij_w.assign((size_t)nb * nb, 0.0);
        unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
        std::vector<std::thread> pool;
        for (unsigned w = 0; w < nt; w++) {
            pool.emplace_back([&, w]() {
                for (int i = (int)w; i < nb; i += (int)nt) {
                    double iw = 0.0;
                    for (int j = 0; j < nb; j++) {
                        double s = 0.0;
                        if (i != j)
                            for (int a = 0; a < nb; a++)
                                for (int b = 0; b < nb; b++) s = s + weight(i, j, a, b);
                        ij_w[(size_t)i * nb + j] = s;
                        iw = iw + s;
                    }
                    i_w[i] = iw;
                }
            });
        }
        for (auto &th : pool) th.join();
    }

    // find_parallel_spin_prob_mol (src/qmc_common.F90:265-378): the share of
    // sum |<ij||ab>| over allowed (i, j, a, b) carried by parallel-spin pairs.
    // The sums run over j, a, b for each i (one thread per i) and the per-i
    // sums are added in i order, as the CPU restatement does.
    double parallel_spin_prob() const {
        const int nb = nb_;
        std::vector<double> par(nb, 0.0), orth(nb, 0.0);
        unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
        std::vector<std::thread> pool;
        for (unsigned w = 0; w < nt; w++) {
            pool.emplace_back([&, w]() {
                for (int i = (int)w; i < nb; i += (int)nt) {
                    double pi = 0.0, oi = 0.0;
                    for (int j = 0; j < nb; j++) {
                        if (i == j) continue;
                        const bool parallel = sys_->orb_ms[i] == sys_->orb_ms[j];
                        for (int a = 0; a < nb; a++)
                            for (int b = 0; b < nb; b++) {
                                double h = weight(i, j, a, b);
                                if (h == 0.0) continue;
                                if (parallel) pi = pi + h;
                                else oi = oi + h;
                            }
                    }
                    par[i] = pi;
                    orth[i] = oi;
                }
            });
        }
        for (auto &t : pool) t.join();
        double p = 0.0, o = 0.0;
        for (int i = 0; i < nb; i++) {
            p = p + par[i];
            o = o + orth[i];
        }
        return p / (p + o);
    }

  private:
    static int xsym(int a, int b) { return a ^ b; }

    // (pq|rs) over spatial orbitals, 8-fold packed (two_body_int_indx,
    // src/molecular_integrals.F90:736-845).
    double v2(int i, int j, int a, int b) const {
        auto tri0 = [](int64_t x, int64_t y) { return x * (x + 1) / 2 + y; };
        int si = i >> 1, sj = j >> 1, sa = a >> 1, sb = b >> 1;
        int64_t ia = si >= sa ? tri0(si, sa) : tri0(sa, si);
        int64_t jb = sj >= sb ? tri0(sj, sb) : tri0(sb, sj);
        return sys_->v2[ia >= jb ? tri0(ia, jb) : tri0(jb, ia)];
    }

    // slater_condon2_mol_excit (src/hamiltonian_molecular.f90:300-346), perm = false.
    double sc2(int i, int j, int a, int b) const {
        const int32_t *ms = sys_->orb_ms;
        double h = 0.0;
        if (ms[i] == ms[a]) h = v2(i, j, a, b);
        if (ms[i] == ms[b]) h = h - v2(i, j, b, a);
        return h;
    }

    const hgpu_system *sys_;
    int nb_;
};

}  // namespace hgpu
