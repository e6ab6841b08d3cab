// hgpu_power_pitzer.h -- host construction of the tables of the
// heat_bath_power_pitzer_ref generator (init_excit_mol_power_pitzer_orderN,
// src/excit_gen_power_pitzer_mol.F90:215-572), in the reference's arithmetic
// order so that every weight, total and alias entry is the reference's value.
//
// Six tables, each a set of rows of `stride` entries: w (weights), U and K
// (alias table), tot (row totals):
//   PPN_IS  i of a single excitation, one row over the reference's occupied list
//   PPN_ID  i of a double excitation, one row over the reference's occupied list
//   PPN_IJD j given the orbital i, rows [nbasis] over the reference's occupied list
//   PPN_IAS a of a single from orbital i, rows [nbasis] over i's (spin, irrep) list
//   PPN_IAD a of a double from orbital i, rows [nbasis] over all orbitals of i's spin
//   PPN_JBD b of a double from orbital j, rows [nbasis * nsym] over each (spin, irrep) list
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/hande_gpu.h"
#include "hgpu_heat_bath.h"  // hb_alias_build

namespace hgpu {

enum { PPN_IS = 0, PPN_ID = 1, PPN_IJD = 2, PPN_IAS = 3, PPN_IAD = 4, PPN_JBD = 5, PPN_NTAB = 6 };

struct PPNTables {
    std::vector<double> w[PPN_NTAB], U[PPN_NTAB], tot[PPN_NTAB];
    std::vector<uint8_t> K[PPN_NTAB];
    int stride[PPN_NTAB] = {0, 0, 0, 0, 0, 0};
};

class PowerPitzerRefBuilder {
  public:
    PowerPitzerRefBuilder(const hgpu_system *sys, const uint64_t *ref, double min_ratio)
        : sys_(sys), nb_(sys->nbasis), nsym_(sys->nsym_pg), maxss_(sys->max_sym_spin), min_ratio_(min_ratio) {
        for (int p = 0; p < nb_; p++) {
            if ((ref[p >> 6] >> (p & 63)) & 1u) occ_.push_back(p);
            else virt_.push_back(p);
        }
    }

    void build(PPNTables &t) const {
        const int nel = (int)occ_.size(), half = nb_ / 2;
        alloc(t, PPN_IS, 1, nel);
        alloc(t, PPN_ID, 1, nel);
        alloc(t, PPN_IJD, nb_, nel);
        alloc(t, PPN_IAS, nb_, maxss_);
        alloc(t, PPN_IAD, nb_, half);
        alloc(t, PPN_JBD, nb_ * nsym_, maxss_);
        // i of a single: summed single weights over a of i's spin and irrep
        parallel_for(nel, [&](int i) {
            const int oi = occ_[i];
            double w = 0.0;
            for (int a = 0; a < nb_; a++)
                if (a != oi && sys_->orb_sym[a] == sys_->orb_sym[oi] && sys_->orb_ms[a] == sys_->orb_ms[oi])
                    w = w + single_weight(oi, a);
            if (w < 1.0e-12) w = 10.0 * 1.0e-12;
            t.w[PPN_IS][i] = w;
        });
        for (int i = 0; i < nel; i++) t.tot[PPN_IS][0] = t.tot[PPN_IS][0] + t.w[PPN_IS][i];
        finish(t, PPN_IS, 0, nel, true);
        // a of a single from any orbital i
        parallel_for(nb_, [&](int i) {
            const int ims = ims_of(i), sym = sys_->orb_sym[i], na = nbss(ims, sym);
            double tot = 0.0;
            for (int a = 0; a < na; a++) {
                double w = 0.0;
                const int q = ssbf(ims, sym, a);
                if (q != i) {
                    w = single_weight(i, q);
                    if (w < 1.0e-12) w = 10.0 * 1.0e-12;
                }
                t.w[PPN_IAS][(size_t)i * t.stride[PPN_IAS] + a] = w;
                tot = tot + w;
            }
            t.tot[PPN_IAS][i] = tot;
            finish(t, PPN_IAS, i, na, true);
        });
        // i of a double: one accumulator over j and then a, b
        parallel_for(nel, [&](int i) {
            double w = 0.0;
            for (int j = 0; j < nel; j++)
                if (i != j) w = double_weights_ab(occ_[i], occ_[j], w);
            if (w < 1.0e-12) w = 10.0 * 1.0e-12;
            t.w[PPN_ID][i] = w;
        });
        for (int i = 0; i < nel; i++) t.tot[PPN_ID][0] = t.tot[PPN_ID][0] + t.w[PPN_ID][i];
        finish(t, PPN_ID, 0, nel, true);
        // j (a position in the reference's list) given any orbital i
        parallel_for(nb_, [&](int i) {
            double tot = 0.0;
            for (int j = 0; j < nel; j++) {
                double w = 0.0;
                if (occ_[j] != i) w = double_weights_ab(i, occ_[j], 0.0);
                if (w < 1.0e-12) w = 10.0 * 1.0e-12;
                t.w[PPN_IJD][(size_t)i * t.stride[PPN_IJD] + j] = w;
                tot = tot + w;
            }
            t.tot[PPN_IJD][i] = tot;
            finish(t, PPN_IJD, i, nel, true);
        });
        // a of a double over all orbitals of i's spin, b per irrep (i itself weighted 0)
        parallel_for(nb_, [&](int i) {
            const int ims = ims_of(i);
            std::vector<int> list;
            for (int k = 0; k < half; k++) list.push_back(2 * k + (ims == 0 ? 1 : 0));
            t.tot[PPN_IAD][i] = weight_list(i, list, &t.w[PPN_IAD][(size_t)i * t.stride[PPN_IAD]]);
            finish(t, PPN_IAD, i, half, false);
            for (int bsym = 0; bsym < nsym_; bsym++) {
                const int n = nbss(ims, bsym), r = i * nsym_ + bsym;
                if (n <= 0) continue;
                list.clear();
                for (int q = 0; q < n; q++) list.push_back(ssbf(ims, bsym, q));
                t.tot[PPN_JBD][r] = weight_list(i, list, &t.w[PPN_JBD][(size_t)r * t.stride[PPN_JBD]]);
                finish(t, PPN_JBD, r, n, false);
            }
        });
    }

  private:
    const hgpu_system *sys_;
    int nb_, nsym_, maxss_;
    double min_ratio_;
    std::vector<int> occ_, virt_;

    template <typename F>
    static void parallel_for(int n, F fn) {
        unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
        std::vector<std::thread> pool;
        for (unsigned w = 0; w < nt; w++)
            pool.emplace_back([&, w]() {
                for (int i = (int)w; i < n; i += (int)nt) fn(i);
            });
        for (auto &th : pool) th.join();
    }

    static void alloc(PPNTables &t, int k, int rows, int stride) {
        if (stride < 1) stride = 1;
        t.stride[k] = stride;
        t.w[k].assign((size_t)rows * stride, 0.0);
        t.U[k].assign((size_t)rows * stride, 0.0);
        t.K[k].resize((size_t)rows * stride);
        for (size_t q = 0; q < t.K[k].size(); q++) t.K[k][q] = (uint8_t)(q % stride);
        t.tot[k].assign(rows, 0.0);
    }

    // check_min_weight_ratio (src/excit_gen_power_pitzer_mol.F90:140-213)
    static void min_weight_ratio(double *w, double &tot, int n, double min_ratio) {
        double min_weight_tmp = 0.0, min_weight;
        int nz = 0;
        if (!(tot > 0.0 && min_ratio > 0.0)) return;
        for (int i = 0; i < n; i++)
            if (w[i] > 0.0) nz++;
        min_weight = (min_ratio / (double)nz) * tot;
        for (int it = 0; it < 100000 && std::fabs(min_weight_tmp - min_weight) > 1.0e-12; it++) {
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
        double s = 0.0;
        for (int j = 0; j < n; j++) {
            if (w[j] > 0.0 && w[j] < min_weight) w[j] = min_weight;
            s = s + w[j];
        }
        tot = s;
    }

    void finish(PPNTables &t, int k, int r, int n, bool floor) const {
        double *w = &t.w[k][(size_t)r * t.stride[k]];
        if (floor) min_weight_ratio(w, t.tot[k][r], n, min_ratio_);
        hb_alias_build<double>(n, w, t.tot[k][r], &t.U[k][(size_t)r * t.stride[k]], &t.K[k][(size_t)r * t.stride[k]]);
    }

    int ims_of(int p) const { return (sys_->orb_ms[p] + 1) / 2; }  // 0 beta, 1 alpha
    int nbss(int ims, int sym) const { return sys_->nbasis_sym_spin[ims * nsym_ + sym]; }
    int ssbf(int ims, int sym, int k) const { return sys_->sym_spin_basis_fns[(sym * 2 + ims) * maxss_ + k]; }

    // <ij|ab> = (ia|jb) over spatial orbitals, 8-fold packed
    double v2(int i, int j, int a, int b) const {
        auto tri0 = [](int64_t x, int64_t y) { return x >= y ? x * (x + 1) / 2 + y : y * (y + 1) / 2 + x; };
        return sys_->v2[tri0(tri0(i >> 1, a >> 1), tri0(j >> 1, b >> 1))];
    }

    // slater_condon2_mol_excit (src/hamiltonian_molecular.f90:300-346), perm = false
    double sc2(int i, int j, int a, int b) const {
        const int32_t *ms = sys_->orb_ms;
        double h = 0.0;
        if (ms[i] == ms[a]) h = v2(i, j, a, b);
        if (ms[i] == ms[b]) h = h - v2(i, j, b, a);
        return h;
    }

    // single_excitation_weight_mol (src/hamiltonian_molecular.f90:444-523)
    double single_weight(int i, int a) const {
        const int32_t *ms = sys_->orb_ms;
        int n_jb = 0;
        double weight = 0.0;
        for (int j : occ_)
            for (int b : virt_) {
                n_jb++;
                const double t1 = (ms[i] == ms[j] && ms[j] == ms[a]) ? v2(i, j, j, a) : 0.0;
                const double t2 = ms[i] == ms[a] ? v2(i, j, a, j) : 0.0;
                const double t3 = ms[i] == ms[a] ? v2(i, b, a, b) : 0.0;
                const double t4 = (ms[i] == ms[b] && ms[b] == ms[a]) ? v2(i, b, b, a) : 0.0;
                weight = weight + std::fabs(t1 - t2 + t3 - t4);
            }
        return weight / (double)n_jb;
    }

    // init_double_weights_ab (src/excit_gen_utils.f90:68-138), added to w
    double double_weights_ab(int i, int j, double w) const {
        const int32_t *sym = sys_->orb_sym, *ms = sys_->orb_ms;
        const int it = i < j ? i : j, jt = i < j ? j : i;
        const int ij_sym = sym[it] ^ sym[jt];
        for (int a = 0; a < nb_; a++) {
            if (a == it || a == jt) continue;
            const int isymb = ij_sym ^ sym[a];
            for (int b = 0; b < nb_; b++) {
                const bool spin = (ms[it] == ms[a] && ms[jt] == ms[b]) || (ms[it] == ms[b] && ms[jt] == ms[a]);
                if (spin && sym[b] == isymb && a != b && b != it && b != jt)
                    w = w + std::fabs(sc2(it, jt, b < a ? b : a, b < a ? a : b));
            }
        }
        return w;
    }

    // create_weighted_excitation_list_mol with get_two_body_int_ex_mol_real
    // (src/hamiltonian_molecular.f90:348-411): sqrt|<iq|qi>| for equal spins,
    // the entry q == i weighted 0; returns the total in list order
    double weight_list(int i, const std::vector<int> &list, double *w) const {
        double tot = 0.0;
        for (size_t k = 0; k < list.size(); k++) {
            const int q = list[k];
            if (q != i) {
                const double v = sys_->orb_ms[i] == sys_->orb_ms[q] ? v2(i, q, q, i) : 0.0;
                w[k] = std::sqrt(std::fabs(v));
                tot = tot + w[k];
            } else {
                w[k] = 0.0;
            }
        }
        return tot;
    }
};

}  // namespace hgpu
