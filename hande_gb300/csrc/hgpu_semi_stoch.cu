// hgpu_semi_stoch.cu -- semi-stochastic projection (src/semi_stoch.F90,
// separate annihilation): the deterministic Hamiltonian, built once per
// space by column, and each cycle's exact projection of the deterministic
// amplitudes, stochastically rounded and added to the main list.
#include "hgpu_common.cuh"

namespace hgpu {

// create_determ_hamil (src/semi_stoch.F90:533-685) by column: one warp per
// column j walks the rows i in ascending order, 32 at a time, and keeps
// H(D_i, D_j) (get_hmatel with D_i as the bra; on the diagonal the exact
// K_jj of the main list) when |H| > depsilon.  FILL = false counts the
// entries of each column; FILL = true writes them at dcol_ptr[j].
template <int W, bool FILL>
__global__ void __launch_bounds__(kBlock) k_determ_columns(DevBuffers b, int64_t *counts, int32_t *col_i,
                                                           double *col_h) {
    __shared__ DevSys s;
    extern __shared__ uint8_t smem[];
    stage_sys(s, b.sys);
    HubTables t = stage_hub(b.sys, smem);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (kBlock / 32);
    const int64_t nd = b.nd;
    for (int64_t j = (int64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); j < nd; j += nwarps) {
        const Det<W> dj = load_det<W>(b.ddets, j);
        const double kjj = kii_of<W>(s, dj);
        int64_t pos = FILL ? b.dcol_ptr[j] : 0;
        for (int64_t i0 = 0; i0 < nd; i0 += 32) {
            const int64_t i = i0 + lane;
            double h = 0.0;
            if (i < nd) {
                if (i == j) {
                    h = kjj;
                } else {
                    const Det<W> di = load_det<W>(b.ddets, i);
                    const Excit e = get_excitation<W>(di, dj, s.nel);
                    if (e.nexcit == 1 || e.nexcit == 2) h = proj_hmatel<W>(s, t, di, e);
                }
            }
            const bool keep = i < nd && fabs(h) > 1.0e-12;
            const uint32_t m = __ballot_sync(FULL_MASK, keep);
            if (FILL && keep) {
                const int64_t q = pos + __popc(m & lanemask_lt());
                col_i[q] = (int32_t)i;
                col_h[q] = h;
            }
            pos += __popc(m);
        }
        if (!FILL && lane == 0) counts[j] = pos;
    }
}

// determ_proj_separate_annihil (src/semi_stoch.F90:1009-1094) without
// quasi-Newton (rho_minus_qn_weight = 0, quasi_newton_pop_control = 1):
// y_j = (tau S) v_j, then y_j += (-tau H_ij) v_i over the rows of column j in
// ascending order (csrpgemv with the transpose, lib/local/csr.f90:148-204);
// deterministic_annihilation (src/annihilation.f90:488-535): y in walker units,
// rounded up with probability of its fraction, added to the main list.
__global__ void __launch_bounds__(kBlock) k_determ_project(DevBuffers b, int R, int cur) {
    const DevSys *s = b.sys;
    DevState *st = b.state;
    const uint64_t iter = (uint64_t)st->iter;
    const double tau = s->tau, rf = (double)s->real_factor;
    const double a = -1.0 * tau;
    int64_t *pops = b.pops[cur];
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < b.nd; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t z0 = b.dcol_ptr[j], z1 = b.dcol_ptr[j + 1];
        const int64_t ind = b.dind[j];
        if (ind < 0 || ind >= st->n_main) {  // every deterministic state stays in the main list
            atomicOr(&st->error_flags, HGPU_FLAG_INTERNAL);
            continue;
        }
        for (int sp = 0; sp < R; sp++) {
            const double scale = -tau * (0.0 - st->shift[sp] * 1.0);
            double y = scale * b.dvec[j * R + sp];
            for (int64_t z = z0; z < z1; z++) y = y + a * b.dcol_h[z] * b.dvec[(int64_t)b.dcol_i[z] * R + sp];
            double amp = y * rf;
            const int64_t sign = amp < 0.0 ? -1 : 1;
            amp = fabs(amp);
            int64_t n = (int64_t)amp;
            amp = amp - (double)n;
            RStream rs;
            rs.init(s->seed, P_DETERM, sp, j, 0, iter);
            if (amp > rs.next()) n = n + 1;
            pops[ind * R + sp] += sign * n;
        }
    }
}

void launch_determ_columns(const DevBuffers &b, int W, int kind, bool fill, int64_t *counts, int32_t *col_i,
                           double *col_h, cudaStream_t st) {
    // the momentum tables of a Hubbard system in shared memory (stage_hub)
    const size_t sm = kind == HGPU_SYS_HUB_K ? (size_t)(b.nk * b.nk + b.nk + 16) : 16;
    int64_t blocks = (b.nd + (kBlock / 32) - 1) / (kBlock / 32);
    const int grid = (int)(blocks < 1 ? 1 : (blocks > b.grid ? b.grid : blocks));
    const void *fn = W == 1 ? (fill ? (const void *)k_determ_columns<1, true> : (const void *)k_determ_columns<1, false>)
                            : (fill ? (const void *)k_determ_columns<2, true> : (const void *)k_determ_columns<2, false>);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (W == 1) {
        if (fill) k_determ_columns<1, true><<<grid, kBlock, sm, st>>>(b, counts, col_i, col_h);
        else k_determ_columns<1, false><<<grid, kBlock, sm, st>>>(b, counts, col_i, col_h);
    } else {
        if (fill) k_determ_columns<2, true><<<grid, kBlock, sm, st>>>(b, counts, col_i, col_h);
        else k_determ_columns<2, false><<<grid, kBlock, sm, st>>>(b, counts, col_i, col_h);
    }
}

// The spawned entries of the deterministic space come after every spawning
// attempt's: their count marks where they start in the spawned list.
__global__ void k_mark_stoch_spawns(DevState *st) { st->n_spawn_stoch = st->n_spawn; }

// determ_proj_combined_annihil (src/semi_stoch.F90:897-975) without
// quasi-Newton (rho_minus_qn_weight = 0, quasi_newton_pop_control = 1), one
// thread per deterministic state r: for each space, out = sum_j H(r, j) v_j
// over row r in ascending column order (csrpgemv_single_row,
// lib/local/csr.f90:206-235; row r of the symmetric matrix is the stored
// column r), then out = -tau (out + (-S) v_r); create_spawned_particle_determ
// (:1096-1146): out in walker units, rounded up with probability of its
// fraction (the same stream as the separate projection's), appended to the
// spawned list as a spawn from an initiator, generation order after every
// spawning attempt (row-major over (state, space)).
__global__ void __launch_bounds__(kBlock) k_determ_spawn(DevBuffers b, int R) {
    const DevSys *s = b.sys;
    DevState *st = b.state;
    const uint64_t iter = (uint64_t)st->iter;
    const double tau = s->tau, rf = (double)s->real_factor;
    const int W = s->nw;
    const uint64_t abase = (uint64_t)st->n_attempts;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < b.nd; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t z0 = b.dcol_ptr[r], z1 = b.dcol_ptr[r + 1];
        for (int sp = 0; sp < R; sp++) {
            double out = 0.0;
            for (int64_t z = z0; z < z1; z++) out = out + b.dcol_h[z] * b.dvec[(int64_t)b.dcol_i[z] * R + sp];
            const double coef = 0.0 * 0.0 - 1.0 * st->shift[sp];
            out = -tau * (out + coef * b.dvec[r * R + sp]);
            const double scaled = out * rf;
            const int64_t sign = scaled < 0.0 ? -1 : 1;
            const double amp = fabs(scaled);
            int64_t n = (int64_t)amp;
            RStream rs;
            rs.init(s->seed, P_DETERM, sp, r, 0, iter);
            if (amp - (double)n > rs.next()) n = n + 1;
            n = n * sign;
            const unsigned long long pos = atomicAdd((unsigned long long *)&st->n_spawn, 1ull);
            if ((int64_t)pos >= b.scap) {
                atomicOr(&st->error_flags, HGPU_FLAG_SPAWN_OVERFLOW);
                continue;
            }
            for (int w = 0; w < W; w++) b.sdets[pos * W + w] = b.ddets[r * W + w];
            for (int q = 0; q < R; q++) b.spops[pos * R + q] = q == sp ? n : 0;
            if (b.sflag) b.sflag[pos] = (abase + (uint64_t)r * R + sp) << 2;
        }
    }
}

void launch_determ_project(const DevBuffers &b, int R, int cur, cudaStream_t st) {
    int64_t blocks = (b.nd + kBlock - 1) / kBlock;
    const int grid = (int)(blocks < 1 ? 1 : (blocks > b.grid ? b.grid : blocks));
    if (b.ss_combined) {
        k_mark_stoch_spawns<<<1, 1, 0, st>>>(b.state);
        k_determ_spawn<<<grid, kBlock, 0, st>>>(b, R);
    } else {
        k_determ_project<<<grid, kBlock, 0, st>>>(b, R, cur);
    }
}

}  // namespace hgpu
