// hgpu_kernels.cu -- the kernels of one FCIQMC Monte Carlo cycle on one GPU.
//
// One cycle (src/fciqmc.f90:293-413) is a fixed sequence of launches whose
// grids do not depend on the list sizes: every kernel reads N, S, U, A from
// DevState and loops over its share.  The sequence can therefore be captured
// once as a CUDA graph and replayed every cycle.
//
//   cycle_begin     iteration counter, nattempts = nint(2 N_w)      (qmc_common.F90:950)
//   prep_parents    E_proj / N_0 partials, decide_nattempts, initiator
//                   flags, stochastic_death in place                 (fciqmc.f90:315-373)
//   scan            attempt offsets (one flattened attempt per thread)
//   spawn           excitation generation + spawning, appended with
//                   warp-aggregated atomics                          (spawning.F90:34/215)
//   radix sort      stable LSD sort of the spawned determinants       (spawn_data.F90:406)
//   annihilation    one pass over the merge of the main list and the
//                   sorted spawned list: self-annihilation incl. the
//                   initiator flag rule, annihilate_main_list, both
//                   roundings and insert_new_walkers with K_ii
//                   (spawn_data.F90:859-1101, annihilation.f90:9-901;
//                   hgpu_annihilate.cu)
//   cycle_end       per-cycle statistics, report accumulators         (qmc_common.F90:1240)
#include "hgpu_kernels.cuh"

#include <cstdio>

#include "hgpu_common.cuh"

namespace hgpu {

// ---------------------------------------------------------------------------
// Device-wide exclusive scan, three phases over a fixed grid.
// ---------------------------------------------------------------------------
template <typename T, typename Load>
__global__ void __launch_bounds__(kBlock) k_scan_reduce(Load load, const int64_t *n_ptr, T *part) {
    int64_t n = *n_ptr, begin, end;
    chunk_range(n, begin, end);
    T acc = zero_of<T>();
    for (int64_t i = begin + threadIdx.x; i < end; i += blockDim.x) acc = acc + load(i);
    T tot;
    block_exclusive_scan<T>(acc, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_scan_parts(T *part, int G, T *total) {
    // exclusive scan of G <= 1024 block sums in place
    T v = threadIdx.x < G ? part[threadIdx.x] : zero_of<T>();
    T tot;
    T ex = block_exclusive_scan<T>(v, &tot);
    if (threadIdx.x < G) part[threadIdx.x] = ex;
    if (threadIdx.x == 0 && total) *total = tot;
}

template <typename T, typename Load, typename Store>
__global__ void __launch_bounds__(kBlock) k_scan_down(Load load, Store store, const int64_t *n_ptr, const T *part) {
    int64_t n = *n_ptr, begin, end;
    chunk_range(n, begin, end);
    T running = part[blockIdx.x];
    for (int64_t base = begin; base < end; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        T v = i < end ? load(i) : zero_of<T>();
        T tot;
        T ex = block_exclusive_scan<T>(v, &tot);
        if (i < end) store(i, running + ex, v);
        running = running + tot;
    }
}

// functors
struct LoadNatt {
    const uint32_t *a;
    __device__ int64_t operator()(int64_t i) const { return (int64_t)a[i]; }
};
struct StoreInclusive {
    int64_t *out;
    __device__ void operator()(int64_t i, int64_t ex, int64_t v) const { out[i] = ex + v; }
};

// n_ptr points at an int64 count; for N*R lists a small kernel writes the product.
__global__ void k_set_count(int64_t *dst, const int64_t *a, int64_t mul, const int64_t *b) {
    *dst = *a * mul + (b ? *b : 0);
}

// ---------------------------------------------------------------------------
// Cycle kernels
// ---------------------------------------------------------------------------
__global__ void k_cycle_begin(DevState *st, const DevSys *sys) {
    st->iter += 1;
    st->n_spawn = 0;
    st->n_rdm = 0;
    st->spawn_next = 0;
    st->n_sq = 0;
    st->n_spawn_stoch = INT64_MAX;
    double np = (double)st->abs_pop[0] / (double)sys->real_factor;
    st->nattempts_cycle = llround(2.0 * np);
}

// decide_nattempts (src/qmc_common.F90:379-406).
__device__ __forceinline__ uint32_t decide_nattempts(RStream &rs, double population) {
    double ap = fabs(population);
    int64_t n = (int64_t)ap;
    double pextra = ap - (double)n;
    if (fabs(pextra) > 1.0e-12) {
        if (pextra > rs.next()) n = n + 1;
    }
    return (uint32_t)n;
}

// decide_nattempts for population = p / 2^F (the encoded population and the
// encoding's exponent), in integer arithmetic with the same result while
// |p| < 2^53: the fraction frac 2^-F is non-zero exactly when it exceeds
// 1e-12 (F <= 31), and frac 2^-F > u = k 2^-53 is frac 2^(53-F) > k.
__device__ __forceinline__ uint32_t decide_nattempts_fx(RStream &rs, int64_t p, int F, double population) {
    uint64_t ap = p < 0 ? (uint64_t)(-p) : (uint64_t)p;
    if (ap >= (1ull << 53)) return decide_nattempts(rs, population);
    uint64_t n = ap >> F, frac = ap & ((1ull << F) - 1);
    if (frac != 0 && (frac << (53 - F)) > rs.next_k()) n = n + 1;
    return (uint32_t)n;
}

// stochastic_death (src/death.f90:11-130) with weight = pop_control = 1.
__device__ __forceinline__ int64_t stochastic_death(double tau, RStream &rs, double Kii, double shift,
                                                    int64_t &population) {
    double pd = tau * (Kii - shift);
    pd = pd * fabs((double)population);
    // kill = int(pd); if (|pd - kill| > rand) kill = kill + sign(pd): the
    // truncation and the fraction's comparison in integer arithmetic
    // (hgpu_exact.h), valid while |pd| < 2^63
    uint64_t pb = dbits(pd);
    int64_t kill = round_up_frac(pb & 0x7FFFFFFFFFFFFFFFull, rs.next_k());
    if (pb >> 63) kill = -kill;
    if (population < 0) population = population + kill;
    else population = population - kill;
    return kill < 0 ? -kill : kill;
}

template <int W>
__global__ void __launch_bounds__(kBlock) k_prep_parents(DevBuffers b, int R, int cur) {
    __shared__ DevSys s;
    extern __shared__ uint8_t smem[];
    stage_sys(s, b.sys);
    HubTables t = stage_hub(b.sys, smem);
    __syncthreads();
    const DevState *st = b.state;
    int64_t n = st->n_main;
    uint64_t iter = (uint64_t)st->iter;
    double shift[2] = {st->shift[0], st->shift[1]};
    Det<W> f0;
#pragma unroll
    for (int k = 0; k < W; k++) f0.w[k] = s.f0[k];
    const uint64_t *dets = b.dets[cur];
    int64_t *pops = b.pops[cur];
    const double *kii = b.kii[cur];
    double proj[2] = {0.0, 0.0}, d0[2] = {0.0, 0.0};
    int64_t ndeath = 0;
    // 1 / real_factor is exact (real_factor is a power of two), so p * inv_rf
    // is the quotient p / real_factor without an FP64 division
    const double inv_rf = 1.0 / (double)s.real_factor;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        Det<W> f = load_det<W>(dets, i);
        Excit e = get_excitation<W>(f, f0, s.nel);
        double h = (e.nexcit == 1 || e.nexcit == 2) ? proj_hmatel<W>(s, t, f, e) : 0.0;
        double k = kii[i];
        uint32_t info = 0;
        // set_determ_info (src/semi_stoch.F90:826-857): a deterministic state
        // records its population and position, is an initiator and does not die
        int64_t dk = -1;
        if (b.nd > 0) {
            const int64_t q = lower_bound_det<W>(b.ddets, b.nd, f);
            if (q < b.nd && det_eq<W>(load_det<W>(b.ddets, q), f)) dk = q;
        }
        double rpv[2] = {0.0, 0.0};
        for (int sp = 0; sp < R; sp++) {
            int64_t p = pops[i * R + sp];
            double rp = (double)p * inv_rf;
            rpv[sp] = rp;
            // update_proj_energy
            if (e.nexcit == 0) d0[sp] += rp;
            else proj[sp] += h * rp;
            // set_parent_flag: bit set if not an initiator
            if (!s.quadrature_initiator && !(fabs(rp) > s.initiator_pop) && dk < 0) info |= 4u << sp;
            if (p < 0) info |= 1u << sp;
            RStream rs;
            rs.init(s.seed, P_NATTEMPT, sp, i, 0, iter);
            b.natt[i * R + sp] = decide_nattempts_fx(rs, p, s.real_amplitudes ? 31 : 0, rp);
            if (dk < 0) {
                rs.init(s.seed, P_DEATH, sp, i, 0, iter);
                ndeath += stochastic_death(s.tau, rs, k, shift[sp], p);
                pops[i * R + sp] = p;
            } else {
                b.dvec[dk * R + sp] = rp;
            }
        }
        // set_parent_flag with quadrature_initiator and two spaces
        // (src/ifciqmc.f90:36-45): one test of N_1^2 + N_2^2 for both
        if (s.quadrature_initiator && !(rpv[0] * rpv[0] + rpv[1] * rpv[1] > s.initiator_pop * s.initiator_pop) &&
            dk < 0)
            info |= 12u;
        if (dk >= 0) {
            info |= kDetermBit;
            b.dind[dk] = i;
        }
        b.pinfo[i] = (uint8_t)info;
    }
    double r0 = block_reduce_sum<double>(proj[0]);
    double r1 = block_reduce_sum<double>(proj[1]);
    double r2 = block_reduce_sum<double>(d0[0]);
    double r3 = block_reduce_sum<double>(d0[1]);
    int64_t r4 = block_reduce_sum<int64_t>(ndeath);
    if (threadIdx.x == 0) {
        b.part_d[blockIdx.x * 4 + 0] = r0;
        b.part_d[blockIdx.x * 4 + 1] = r1;
        b.part_d[blockIdx.x * 4 + 2] = r2;
        b.part_d[blockIdx.x * 4 + 3] = r3;
        b.part_i[blockIdx.x * 4 + 2] = r4;
    }
}

}  // namespace hgpu

#include "hgpu_spawn.cuh"

namespace hgpu {

// Neumaier-compensated accumulation.
__device__ __forceinline__ void comp_add(double &sum, double &c, double x) {
    double t = sum + x;
    if (fabs(sum) >= fabs(x)) c += (sum - t) + x;
    else c += (x - t) + sum;
    sum = t;
}

// Fixed-order (hence deterministic) tree reduction over the per-block partials.
template <typename T>
__device__ __forceinline__ T tree_sum(T v, T *buf) {
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) buf[threadIdx.x] = buf[threadIdx.x] + buf[threadIdx.x + w];
        __syncthreads();
    }
    T r = buf[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_cycle_end(DevBuffers b, int R, int G, int had_prep) {
    __shared__ double dbuf[1024];
    __shared__ int64_t ibuf[1024];
    DevState *st = b.state;
    int t = threadIdx.x;
    bool in = t < G;
    int64_t ap0 = tree_sum<int64_t>(in ? b.part_i[t * 4 + 0] : 0, ibuf);
    int64_t ap1 = tree_sum<int64_t>(in ? b.part_i[t * 4 + 1] : 0, ibuf);
    int64_t ndeath = 0;
    double proj[2] = {0, 0}, d0[2] = {0, 0};
    if (had_prep) {
        ndeath = tree_sum<int64_t>(in ? b.part_i[t * 4 + 2] : 0, ibuf);
        proj[0] = tree_sum<double>(in ? b.part_d[t * 4 + 0] : 0.0, dbuf);
        proj[1] = tree_sum<double>(in ? b.part_d[t * 4 + 1] : 0.0, dbuf);
        d0[0] = tree_sum<double>(in ? b.part_d[t * 4 + 2] : 0.0, dbuf);
        d0[1] = tree_sum<double>(in ? b.part_d[t * 4 + 3] : 0.0, dbuf);
    }
    if (t != 0) return;
    const DevSys *s = b.sys;
    uint2 tot = *reinterpret_cast<const uint2 *>(&st->n_merged_keep);
    bool overflow = (int64_t)tot.y > b.cap;
    if (overflow) st->error_flags |= HGPU_FLAG_MAIN_OVERFLOW;
    int64_t nn = overflow ? (int64_t)tot.x : (int64_t)tot.y;
    st->n_main = nn < b.cap ? nn : b.cap;
    st->abs_pop[0] = ap0;
    st->abs_pop[1] = R > 1 ? ap1 : 0;
    if (!had_prep) return;
    for (int q = 0; q < R; q++) {
        comp_add(st->acc_proj[q], st->acc_proj_c[q], proj[q]);
        comp_add(st->acc_d0[q], st->acc_d0_c[q], d0[q]);
    }
    int64_t S = st->n_spawn;
    // spawning_rate (src/qmc_common.F90:1264-1304)
    if (st->nattempts_cycle > 0)
        st->acc_rspawn += ((double)S + (double)ndeath / (double)s->real_factor) / (double)st->nattempts_cycle;
    st->acc_attempts += st->n_attempts;
    st->acc_spawned += S;
    st->last_nspawn_events = S;
    st->rep_cycles += 1;
}

__global__ void k_zero_parts(int64_t *part_i, int G) {
    for (int k = threadIdx.x; k < G * 4; k += blockDim.x) part_i[k] = 0;
}

// Kernels of the parity / utility entry points.
template <int W, int KIND, typename Real>
__global__ void __launch_bounds__(kBlock) k_eval_excitations(const DevSys *gsys, const uint64_t *parents,
                                                             const int64_t *ppops, int64_t n, uint64_t iteration,
                                                             int32_t *orbs, double *pgen, double *hmatel,
                                                             int32_t *allowed, int64_t *nspawn) {
    __shared__ DevSys s;
    extern __shared__ uint8_t smem[];
    stage_sys(s, gsys);
    HubTables t = stage_hub(gsys, smem);
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        Det<W> f = load_det<W>(parents, i);
        RStream rs;
        rs.init(s.seed, P_SPAWN, 0, i, 0, iteration);
        Attempt at;
        if (KIND == HGPU_SYS_HUB_K) {
            attempt_hub_k<W>(s, t, rs, f, ppops[i], true, at);
        } else {
            MolDet<W> d;
            mol_decode<W>(s, f, d);
            if (KIND == kKindHeatBath || KIND == kKindHeatBathUniform) attempt_heat_bath<W, Real>(s, rs, d, ppops[i], at);
            else attempt_mol<W, Real>(s, rs, d, ppops[i], at);
        }
        orbs[4 * i + 0] = at.from[0];
        orbs[4 * i + 1] = at.nexcit == 2 ? at.from[1] : -1;
        orbs[4 * i + 2] = at.to[0];
        orbs[4 * i + 3] = at.nexcit == 2 ? at.to[1] : -1;
        pgen[i] = at.pgen;
        hmatel[i] = at.hmatel;
        allowed[i] = at.allowed ? 1 : 0;
        nspawn[i] = at.nspawn;
    }
}

template <int W>
__global__ void __launch_bounds__(kBlock) k_eval_diagonal(const DevSys *gsys, const uint64_t *dets, int64_t n,
                                                          double *kii) {
    __shared__ DevSys s;
    stage_sys(s, gsys);
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        kii[i] = kii_of<W>(s, load_det<W>(dets, i));
}

template <int W>
__global__ void __launch_bounds__(kBlock) k_load_fixed(DevBuffers b, int R, const int64_t *sdata, int64_t n) {
    int el = W + R + 1;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t *e = sdata + i * el;
        for (int k = 0; k < W; k++) b.sdets[i * W + k] = (uint64_t)e[k];
        for (int q = 0; q < R; q++) b.spops[i * R + q] = e[W + q];
        if (b.sflag) b.sflag[i] = ((uint64_t)e[W + R] & 3ull) | ((uint64_t)i << 2);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        b.state->n_spawn = n;
        b.state->n_spawn_stoch = INT64_MAX;  // every entry a spawning event
    }
}

__global__ void __launch_bounds__(kBlock) k_abs_pop(DevBuffers b, int R, int cur) {
    int64_t n = b.state->n_main;
    int64_t a0 = 0, a1 = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t p0 = b.pops[cur][i * R];
        a0 += p0 < 0 ? -p0 : p0;
        if (R > 1) {
            int64_t p1 = b.pops[cur][i * R + 1];
            a1 += p1 < 0 ? -p1 : p1;
        }
    }
    int64_t r0 = block_reduce_sum<int64_t>(a0);
    int64_t r1 = block_reduce_sum<int64_t>(a1);
    if (threadIdx.x == 0) {
        atomicAdd((unsigned long long *)&b.state->abs_pop[0], (unsigned long long)r0);
        atomicAdd((unsigned long long *)&b.state->abs_pop[1], (unsigned long long)r1);
    }
}

// ---------------------------------------------------------------------------
// Host-side launch sequences
// ---------------------------------------------------------------------------
static size_t hub_smem(int kind, int nk) {
    return kind == HGPU_SYS_HUB_K ? (size_t)(nk * nk + nk + 16) : 16;
}

template <typename T, typename Load, typename Store>
static void device_scan(const DevBuffers &b, Load load, Store store, const int64_t *n_ptr, T *part, T *total,
                        cudaStream_t st) {
    k_scan_reduce<T, Load><<<b.grid, kBlock, 0, st>>>(load, n_ptr, part);
    k_scan_parts<T><<<1, 1024, 0, st>>>(part, b.grid, total);
    k_scan_down<T, Load, Store><<<b.grid, kBlock, 0, st>>>(load, store, n_ptr, part);
}


template <int W>
static void cycle_w(const DevBuffers &b, int R, int kind, int precision, int cur, cudaStream_t st,
                    const PhaseMarks *pm) {
    DevState *S = b.state;
    size_t sm = hub_smem(kind, b.nk);
    if (pm) cudaEventRecord(pm->ev[0], st);
    k_cycle_begin<<<1, 1, 0, st>>>(S, b.sys);
    k_prep_parents<W><<<b.grid, kBlock, sm, st>>>(b, R, cur);
    if (pm) cudaEventRecord(pm->ev[1], st);
    // attempt offsets over the N*R (parent, space) slots; total -> n_attempts
    k_set_count<<<1, 1, 0, st>>>(&S->n_slots, &S->n_main, R, nullptr);
    device_scan<int64_t>(b, LoadNatt{b.natt}, StoreInclusive{b.aoff}, &S->n_slots, b.scan_part, &S->n_attempts, st);
    if (pm) cudaEventRecord(pm->ev[2], st);
#define HGPU_SPAWN(KK)                                                       \
    do {                                                                     \
        if (precision == HGPU_PREC_MIXED)                                    \
            launch_spawn_kernels<W, KK, float, false>(b, R, cur, sm, st);    \
        else                                                                 \
            launch_spawn_kernels<W, KK, double, false>(b, R, cur, sm, st);   \
    } while (0)
    if (b.rdm) launch_spawn_rdm(b, W, R, kind, precision, cur, sm, st);  // hgpu_spawn_rdm.cu
    else if (kind == HGPU_SYS_HUB_K)
        launch_spawn_kernels<W, HGPU_SYS_HUB_K, double, false>(b, R, cur, sm, st);
    else if (kind == kKindHeatBath) HGPU_SPAWN(kKindHeatBath);
    else if (kind == kKindHeatBathUniform) HGPU_SPAWN(kKindHeatBathUniform);
    else if (kind == kKindReadInNoRenorm) HGPU_SPAWN(kKindReadInNoRenorm);
    else if (kind == kKindPowerPitzerOcc)
        launch_spawn_kernels<W, kKindPowerPitzerOcc, double, false>(b, R, cur, sm, st);
    else if (kind == kKindPowerPitzerRef)
        launch_spawn_kernels<W, kKindPowerPitzerRef, double, false>(b, R, cur, sm, st);
    else HGPU_SPAWN(HGPU_SYS_READ_IN);
#undef HGPU_SPAWN
    // determ_projection and deterministic_annihilation (src/fciqmc.f90:394,
    // src/annihilation.f90:63-66) before the main list is merged
    if (b.nd > 0) launch_determ_project(b, R, cur, st);
    if (pm) cudaEventRecord(pm->ev[3], st);
    launch_sort_annihilate(b, W, R, cur, st, pm);
    k_cycle_end<<<1, 1024, 0, st>>>(b, R, b.grid, 1);
    // update_rdm_from_spawns on the new main list (src/fciqmc.f90:402-405)
    if (b.rdm) launch_rdm_cycle(b, W, R, 1 - cur, st);
    if (pm) cudaEventRecord(pm->ev[7], st);
}

void launch_cycle(const DevBuffers &b, int W, int R, int kind, int precision, int cur, cudaStream_t st,
                  const PhaseMarks *pm) {
    if (W == 1) cycle_w<1>(b, R, kind, precision, cur, st, pm);
    else cycle_w<2>(b, R, kind, precision, cur, st, pm);
}

int set_kernel_attributes(const DevBuffers &b) {
    // hub_k momentum tables (hub_smem) next to the spawning queues, for up to 255 k-points
    const int hub_max = (int)hub_smem(HGPU_SYS_HUB_K, 255);
    if (cudaFuncSetAttribute(k_spawn<1, HGPU_SYS_HUB_K, double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             hub_max) != cudaSuccess ||
        cudaFuncSetAttribute(k_spawn<2, HGPU_SYS_HUB_K, double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             hub_max) != cudaSuccess)
        return 1;
    if (set_rdm_attributes()) return 1;
    return set_annihilate_attributes(b);
}

int launches_per_cycle(const DevBuffers &b) {
    // begin, prep, count, scan(3), spawn (and singles), clamp, sort_hist,
    // sort_offsets, one per pass, ann_splits, annihilate (twice), end
    return 2 + 1 + 3 + 1 + (b.sq ? 1 : 0) + 1 + 2 + b.sort_passes + 3 + 1;
}

void launch_annihilation(const DevBuffers &b, int W, int R, int kind, int cur, cudaStream_t st) {
    (void)kind;
    k_zero_parts<<<1, kBlock, 0, st>>>(b.part_i, b.grid);
    launch_sort_annihilate(b, W, R, cur, st, nullptr);
    k_cycle_end<<<1, 1024, 0, st>>>(b, R, b.grid, 0);
}

void launch_eval_excitations(const DevBuffers &b, int W, int kind, int precision, const uint64_t *parents,
                             const int64_t *parent_pops, int64_t n, int64_t iteration, int32_t *orbs, double *pgen,
                             double *hmatel, int32_t *allowed, int64_t *nspawn, cudaStream_t st) {
    size_t sm = hub_smem(kind, b.nk);
    int grid = (int)((n + kBlock - 1) / kBlock);
    if (grid < 1) grid = 1;
    if (grid > b.grid) grid = b.grid;
#define HGPU_EVAL(WW, KK, RR)                                                                                   \
    k_eval_excitations<WW, KK, RR><<<grid, kBlock, sm, st>>>(b.sys, parents, parent_pops, n, (uint64_t)iteration, \
                                                             orbs, pgen, hmatel, allowed, nspawn)
    if (W == 1) {
        if (kind == HGPU_SYS_HUB_K) HGPU_EVAL(1, HGPU_SYS_HUB_K, double);
        else if ((kind == kKindHeatBath || kind == kKindHeatBathUniform) && precision == HGPU_PREC_MIXED)
            HGPU_EVAL(1, kKindHeatBath, float);
        else if (kind == kKindHeatBath || kind == kKindHeatBathUniform) HGPU_EVAL(1, kKindHeatBath, double);
        else if (precision == HGPU_PREC_MIXED) HGPU_EVAL(1, HGPU_SYS_READ_IN, float);
        else HGPU_EVAL(1, HGPU_SYS_READ_IN, double);
    } else {
        if (kind == HGPU_SYS_HUB_K) HGPU_EVAL(2, HGPU_SYS_HUB_K, double);
        else if ((kind == kKindHeatBath || kind == kKindHeatBathUniform) && precision == HGPU_PREC_MIXED)
            HGPU_EVAL(2, kKindHeatBath, float);
        else if (kind == kKindHeatBath || kind == kKindHeatBathUniform) HGPU_EVAL(2, kKindHeatBath, double);
        else if (precision == HGPU_PREC_MIXED) HGPU_EVAL(2, HGPU_SYS_READ_IN, float);
        else HGPU_EVAL(2, HGPU_SYS_READ_IN, double);
    }
#undef HGPU_EVAL
}

void launch_eval_diagonal(const DevBuffers &b, int W, const uint64_t *dets, int64_t n, double *kii, cudaStream_t st) {
    int grid = (int)((n + kBlock - 1) / kBlock);
    if (grid < 1) grid = 1;
    if (grid > b.grid) grid = b.grid;
    if (W == 1) k_eval_diagonal<1><<<grid, kBlock, 0, st>>>(b.sys, dets, n, kii);
    else k_eval_diagonal<2><<<grid, kBlock, 0, st>>>(b.sys, dets, n, kii);
}

void launch_load_fixed_spawns(const DevBuffers &b, int W, int R, const int64_t *sdata, int64_t n, cudaStream_t st) {
    if (W == 1) k_load_fixed<1><<<b.grid, kBlock, 0, st>>>(b, R, sdata, n);
    else k_load_fixed<2><<<b.grid, kBlock, 0, st>>>(b, R, sdata, n);
}

void launch_abs_pop(const DevBuffers &b, int R, int cur, cudaStream_t st) {
    k_abs_pop<<<b.grid, kBlock, 0, st>>>(b, R, cur);
}

}  // namespace hgpu
