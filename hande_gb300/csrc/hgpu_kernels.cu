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
        for (int sp = 0; sp < R; sp++) {
            int64_t p = pops[i * R + sp];
            double rp = (double)p * inv_rf;
            // update_proj_energy
            if (e.nexcit == 0) d0[sp] += rp;
            else proj[sp] += h * rp;
            // set_parent_flag: bit set if not an initiator
            if (!(fabs(rp) > s.initiator_pop)) info |= 4u << sp;
            if (p < 0) info |= 1u << sp;
            RStream rs;
            rs.init(s.seed, P_NATTEMPT, sp, i, 0, iter);
            b.natt[i * R + sp] = decide_nattempts_fx(rs, p, s.real_amplitudes ? 31 : 0, rp);
            rs.init(s.seed, P_DEATH, sp, i, 0, iter);
            ndeath += stochastic_death(s.tau, rs, k, shift[sp], p);
            pops[i * R + sp] = p;
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

// first k in [0, n) with off[k] > a (off is the inclusive scan of attempts)
__device__ __forceinline__ int64_t upper_bound_off(const int64_t *off, int64_t n, int64_t a) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (off[mid] > a) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Attempts per chunk a warp claims from the spawning kernel's work counter.
constexpr int kSpawnChunk = 8 * 32;

// A warp's chunk of attempts: (parent, space) slot, attempt number in the slot
// and, for generators whose first draw chooses a single or a double excitation,
// the stream position after that draw; dlist/slist hold the chunk offsets of
// the doubles (or of every attempt) and of the singles.
struct SpawnQueue {
    uint32_t slot[kSpawnChunk];
    uint32_t att[kSpawnChunk];
    uint64_t bufk[kSpawnChunk];
    uint8_t dlist[kSpawnChunk];
    uint8_t slist[kSpawnChunk];
};

// One spawning attempt of a queued chunk entry; returns the spawned amount.
template <int W, int KIND, typename Real, bool SINGLE>
__device__ __forceinline__ int64_t spawn_entry(const DevSys &s, const HubTables &t, const DevBuffers &b, int R,
                                               const uint64_t *dets, uint64_t iter, uint32_t slot, uint32_t att,
                                               bool drew, uint64_t bufk, bool rdm, Det<W> &child, int &sp,
                                               uint32_t &info, Det<W> &parent_det, int64_t &nspawn_rdm) {
    constexpr bool single = SINGLE;
    int64_t i = slot / R;
    sp = (int)(slot - i * R);
    Det<W> f = load_det<W>(dets, i);
    info = b.pinfo[i];
    int64_t parent = (info >> sp) & 1u ? -1 : 1;
    RStream rs;
    rs.init(s.seed, P_SPAWN, sp, i, att, iter);
    if (drew) {  // resume after the single/double draw
        rs.block = 1;
        rs.have = true;
        rs.bufk = bufk;
    }
    Attempt at;
    at.from[0] = at.from[1] = at.to[0] = at.to[1] = -1;
    if (KIND == HGPU_SYS_HUB_K) {
        attempt_hub_k<W>(s, t, rs, f, parent, false, at);
    } else {
        MolDet<W> d;
        mol_decode<W>(s, f, d);
        double pgen;
        Real hm;
        if (KIND == kKindHeatBath) gen_heat_bath<W, Real>(s, rs, f, at, pgen, hm);
        else if (single && KIND == kKindHeatBathUniform && s.excit_gen == HGPU_EXCIT_GEN_HEAT_BATH_SINGLE)
            gen_single_hb_exact<W, Real>(s, rs, d, at, pgen, hm);
        else if (single) gen_single_mol<W, Real>(s, rs, d, KIND != kKindReadInNoRenorm, at, pgen, hm);
        else if (KIND == kKindHeatBathUniform) gen_heat_bath_uniform_double<W, Real>(s, rs, f, at, pgen, hm);
        else gen_double_mol<W, Real>(s, rs, d, KIND == HGPU_SYS_READ_IN, at, pgen, hm);
        attempt_to_spawn(s, rs, parent, pgen, (double)hm, at);
        at.nspawn_rdm = 0;
        if (rdm) attempt_to_spawn_rdm(s, rs, parent, at);
    }
    nspawn_rdm = KIND == HGPU_SYS_HUB_K ? 0 : at.nspawn_rdm;
    parent_det = f;
    if (at.nspawn != 0 || nspawn_rdm != 0) child = excited<W>(f, at);
    return at.nspawn;
}

// The singles (a tenth of the attempts) in a function of their own, so that the
// doubles' loop in k_spawn stays small in the instruction cache.
template <int W, int KIND, typename Real>
__device__ __noinline__ int64_t spawn_entry_single(const DevSys &s, const HubTables &t, const DevBuffers &b, int R,
                                                   const uint64_t *dets, uint64_t iter, uint32_t slot, uint32_t att,
                                                   uint64_t bufk, bool rdm, Det<W> &child, int &sp, uint32_t &info,
                                                   Det<W> &parent_det, int64_t &nspawn_rdm) {
    return spawn_entry<W, KIND, Real, true>(s, t, b, R, dets, iter, slot, att, true, bufk, rdm, child, sp, info,
                                            parent_det, nspawn_rdm);
}

template <int W, int KIND, typename Real>
__global__ void __launch_bounds__(kBlock) k_spawn(DevBuffers b, int R, int cur) {
    __shared__ DevSys s;
    __shared__ SpawnQueue queue[kBlock / 32];
    extern __shared__ uint8_t smem[];
    stage_sys(s, b.sys);
    HubTables t = stage_hub(b.sys, smem);
    __syncthreads();
    DevState *st = b.state;
    const int64_t A = st->n_attempts;
    const int64_t NR = st->n_main * R;
    const uint64_t iter = (uint64_t)st->iter;
    const uint64_t *dets = b.dets[cur];
    const int lane = threadIdx.x & 31;
    SpawnQueue &q = queue[threadIdx.x >> 5];
    // replica 2-RDM sampling (spawn_rdm) once the engine turned it on
    const bool rdm = b.rdm != nullptr && st->rdm_on != 0;
    // generators whose first draw is the single/double choice: the chunk is
    // split by that draw so that each excitation type runs with the warp
    // converged (a tenth of the attempts are singles, with their own code)
    constexpr bool drew = KIND == HGPU_SYS_READ_IN || KIND == kKindReadInNoRenorm || KIND == kKindHeatBathUniform;
    // Each warp claims chunks of kSpawnChunk consecutive attempts.  The (parent,
    // space) slot of attempt a is the first k with aoff[k] > a; one binary search
    // per chunk finds the slot of its first attempt, and every later step of 32
    // attempts searches a window of 32 slots starting at the slot of the previous
    // step's last attempt (a lower bound), with the binary search as fallback when
    // a window holds no slot for an attempt (runs of zero-attempt slots).
    for (;;) {
        unsigned long long cbase = 0;
        if (lane == 0) cbase = atomicAdd((unsigned long long *)&st->spawn_next, (unsigned long long)kSpawnChunk);
        cbase = __shfl_sync(FULL_MASK, cbase, 0);
        if ((int64_t)cbase >= A) break;
        const int64_t cend = min((int64_t)cbase + kSpawnChunk, A);
        int64_t k0 = 0;
        if (lane == 0) k0 = upper_bound_off(b.aoff, NR, (int64_t)cbase);
        k0 = __shfl_sync(FULL_MASK, k0, 0);
        int nd = 0, ns = 0;
        for (int64_t base = (int64_t)cbase; base < cend; base += 32) {
            int64_t a = base + lane;
            int64_t wv = k0 + lane < NR ? b.aoff[k0 + lane] : INT64_MAX;
            uint32_t le_mask = 0;
#pragma unroll 1
            for (int m = 0; m < 32; m++) {
                int64_t v = __shfl_sync(FULL_MASK, wv, m);
                if (v <= a) le_mask |= 1u << m;
            }
            int64_t k = NR;
            bool valid = a < cend, single = false;
            if (valid) {
                int cnt = __popc(le_mask);
                k = (cnt < 32 && k0 + cnt < NR) ? k0 + cnt : upper_bound_off(b.aoff, NR, a);
                int64_t att = a - (k > 0 ? b.aoff[k - 1] : 0);
                int off = (int)(a - (int64_t)cbase);
                q.slot[off] = (uint32_t)k;
                q.att[off] = (uint32_t)att;
                if (drew) {
                    int64_t i = k / R;
                    RStream rs;
                    rs.init(s.seed, P_SPAWN, (uint32_t)(k - i * R), i, att, iter);
                    single = rs.next_k() < s.t_single;  // rs.next() < pattempt_single
                    q.bufk[off] = rs.bufk;
                }
            }
            uint32_t dball = __ballot_sync(FULL_MASK, valid && !single);
            uint32_t sball = __ballot_sync(FULL_MASK, valid && single);
            int off = (int)(a - (int64_t)cbase);
            if (valid && !single) q.dlist[nd + __popc(dball & lanemask_lt())] = (uint8_t)off;
            if (valid && single) q.slist[ns + __popc(sball & lanemask_lt())] = (uint8_t)off;
            nd += __popc(dball);
            ns += __popc(sball);
            // slot of the last valid attempt of this step: lower bound for the next step
            int last = (int)min((int64_t)31, cend - 1 - base);
            k0 = __shfl_sync(FULL_MASK, k, last);
        }
        __syncwarp();
        // doubles (or every attempt), then singles, 32 at a time
        for (int pass = 0; pass < 2; pass++) {
            const int n = pass == 0 ? nd : ns;
            const uint8_t *list = pass == 0 ? q.dlist : q.slist;
            for (int j0 = 0; j0 < n; j0 += 32) {
                bool want = false;
                Det<W> child, parent_det;
                int64_t nspawn = 0, nrdm = 0;
                int sp = 0;
                uint64_t flagword = 0;
                if (j0 + lane < n) {
                    int off = list[j0 + lane];
                    uint32_t info;
                    if (pass == 0)
                        nspawn = spawn_entry<W, KIND, Real, false>(s, t, b, R, dets, iter, q.slot[off], q.att[off],
                                                                   drew, q.bufk[off], rdm, child, sp, info,
                                                                   parent_det, nrdm);
                    else
                        nspawn = spawn_entry_single<W, KIND, Real>(s, t, b, R, dets, iter, q.slot[off], q.att[off],
                                                                   q.bufk[off], rdm, child, sp, info, parent_det,
                                                                   nrdm);
                    if (nspawn != 0) {
                        want = true;
                        flagword = (uint64_t)((info >> 2) & 3u) | ((uint64_t)(cbase + off) << 2);
                    }
                }
                uint32_t ball = __ballot_sync(FULL_MASK, want);
                if (ball) {
                    int leader = __ffs(ball) - 1;
                    unsigned long long basepos = 0;
                    if (lane == leader)
                        basepos = atomicAdd((unsigned long long *)&st->n_spawn, (unsigned long long)__popc(ball));
                    basepos = __shfl_sync(FULL_MASK, basepos, leader);
                    if (want) {
                        int64_t pos = (int64_t)basepos + __popc(ball & lanemask_lt());
                        if (pos < b.scap) {
                            store_det<W>(b.sdets, pos, child);
                            for (int qq = 0; qq < R; qq++) b.spops[pos * R + qq] = qq == sp ? nspawn : 0;
                            if (b.sflag) b.sflag[pos] = flagword;
                        } else {
                            atomicOr(&st->error_flags, HGPU_FLAG_SPAWN_OVERFLOW);
                        }
                    }
                }
                if (rdm) {
                    // create_spawned_particle_replica_rdm: (parent, child) and the amount
                    const uint32_t rball = __ballot_sync(FULL_MASK, nrdm != 0);
                    if (rball) {
                        const int leader = __ffs(rball) - 1;
                        unsigned long long rbase = 0;
                        if (lane == leader)
                            rbase = atomicAdd((unsigned long long *)&st->n_rdm, (unsigned long long)__popc(rball));
                        rbase = __shfl_sync(FULL_MASK, rbase, leader);
                        if (nrdm != 0) {
                            const int64_t pos = (int64_t)rbase + __popc(rball & lanemask_lt());
                            if (pos < b.scap) {
                                store_det<W>(b.rdm_sdets, 2 * pos, parent_det);
                                store_det<W>(b.rdm_sdets, 2 * pos + 1, child);
                                b.rdm_spops[pos] = nrdm;
                                b.rdm_sspace[pos] = (uint8_t)sp;
                            } else {
                                atomicOr(&st->error_flags, HGPU_FLAG_SPAWN_OVERFLOW);
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();
    }
}


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
    if (blockIdx.x == 0 && threadIdx.x == 0) b.state->n_spawn = n;
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
#define HGPU_SPAWN(KK)                                                                      \
    do {                                                                                    \
        if (precision == HGPU_PREC_MIXED)                                                   \
            k_spawn<W, KK, float><<<b.spawn_grid, kBlock, sm, st>>>(b, R, cur);             \
        else                                                                                \
            k_spawn<W, KK, double><<<b.spawn_grid, kBlock, sm, st>>>(b, R, cur);            \
    } while (0)
    if (kind == HGPU_SYS_HUB_K) k_spawn<W, HGPU_SYS_HUB_K, double><<<b.spawn_grid, kBlock, sm, st>>>(b, R, cur);
    else if (kind == kKindHeatBath) HGPU_SPAWN(kKindHeatBath);
    else if (kind == kKindHeatBathUniform) HGPU_SPAWN(kKindHeatBathUniform);
    else if (kind == kKindReadInNoRenorm) HGPU_SPAWN(kKindReadInNoRenorm);
    else HGPU_SPAWN(HGPU_SYS_READ_IN);
#undef HGPU_SPAWN
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
    if (cudaFuncSetAttribute(k_spawn<1, HGPU_SYS_HUB_K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             hub_max) != cudaSuccess ||
        cudaFuncSetAttribute(k_spawn<2, HGPU_SYS_HUB_K, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             hub_max) != cudaSuccess)
        return 1;
    if (set_rdm_attributes()) return 1;
    return set_annihilate_attributes(b);
}

int launches_per_cycle(const DevBuffers &b) {
    // begin, prep, count, scan(3), spawn, clamp, sort_hist, sort_offsets,
    // one per pass, ann_splits, annihilate (twice), end
    return 2 + 1 + 3 + 1 + 1 + 2 + b.sort_passes + 3 + 1;
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
