// hgpu_spawn.cuh -- the spawning kernels of one cycle: excitation generation,
// attempt_to_spawn and the append to the spawned list (src/spawning.F90:34-123,
// 215-315, 588-768), templated on the system / generator kind, the arithmetic
// of the generators and whether replica 2-RDM spawns are recorded.  k_spawn
// classifies the attempts and runs the doubles (or, for the generators that do
// not draw the single/double choice first, every attempt); k_spawn_singles runs
// the singles it queued.  Included by the translation units that instantiate
// them (hgpu_kernels.cu without the RDM, hgpu_spawn_rdm.cu with it).
#pragma once

#include "hgpu_common.cuh"

namespace hgpu {

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


// A warp's chunk of attempts: (parent, space) slot, attempt number in the slot
// and, for generators whose first draw chooses a single or a double excitation,
// the stream position after that draw; list holds the chunk offsets of the
// doubles (or of every attempt) from its start and those of the singles from
// its end.  Entries kSpawnChunk + 32 t + j (t = 0 doubles, 1 singles; j < 32)
// hold the entries of type t left over from the warp's earlier chunks (fewer
// than 32): they run in the next group of 32 of that type, so that every group
// but the warp's last runs with all lanes busy.  (Singles reach type 1 only
// when the singles kernel's queue is full.)
struct SpawnQueue {
    uint32_t slot[kSpawnChunk + 64];
    uint32_t att[kSpawnChunk + 64];
    uint64_t bufk[kSpawnChunk + 64];
    uint8_t list[kSpawnChunk];
};

// One spawning attempt of a queued chunk entry; returns the spawned amount.
template <int W, int KIND, typename Real, bool SINGLE>
__device__ __forceinline__ int64_t spawn_entry(const DevSys &s, const HubTables &t, const DevBuffers &b, int R,
                                               const uint64_t *dets, uint64_t iter, uint32_t slot, uint32_t att,
                                               bool drew, uint64_t bufk, bool rdm, Det<W> &child, int &sp,
                                               uint32_t &info, int64_t &nspawn_rdm) {
    constexpr bool single = SINGLE;
    // R is 1 or 2: a shift instead of an integer division
    const int64_t i = slot >> (R - 1);
    sp = (int)(slot & (uint32_t)(R - 1));
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
        else if (single && KIND == kKindPowerPitzerRef) {
            double h;
            gen_ppn_single<W>(s, rs, d, at, pgen, h);
            hm = (Real)h;
        } else if (single) gen_single_mol<W, Real>(s, rs, d, KIND != kKindReadInNoRenorm, at, pgen, hm);
        else if (KIND == kKindHeatBathUniform) gen_heat_bath_uniform_double<W, Real>(s, rs, f, at, pgen, hm);
        else if (KIND == kKindPowerPitzerOcc) {
            double h;
            gen_pp_occ_double<W>(s, rs, d, at, pgen, h);
            hm = (Real)h;
        } else if (KIND == kKindPowerPitzerRef) {
            double h;
            gen_ppn_double<W>(s, rs, d, at, pgen, h);
            hm = (Real)h;
        } else gen_double_mol<W, Real>(s, rs, d, KIND == HGPU_SYS_READ_IN, at, pgen, hm);
        attempt_to_spawn(s, rs, parent, pgen, (double)hm, at);
        at.nspawn_rdm = 0;
        if (rdm) attempt_to_spawn_rdm(s, rs, parent, at);
    }
    nspawn_rdm = KIND == HGPU_SYS_HUB_K ? 0 : at.nspawn_rdm;
    if (at.nspawn != 0 || nspawn_rdm != 0) child = excited<W>(f, at);
    // no spawning from a deterministic state onto another (src/fciqmc.f90:777-790)
    if (at.nspawn != 0 && b.nd > 0 && (info & kDetermBit)) {
        const int64_t q = lower_bound_det<W>(b.ddets, b.nd, child);
        if (q < b.nd && det_eq<W>(load_det<W>(b.ddets, q), child)) at.nspawn = 0;
    }
    return at.nspawn;
}

// The singles (a tenth of the attempts) in a function of their own, so that the
// doubles' loop in k_spawn stays small in the instruction cache.
template <int W, int KIND, typename Real>
__device__ __noinline__ int64_t spawn_entry_single(const DevSys &s, const HubTables &t, const DevBuffers &b, int R,
                                                   const uint64_t *dets, uint64_t iter, uint32_t slot, uint32_t att,
                                                   uint64_t bufk, bool rdm, Det<W> &child, int &sp, uint32_t &info,
                                                   int64_t &nspawn_rdm) {
    return spawn_entry<W, KIND, Real, true>(s, t, b, R, dets, iter, slot, att, true, bufk, rdm, child, sp, info,
                                            nspawn_rdm);
}

// Generators whose first draw chooses a single or a double excitation: their
// attempts are classified before they run, and the singles (a tenth of the
// attempts, with code of their own) go to the singles kernel.
template <int KIND>
constexpr bool spawn_drew() {
    return KIND == HGPU_SYS_READ_IN || KIND == kKindReadInNoRenorm || KIND == kKindHeatBathUniform ||
           KIND == kKindPowerPitzerOcc || KIND == kKindPowerPitzerRef;
}

// The warp's spawned particles appended to the spawned list and, with the
// replica 2-RDM, its RDM spawns to theirs (create_spawned_particle*): one
// atomic per warp for each list.  Every lane of the warp takes part.
template <int W>
__device__ __forceinline__ void spawn_emit(const DevBuffers &b, DevState *st, int R, int lane, bool want,
                                           const Det<W> &child, int sp, int64_t nspawn, uint64_t flagword,
                                           bool rdm, int64_t nrdm, uint32_t parent) {
    const uint32_t ball = __ballot_sync(FULL_MASK, want);
    if (ball) {
        const int leader = __ffs(ball) - 1;
        unsigned long long basepos = 0;
        if (lane == leader) basepos = atomicAdd((unsigned long long *)&st->n_spawn, (unsigned long long)__popc(ball));
        basepos = __shfl_sync(FULL_MASK, basepos, leader);
        if (want) {
            const int64_t pos = (int64_t)basepos + __popc(ball & lanemask_lt());
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
        // create_spawned_particle_replica_rdm: (parent, child) and the amount; the
        // parent as its main-list index (its determinant is read back from the
        // list when the RDM spawns are added)
        const uint32_t rball = __ballot_sync(FULL_MASK, nrdm != 0);
        if (rball) {
            const int leader = __ffs(rball) - 1;
            unsigned long long rbase = 0;
            if (lane == leader) rbase = atomicAdd((unsigned long long *)&st->n_rdm, (unsigned long long)__popc(rball));
            rbase = __shfl_sync(FULL_MASK, rbase, leader);
            if (nrdm != 0) {
                const int64_t pos = (int64_t)rbase + __popc(rball & lanemask_lt());
                if (pos < b.scap) {
                    store_det<W>(b.rdm_schild, pos, child);
                    b.rdm_sparent[pos] = parent;
                    b.rdm_spops[pos] = nrdm;
                    b.rdm_sspace[pos] = (uint8_t)sp;
                } else {
                    atomicOr(&st->error_flags, HGPU_FLAG_SPAWN_OVERFLOW);
                }
            }
        }
    }
}

// Resident blocks per SM the spawning kernel is compiled for: four (at most 64
// registers, half the SM's warps) for the uniform generators, whose code fits
// that budget without spilling; 0 (no minimum) leaves the heat-bath and
// power-Pitzer kernels to the compiler, which gives them up to 128.
template <int W, int KIND>
constexpr int spawn_min_blocks() {
    return (KIND == HGPU_SYS_HUB_K || KIND == HGPU_SYS_READ_IN || KIND == kKindReadInNoRenorm) ? 4 : 0;
}

template <int W, int KIND, typename Real, bool RDM>
__global__ void __launch_bounds__(kBlock, spawn_min_blocks<W, KIND>()) k_spawn(DevBuffers b, int R, int cur) {
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
    // replica 2-RDM sampling (spawn_rdm) once the engine turned it on; the
    // kernels without it (RDM false) carry none of its code
    const bool rdm = RDM && b.rdm != nullptr && st->rdm_on != 0;
    // generators whose first draw is the single/double choice: the chunk is
    // split by that draw so that each excitation type runs with the warp
    // converged (a tenth of the attempts are singles, with their own code)
    constexpr bool drew = spawn_drew<KIND>();
    // Each warp claims chunks of b.spawn_chunk consecutive attempts.  The (parent,
    // space) slot of attempt a is the first k with aoff[k] > a; one binary search
    // per chunk finds the slot of its first attempt, and every later step of 32
    // attempts searches a window of 32 slots starting at the slot of the previous
    // step's last attempt (a lower bound), with the binary search as fallback when
    // a window holds no slot for an attempt (runs of zero-attempt slots).
    // Each type's attempts run in groups of 32; a chunk's last, partial group of
    // a type is carried to the next chunk (SpawnQueue), and the carried entries
    // run once the warp finds no more chunks.
    int ncarry0 = 0, ncarry1 = 0;  // carried doubles, singles
    for (;;) {
        unsigned long long cbase = 0;
        if (lane == 0) cbase = atomicAdd((unsigned long long *)&st->spawn_next, (unsigned long long)b.spawn_chunk);
        cbase = __shfl_sync(FULL_MASK, cbase, 0);
        const bool more = (int64_t)cbase < A;
        if (!more && ncarry0 == 0 && ncarry1 == 0) break;
        const int64_t cend = more ? min((int64_t)cbase + b.spawn_chunk, A) : (int64_t)cbase;
        int64_t k0 = 0;
        if (lane == 0 && more) k0 = upper_bound_off(b.aoff, NR, (int64_t)cbase);
        k0 = __shfl_sync(FULL_MASK, k0, 0);
        int nd = 0, ns = 0;
        for (int64_t base = (int64_t)cbase; base < cend; base += 32) {
            int64_t a = base + lane;
            const int64_t wv = k0 + lane < NR ? b.aoff[k0 + lane] : INT64_MAX;
            // end of window slot m relative to this step, clamped to [0, 33]:
            // aoff[k0 + m] <= a exactly when e_m <= lane, and e is
            // non-decreasing in m, so the count of such m is found by a
            // binary search over the lanes
            const int64_t ed = wv - base;
            const int e = ed < 0 ? 0 : (ed > 33 ? 33 : (int)ed);
            int cnt = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(FULL_MASK, e, cnt + step - 1) <= lane) cnt += step;
            if (__shfl_sync(FULL_MASK, e, cnt) <= lane) cnt++;
            int64_t k = NR;
            bool valid = a < cend, single = false;
            if (valid) {
                k = (cnt < 32 && k0 + cnt < NR) ? k0 + cnt : upper_bound_off(b.aoff, NR, a);
                int64_t att = a - (k > 0 ? b.aoff[k - 1] : 0);
                int off = (int)(a - (int64_t)cbase);
                q.slot[off] = (uint32_t)k;
                q.att[off] = (uint32_t)att;
                if (drew) {
                    const int64_t i = k >> (R - 1);
                    RStream rs;
                    rs.init(s.seed, P_SPAWN, (uint32_t)(k & (R - 1)), i, att, iter);
                    single = rs.next_k() < s.t_single;  // rs.next() < pattempt_single
                    q.bufk[off] = rs.bufk;
                }
            }
            uint32_t dball = __ballot_sync(FULL_MASK, valid && !single);
            uint32_t sball = __ballot_sync(FULL_MASK, valid && single);
            int off = (int)(a - (int64_t)cbase);
            if (valid && !single) q.list[nd + __popc(dball & lanemask_lt())] = (uint8_t)off;
            if (valid && single) q.list[kSpawnChunk - 1 - ns - __popc(sball & lanemask_lt())] = (uint8_t)off;
            nd += __popc(dball);
            ns += __popc(sball);
            // slot of the last valid attempt of this step: lower bound for the next step
            int last = (int)min((int64_t)31, cend - 1 - base);
            k0 = __shfl_sync(FULL_MASK, k, last);
        }
        __syncwarp();
        // the chunk's singles to the singles kernel's queue; those past its
        // capacity (the counter may pass it) run here
        int s0 = 0;
        if (drew && b.sq && ns > 0) {
            unsigned long long qb = 0;
            if (lane == 0) qb = atomicAdd((unsigned long long *)&st->n_sq, (unsigned long long)ns);
            qb = __shfl_sync(FULL_MASK, qb, 0);
            const int64_t room = b.sq_cap - (int64_t)qb;
            s0 = room <= 0 ? 0 : (room < ns ? (int)room : ns);
            for (int j = lane; j < s0; j += 32) {
                const int off = q.list[kSpawnChunk - 1 - j];
                const uint64_t bk = q.bufk[off];
                b.sq[qb + j] = make_uint4(q.slot[off], q.att[off], (uint32_t)bk, (uint32_t)(bk >> 32));
            }
        }
        // doubles (or every attempt), then singles, in groups of 32: the carried
        // entries of the type first, then the chunk's; the last partial group
        // is carried unless no chunk is left
        for (int pass = 0; pass < 2; pass++) {
            const int c = pass == 0 ? ncarry0 : ncarry1;
            const int tot = c + (pass == 0 ? nd : ns - s0);
            const int full = more ? tot & ~31 : tot;
            const int cbase_e = kSpawnChunk + 32 * pass;  // the type's carried entries
            for (int j0 = 0; j0 < full; j0 += 32) {
                bool want = false;
                Det<W> child;
                int64_t nspawn = 0, nrdm = 0;
                int sp = 0;
                uint64_t flagword = 0;
                uint32_t pidx = 0;
                const int j = j0 + lane;
                if (j < full) {
                    const int e = j < c ? cbase_e + j : q.list[pass == 0 ? j - c : kSpawnChunk - 1 - s0 - (j - c)];
                    pidx = q.slot[e] >> (R - 1);
                    uint32_t info;
                    if (pass == 0)
                        nspawn = spawn_entry<W, KIND, Real, false>(s, t, b, R, dets, iter, q.slot[e], q.att[e],
                                                                   drew, q.bufk[e], rdm, child, sp, info, nrdm);
                    else
                        nspawn = spawn_entry_single<W, KIND, Real>(s, t, b, R, dets, iter, q.slot[e], q.att[e],
                                                                   q.bufk[e], rdm, child, sp, info, nrdm);
                    if (nspawn != 0) {
                        want = true;
                        // the attempt's index: a carried entry's from its slot (aoff[slot - 1] + att)
                        const uint32_t sl = q.slot[e];
                        const uint64_t aidx = e >= kSpawnChunk ? (sl > 0 ? b.aoff[sl - 1] : 0) + q.att[e] : cbase + e;
                        flagword = (uint64_t)((info >> 2) & 3u) | (aidx << 2);
                    }
                }
                spawn_emit<W>(b, st, R, lane, want, child, sp, nspawn, flagword, rdm, nrdm, pidx);
            }
            __syncwarp();
            // carry entries full..tot-1 (fewer than 32; none once no chunk is
            // left): with full == 0 the carried ones stay where they are and
            // the chunk's are appended; otherwise every carried one ran and the
            // rest are the chunk's
            const int rest = tot - full;
            const int j = full + lane;
            if (lane < rest && j >= c) {
                const int off = q.list[pass == 0 ? j - c : kSpawnChunk - 1 - s0 - (j - c)];
                q.slot[cbase_e + lane] = q.slot[off];
                q.att[cbase_e + lane] = q.att[off];
                q.bufk[cbase_e + lane] = q.bufk[off];
            }
            if (pass == 0) ncarry0 = rest;
            else ncarry1 = rest;
            __syncwarp();
        }
        if (!more) break;
    }
}

// The queued singles (k_spawn above), 32 per warp at a time: the single
// excitations' code runs in a kernel of its own, so that the spawning kernel's
// loop stays small in the instruction cache.
template <int W, int KIND, typename Real, bool RDM>
__global__ void __launch_bounds__(kBlock, spawn_min_blocks<W, KIND>()) k_spawn_singles(DevBuffers b, int R, int cur) {
    __shared__ DevSys s;
    extern __shared__ uint8_t smem[];
    stage_sys(s, b.sys);
    HubTables t = stage_hub(b.sys, smem);
    __syncthreads();
    DevState *st = b.state;
    const int64_t n = st->n_sq < b.sq_cap ? st->n_sq : b.sq_cap;
    const uint64_t iter = (uint64_t)st->iter;
    const uint64_t *dets = b.dets[cur];
    const int lane = threadIdx.x & 31;
    const bool rdm = RDM && b.rdm != nullptr && st->rdm_on != 0;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32) {
        bool want = false;
        Det<W> child;
        int64_t nspawn = 0, nrdm = 0;
        int sp = 0;
        uint64_t flagword = 0;
        uint32_t pidx = 0;
        const int64_t j = base + lane;
        if (j < n) {
            const uint4 e = b.sq[j];
            pidx = e.x >> (R - 1);
            uint32_t info;
            nspawn = spawn_entry_single<W, KIND, Real>(s, t, b, R, dets, iter, e.x, e.y,
                                                       (uint64_t)e.z | ((uint64_t)e.w << 32), rdm, child, sp, info,
                                                       nrdm);
            if (nspawn != 0) {
                want = true;
                // the attempt's index: aoff[slot - 1] + attempt in the slot
                const uint64_t aidx = (e.x > 0 ? b.aoff[e.x - 1] : 0) + e.y;
                flagword = (uint64_t)((info >> 2) & 3u) | (aidx << 2);
            }
        }
        spawn_emit<W>(b, st, R, lane, want, child, sp, nspawn, flagword, rdm, nrdm, pidx);
    }
}

// The spawning kernel and, for the generators that classify their attempts,
// the singles kernel after it.
template <int W, int KIND, typename Real, bool RDM>
void launch_spawn_kernels(const DevBuffers &b, int R, int cur, size_t sm, cudaStream_t st) {
    k_spawn<W, KIND, Real, RDM><<<b.spawn_grid, kBlock, sm, st>>>(b, R, cur);
    if constexpr (spawn_drew<KIND>()) {
        if (b.sq) k_spawn_singles<W, KIND, Real, RDM><<<b.spawn_grid, kBlock, sm, st>>>(b, R, cur);
    }
}

}  // namespace hgpu
