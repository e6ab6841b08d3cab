// hgpu_annihilate.cu -- sort and annihilation of one cycle: the radix sort of
// the spawned list (hgpu_sort.cuh) and the annihilation of the sorted spawned
// list with the main list in one pass over the merged sequence.
//
// direct_annihilation (src/annihilation.f90:9-80) runs, in the reference, as
// annihilate_spawn_t[_initiator] (src/spawn_data.F90:859-1101: equal spawned
// determinants summed), annihilate_main_list[_initiator]
// (src/annihilation.f90:294-486: the sums added to the main list),
// remove_unoccupied_dets (:537-598), round_low_population_spawns (:600-675) and
// insert_new_walkers (:677-901: the surviving new determinants merged in, with
// K_ii).  Here all of it is one merge of the main list (sorted, distinct) with
// the sorted spawned list (duplicates adjacent), main entry first among equal
// determinants, so that every determinant forms one contiguous group
// [main entry][spawned entries].  The merged sequence is cut into tiles of
// ann_tile<W>() elements at group boundaries (k_ann_splits); a tile (k_annihilate)
// stages its slices in shared memory, sums every group at its head, rounds,
// counts its survivors, takes its output offset from a decoupled look-back over
// the preceding tiles, and writes the survivors, in order, to the other main
// buffer.  Nothing but the sort and the new main list goes through HBM.
//
// The rounding stream of a new determinant is keyed by the sorted position of
// its first spawned entry (the number of spawned entries below it), which
// does not depend on the order in which equal entries were spawned.
#include "hgpu_common.cuh"

namespace hgpu {

__global__ void k_clamp_spawns(DevState *st, int64_t scap) {
    if (st->n_spawn > scap) {
        st->n_spawn = scap;
        st->error_flags |= HGPU_FLAG_SPAWN_OVERFLOW;
    }
}

}  // namespace hgpu

#include "hgpu_sort.cuh"

namespace hgpu {


// Sums of one group's spawned entries; for the initiator approximation also
// the particles from initiators, the coherent events of the others and the
// entry generated first (annihilate_spawn_t_initiator, src/spawn_data.F90:937-1101).
// Every part is order-independent, so partial sums combine in any order.
struct SegAcc {
    int64_t sum[2], ip[2], ev[2], fpop[2];
    uint64_t ford, fflag;  // generation order and flag word of the first entry
    __device__ __forceinline__ void init() {
        sum[0] = sum[1] = ip[0] = ip[1] = ev[0] = ev[1] = fpop[0] = fpop[1] = 0;
        ford = ~0ull;
        fflag = 0;
    }
    __device__ __forceinline__ void add(int R, bool initiator, const int64_t p[2], uint64_t fl) {
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (q < R) {
                sum[q] += p[q];
                if (initiator) {
                    if (!((fl >> q) & 1)) ip[q] += p[q];
                    else ev[q] += sgn3(p[q]);
                }
            }
        if (initiator && (fl >> 2) < ford) {
            ford = fl >> 2;
            fflag = fl;
            fpop[0] = p[0];
            fpop[1] = p[1];
        }
    }
    __device__ __forceinline__ void merge(const SegAcc &o) {
        for (int q = 0; q < 2; q++) {
            sum[q] += o.sum[q];
            ip[q] += o.ip[q];
            ev[q] += o.ev[q];
        }
        if (o.ford < ford) {
            ford = o.ford;
            fflag = o.fflag;
            fpop[0] = o.fpop[0];
            fpop[1] = o.fpop[1];
        }
    }
    __device__ __forceinline__ bool any(int R) const { return sum[0] != 0 || (R > 1 && sum[1] != 0); }
    // Spaces whose sum may not create a new walker: neither sign-coherent with
    // the initiator-sourced particles nor carried by more than one coherent
    // event; the first entry counts sign(1, int(pop)) events.
    __device__ __forceinline__ uint64_t flag(int R, bool initiator) const {
        uint64_t f = 0;
        if (!initiator) return f;
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (q < R) {
                int64_t e = ev[q];
                if ((fflag >> q) & 1) e += sign1_int32(fpop[q]) - sgn3(fpop[q]);
                bool keep = (ip[q] != 0 && sgn1(sum[q]) == sgn1(ip[q])) || e > 1 || e < -1;
                if (!keep) f |= 1ull << q;
            }
        return f;
    }
};

__device__ __forceinline__ SegAcc shfl_down_acc(const SegAcc &a, int off) {
    SegAcc o;
    for (int q = 0; q < 2; q++) {
        o.sum[q] = __shfl_down_sync(0xffffffffu, a.sum[q], off);
        o.ip[q] = __shfl_down_sync(0xffffffffu, a.ip[q], off);
        o.ev[q] = __shfl_down_sync(0xffffffffu, a.ev[q], off);
        o.fpop[q] = __shfl_down_sync(0xffffffffu, a.fpop[q], off);
    }
    o.ford = __shfl_down_sync(0xffffffffu, a.ford, off);
    o.fflag = __shfl_down_sync(0xffffffffu, a.fflag, off);
    return o;
}

// Decoupled look-back (Merrill and Garland, "Single-pass Parallel Prefix Scan
// with Decoupled Look-back", 2016) of one tile, by one thread: publishes the
// tile's count, sums the predecessors' counts back to the first inclusive
// prefix, publishes its own inclusive prefix and returns the exclusive one.
// Tiles run in ticket order, so every predecessor is running or done; a wait
// that exceeds kSpinLimit polls raises HGPU_FLAG_TIMEOUT and gives up.
__device__ __forceinline__ uint32_t tile_lookback(uint64_t *status, int64_t tile, uint32_t epoch, uint32_t run,
                                                  DevState *st) {
    volatile uint64_t *my = status + tile;
    if (tile == 0) {
        *my = os_word(kOSPrefix, epoch, run);
        return 0;
    }
    *my = os_word(kOSAggregate, epoch, run);
    uint32_t excl = 0;
    int64_t kk = tile - 1;
    int spins = 0;
    for (;;) {
        uint64_t v[kOSLook];
#pragma unroll
        for (int u = 0; u < kOSLook; u++) v[u] = kk - u >= 0 ? *(volatile uint64_t *)(status + (kk - u)) : 0;
        int u = 0;
        bool done = false;
        for (; u < kOSLook && kk - u >= 0; u++) {
            uint32_t ve = (uint32_t)(v[u] >> 32) & 0x3FFFFFFFu;
            uint64_t fl = v[u] >> 62;
            if (ve != (epoch & 0x3FFFFFFFu) || fl == 0) break;
            excl += (uint32_t)v[u];
            if (fl == kOSPrefix) {
                done = true;
                break;
            }
        }
        if (done) break;
        kk -= u;
        if (u == 0) {
            if (++spins > kSpinLimit) {
                atomicOr(&st->error_flags, HGPU_FLAG_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
    }
    *my = os_word(kOSPrefix, epoch, excl + run);
    return excl;
}

// Sorted spawned entry j: its index in the spawned list and its determinant
// (from the sorted keys when they are the determinants, else gathered).
template <int W, bool RANK>
struct SortedSpawns {
    const uint64_t *keys;
    const uint32_t *idx;
    const uint64_t *sdets;
    __device__ __forceinline__ uint32_t at(int64_t j) const { return idx ? idx[j] : (uint32_t)j; }
    __device__ __forceinline__ Det<W> det(int64_t j) const {
        if (RANK) return load_det<W>(sdets, at(j));
        return load_det<W>(keys, j);
    }
};

// Merge-path cuts (Odeh et al., "Merge Path", 2012) of the main list and the
// sorted spawned list at every diagonal t * ann_tile<W>(), and the same cuts moved
// past the spawned entries equal to the last element before them, so that no
// group of equal determinants straddles two tiles.  msplit[3t..3t+2] = (main
// index, spawned index, spawned index at the group boundary).  One warp per
// cut: each round probes 32 points of the search interval at once, so a cut
// costs log32 of the list length dependent gathers instead of log2.  Also
// resets the counters and tickets of k_annihilate and advances its look-back
// epoch.
template <int W, bool RANK>
__global__ void __launch_bounds__(kBlock) k_ann_splits(DevBuffers b, int cur, const uint64_t *keys,
                                                       const uint32_t *idx) {
    constexpr int TILE = ann_tile<W>();
    DevState *st = b.state;
    const int64_t N = st->n_main, S = st->n_spawn, L = N + S;
    const int64_t ntiles = (L + TILE - 1) / TILE;
    const uint64_t *mdets = b.dets[cur];
    const SortedSpawns<W, RANK> sp{keys, idx, b.sdets};
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->ann_ticket[0] = st->ann_ticket[1] = 0;
        st->n_uniq = 0;
        st->n_merged_keep = 0;
        *b.seg_epoch += 2;
    }
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t t = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t <= ntiles; t += warps) {
        const int64_t d = t * TILE < L ? t * TILE : L;
        // first i in [lo, hi] with spawned[d-1-i] < main[i] (hi if none): main[i]
        // precedes spawned[d-1-i] exactly when main[i] <= spawned[d-1-i]
        int64_t lo = d - S > 0 ? d - S : 0, hi = d < N ? d : N;
        while (hi > lo) {
            const int64_t len = hi - lo;
            const int64_t step = (len + 31) / 32;  // probes lo + step*(lane+1) - 1 cover [lo, hi)
            const int64_t m = lo + step * (lane + 1) - 1;
            bool before = false;  // main[m] precedes spawned[d-1-m]
            if (m < hi) before = !det_less<W>(sp.det(d - 1 - m), load_det<W>(mdets, m));
            const uint32_t bal = __ballot_sync(0xffffffffu, m < hi && before);
            // the predicate is true then false along m: the first false probe bounds the answer
            const int ntrue = __popc(bal);
            const int64_t nlo = lo + step * ntrue;  // every probe below is true
            int64_t nhi = lo + step * (ntrue + 1) - 1;
            if (nhi > hi) nhi = hi;
            lo = nlo;
            hi = nhi;
            if (step == 1) {
                lo = hi = nlo;
            }
        }
        const int64_t i = lo, j = d - lo;
        int64_t jadj = j;
        if (lane == 0 && (i > 0 || j > 0) && j < S) {
            // the element before the cut: main[i-1] unless spawned[j-1] follows it
            const bool prev_main = i > 0 && (j == 0 || det_less<W>(sp.det(j - 1), load_det<W>(mdets, i - 1)));
            const Det<W> prev = prev_main ? load_det<W>(mdets, i - 1) : sp.det(j - 1);
            if (det_eq<W>(sp.det(j), prev)) {
                // galloping search for the end of the run equal to prev
                int64_t in = j, gstep = 1;  // spawned[in] == prev
                while (in + gstep < S && det_eq<W>(sp.det(in + gstep), prev)) {
                    in += gstep;
                    gstep <<= 1;
                }
                int64_t out = in + gstep < S ? in + gstep : S;  // spawned[out] != prev, or out == S
                while (out - in > 1) {
                    int64_t mid = (in + out) >> 1;
                    if (det_eq<W>(sp.det(mid), prev)) in = mid;
                    else out = mid;
                }
                jadj = out;
            }
        }
        if (lane == 0) {
            b.msplit[3 * t + 0] = i;
            b.msplit[3 * t + 1] = j;
            b.msplit[3 * t + 2] = jadj;
        }
    }
}

// One pass of the annihilation over the merged sequence (see the top of this
// file).  mode 0 keeps every survivor; mode 1 runs only when mode 0 found more
// survivors than the main list holds, and then keeps the main-list survivors
// alone (insert_new_walkers refuses the new determinants, and the overflow is
// flagged).  Dynamic shared memory: the exact-diagonal tables
// (fx_table_words, unless they are read from global memory), the tile's
// populations (TILE x R) and, with the initiator approximation, its spawned
// flag words (TILE).
//
// A tile runs in phases that keep the warps converged: the merge walk (each
// thread a run of PER merged positions, from one merge-path search) gives
// the slot of every merged position; the groups are then summed, combined and
// rounded with consecutive threads on consecutive positions, so that the
// Philox rounding of neighbouring entries runs together; the survivors are
// compacted by one block scan and written, K_ii included, with consecutive
// threads on consecutive outputs.
// Resident blocks per SM: four for two-word determinants (tiles of 1024, the
// exact-diagonal tables read through L1: shared memory allows four, and the
// extra warps cover the gathers' latency -- 3 % faster than three at 80
// registers, despite a few spilled words), three for one-word ones (tiles of
// 2048 with staged tables, which shared memory limits to three).
template <int W>
constexpr int ann_min_blocks() {
    return W == 2 ? 4 : 3;
}

template <int W, bool RANK>
__global__ void __launch_bounds__(kBlock, ann_min_blocks<W>()) k_annihilate(DevBuffers b, int R, int cur,
                                                                            const uint64_t *keys, const uint32_t *idx,
                                                                            int mode) {
    constexpr int TILE = ann_tile<W>();
    constexpr int PER = TILE / kBlock;  // consecutive merged positions per thread
    static_assert(PER == 4 || PER == 8, "a thread's codes are read as one 8- or 16-byte word");
    constexpr uint16_t kKept = 0x8000, kNew = 0x4000, kSlot = 0x0FFF;
    __shared__ DevSys s;
    __shared__ uint64_t tdet[TILE * W];          // main slice at [0, nm), spawned slice at [nm, nm + ns)
    __shared__ __align__(16) uint16_t msrc[TILE];  // per merged position: its slot
    __shared__ __align__(16) uint16_t pcode[TILE]; // per merged position: kKept | kNew | slot
    uint16_t *const osrc = msrc;                     // per output of the tile: kNew | slot (after the groups)
    __shared__ SegAcc s_tail;
    __shared__ uint32_t s_tile, s_base, s_nnew;
    extern __shared__ int64_t dyn[];
    DevState *st = b.state;
    const uint2 prior = *reinterpret_cast<const uint2 *>(&st->n_merged_keep);
    if (mode == 1 && (int64_t)prior.y <= b.cap) return;
    stage_sys(s, b.sys);
    __syncthreads();
    // the exact-diagonal tables: staged in shared memory, or read through L1
    const bool fx_staged = b.fx_smem_bytes != 0;
    const FxTabs tb = fx_staged ? stage_fx(s, dyn) : fx_tabs(s);
    int64_t *tpop = dyn + (fx_staged ? fx_table_words(s.kind, s.nbasis, s.norb) : 0);
    uint64_t *tflag = reinterpret_cast<uint64_t *>(tpop + (size_t)TILE * R);
    const bool initiator = b.sflag != nullptr;
    const bool real = s.real_amplitudes != 0;
    const int64_t N = st->n_main, S = st->n_spawn, L = N + S;
    const int64_t ntiles = (L + TILE - 1) / TILE;
    const uint64_t iter = (uint64_t)st->iter;
    const uint32_t epoch = os_epoch(*b.seg_epoch, mode);
    const SortedSpawns<W, RANK> sp{keys, idx, b.sdets};
    const uint64_t *mdets = b.dets[cur];
    const int64_t *mpops = b.pops[cur];
    const double *mkii = b.kii[cur];
    uint64_t *odets = b.dets[1 - cur];
    int64_t *opops = b.pops[1 - cur];
    double *okii = b.kii[1 - cur];
    auto tile_det = [&](int k) {
        Det<W> x;
#pragma unroll
        for (int w = 0; w < W; w++) x.w[w] = tdet[k * W + w];
        return x;
    };
    int64_t ap0 = 0, ap1 = 0;
    // accumulate_bloom_stats (src/bloom_handler.F90:104-145) over the spawned
    // list: every entry is one spawning event (its amount in one space), an event
    // of at least kBloomThreshold particles is a bloom; counted here, where the
    // amounts are read anyway, rather than in the spawning kernel's hot loop
    const int64_t bthr = kBloomThreshold * s.real_factor;
    int64_t bn = 0, btot = 0, bmax = 0;
    // (the deterministic projection's entries of combined semi-stochastic
    // annihilation, at and past n_spawn_stoch, are not spawning events)
    const int64_t nstoch = st->n_spawn_stoch;
    auto bloom_add = [&](const int64_t p[2], int64_t e) {
        const int64_t a = (p[0] < 0 ? -p[0] : p[0]) + (p[1] < 0 ? -p[1] : p[1]);
        if (mode == 0 && a >= bthr && e < nstoch) {
            bn++;
            btot += a;
            bmax = a > bmax ? a : bmax;
        }
    };
    __syncthreads();
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->ann_ticket[mode], 1u);
        __syncthreads();
        const int64_t t = s_tile;
        if (t >= ntiles) break;
        const int64_t ia = b.msplit[3 * t + 0], ja = b.msplit[3 * t + 2];
        const int64_t ib = b.msplit[3 * t + 3], jb = b.msplit[3 * t + 4], jc = b.msplit[3 * t + 5];
        int nm = 0, ns = 0;
        if (ja <= jb && ia <= ib && (ib - ia) + (jb - ja) <= TILE) {
            nm = (int)(ib - ia);
            ns = (int)(jb - ja);
        } else if (ja <= jb) {
            // cannot happen for cuts on one merge path; never index past the tile
            if (threadIdx.x == 0) atomicOr(&st->error_flags, HGPU_FLAG_INTERNAL);
        }
        const int n = nm + ns;
        const int64_t ntail = n > 0 ? jc - jb : 0;
        // stage the slices: determinants, populations, flag words
        {
            uint32_t e[PER];
#pragma unroll
            for (int r = 0; r < PER; r++) {
                const int k = threadIdx.x + r * kBlock;
                e[r] = (k >= nm && k < n) ? sp.at(ja + (k - nm)) : 0u;
            }
#pragma unroll
            for (int r = 0; r < PER; r++) {
                const int k = threadIdx.x + r * kBlock;
                if (k >= n) continue;
                Det<W> d;
                int64_t p[2] = {0, 0};
                uint64_t fl = 0;
                if (k < nm) {
                    d = load_det<W>(mdets, ia + k);
#pragma unroll
                    for (int q = 0; q < 2; q++)
                        if (q < R) p[q] = mpops[(ia + k) * R + q];
                } else {
                    d = RANK ? load_det<W>(b.sdets, e[r]) : load_det<W>(keys, ja + (k - nm));
#pragma unroll
                    for (int q = 0; q < 2; q++)
                        if (q < R) p[q] = b.spops[(int64_t)e[r] * R + q];
                    if (initiator) fl = b.sflag[e[r]];
                    bloom_add(p, e[r]);
                }
#pragma unroll
                for (int w = 0; w < W; w++) tdet[k * W + w] = d.w[w];
#pragma unroll
                for (int q = 0; q < 2; q++)
                    if (q < R) tpop[k * R + q] = p[q];
                if (initiator) tflag[k] = fl;
            }
        }
        if (ntail > 0 && threadIdx.x < 32) {
            // spawned entries past the tile's last element and equal to it
            SegAcc a;
            a.init();
            for (int64_t j = jb + threadIdx.x; j < jc; j += 32) {
                const uint32_t e = sp.at(j);
                int64_t p[2] = {0, 0};
#pragma unroll
                for (int q = 0; q < 2; q++)
                    if (q < R) p[q] = b.spops[(int64_t)e * R + q];
                a.add(R, initiator, p, initiator ? b.sflag[e] : 0);
                bloom_add(p, e);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) a.merge(shfl_down_acc(a, off));
            if (threadIdx.x == 0) s_tail = a;
        }
        __syncthreads();
        // merge walk: the slot of every merged position
        {
            const int p0 = threadIdx.x * PER;
            if (p0 < n) {
                int lo = p0 - ns > 0 ? p0 - ns : 0, hi = p0 < nm ? p0 : nm;
                while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (!det_less<W>(tile_det(nm + p0 - 1 - mid), tile_det(mid))) lo = mid + 1;
                    else hi = mid;
                }
                int a = lo, bb = p0 - lo;
                const int plen = n - p0 < PER ? n - p0 : PER;
                for (int q = 0; q < plen; q++) {
                    const bool take_main = a < nm && (bb >= ns || !det_less<W>(tile_det(nm + bb), tile_det(a)));
                    msrc[p0 + q] = take_main ? (uint16_t)a : (uint16_t)(nm + bb);
                    if (take_main) a++;
                    else bb++;
                }
            }
        }
        __syncthreads();
        // groups: summed, combined and rounded at their heads
        uint32_t uniq = 0;
#pragma unroll 1
        for (int k = threadIdx.x; k < n; k += kBlock) {
            const int slot = msrc[k];
            const Det<W> d = tile_det(slot);
            // a group starts at the tile's first position or at a new determinant
            const bool head = k == 0 || !det_eq<W>(tile_det(msrc[k - 1]), d);
            bool cand = false;
            uint16_t code = 0;
            int64_t p[2] = {0, 0};
            uint32_t purpose = P_ROUND_MAIN;
            int64_t key = 0;
            const bool is_main = slot < nm;
            bool determ = false;
            if (head) {
                SegAcc acc;
                acc.init();
                int j = k + 1;
                bool has = false;
                for (; j < n; j++) {
                    const int m = msrc[j];
                    if (!det_eq<W>(tile_det(m), d)) break;
                    int64_t q2[2] = {tpop[m * R], R > 1 ? tpop[m * R + 1] : 0};
                    acc.add(R, initiator, q2, initiator ? tflag[m] : 0);
                    has = true;
                }
                if (!is_main) {
                    int64_t q2[2] = {tpop[slot * R], R > 1 ? tpop[slot * R + 1] : 0};
                    acc.add(R, initiator, q2, initiator ? tflag[slot] : 0);
                    has = true;
                }
                if (j == n && ntail > 0) {
                    // the last group continues past the tile
                    acc.merge(s_tail);
                    has = true;
                }
                const bool nonzero = has && acc.any(R);
                uniq += nonzero ? 1u : 0u;
                const uint64_t fl = nonzero ? acc.flag(R, initiator) : 0;
                if (is_main) {
                    // annihilate_main_list[_initiator], then remove_unoccupied_dets
                    // (a deterministic state is neither rounded nor removed)
                    determ = b.nd > 0 && (b.pinfo[ia + slot] & kDetermBit) != 0;
                    p[0] = tpop[slot * R];
                    p[1] = R > 1 ? tpop[slot * R + 1] : 0;
                    if (nonzero) {
#pragma unroll
                        for (int r = 0; r < 2; r++)
                            if (r < R) {
                                if (!initiator || p[r] != 0) p[r] += acc.sum[r];
                                else if (!((fl >> r) & 1)) p[r] = acc.sum[r];
                            }
                    }
                    cand = true;
                    key = ia + slot;
                } else if (nonzero && mode == 0) {
                    // a new determinant: the initiator rule, round_low_population_spawns
                    p[0] = acc.sum[0];
                    p[1] = acc.sum[1];
                    bool discard = false;
                    if (initiator) {
                        discard = true;
#pragma unroll
                        for (int r = 0; r < 2; r++)
                            if (r < R) {
                                if ((fl >> r) & 1) p[r] = 0;
                                else discard = false;
                            }
                    }
                    cand = !discard;
                    purpose = P_ROUND_SPAWN;
                    key = ja + (slot - nm);
                }
            }
            // one rounding call for both kinds, so that the lanes that round run together
            if (cand && real && !determ) round_pops(s, p, R, purpose, key, iter);
            if (cand) {
                const bool nz = p[0] != 0 || (R > 1 && p[1] != 0);
                if (nz || determ || (!is_main && !real)) {
#pragma unroll
                    for (int r = 0; r < 2; r++)
                        if (r < R) tpop[slot * R + r] = p[r];
                    code = (uint16_t)(kKept | (is_main ? 0 : kNew) | slot);
                }
            }
            pcode[k] = code;
        }
        __syncthreads();
        // compaction: each thread counts its PER consecutive positions
        uint32_t codes[PER / 2];
        if constexpr (PER == 8) {
            const uint4 v = reinterpret_cast<const uint4 *>(pcode)[threadIdx.x];
            codes[0] = v.x;
            codes[1] = v.y;
            codes[2] = v.z;
            codes[3] = v.w;
        } else {
            const uint2 v = reinterpret_cast<const uint2 *>(pcode)[threadIdx.x];
            codes[0] = v.x;
            codes[1] = v.y;
        }
        uint32_t kept = 0, kept_main = 0;
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const uint32_t c = (codes[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
            const bool in = threadIdx.x * PER + q < n;
            kept += (in && (c & kKept)) ? 1u : 0u;
            kept_main += (in && (c & kKept) && !(c & kNew)) ? 1u : 0u;
        }
        // output offsets: kept | kept main << 21 | groups with a non-zero spawned sum << 42
        const uint64_t packed = (uint64_t)kept | ((uint64_t)kept_main << 21) | ((uint64_t)uniq << 42);
        uint64_t ptot;
        const uint64_t pex = block_exclusive_scan<uint64_t>(packed, &ptot);
        const uint32_t tkept = (uint32_t)(ptot & 0x1FFFFF);
        if (threadIdx.x == 0) {
            s_base = tile_lookback(b.seg_status, t, epoch, tkept, st);
            if (mode == 0) {
                unsigned int *nk = reinterpret_cast<unsigned int *>(&st->n_merged_keep);
                atomicAdd(nk, (unsigned int)((ptot >> 21) & 0x1FFFFF));
                atomicAdd(nk + 1, tkept);
                atomicAdd((unsigned long long *)&st->n_uniq, (unsigned long long)(ptot >> 42));
            }
        }
        {
            int o = (int)(pex & 0x1FFFFF);
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const uint32_t c = (codes[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
                if (threadIdx.x * PER + q < n && (c & kKept)) osrc[o++] = (uint16_t)(c & (kNew | kSlot));
            }
        }
        __syncthreads();
        // the survivors in merged order, coalesced, K_ii copied for the kept
        // main entries; the new determinants' outputs listed (in pcode, free
        // after the compaction) for their K_ii below
        const int64_t base = s_base;
        if (threadIdx.x == 0) s_nnew = 0;
        __syncthreads();
        uint16_t *newo = pcode;
        for (int o = threadIdx.x; o < (int)tkept; o += kBlock) {
            const uint16_t v = osrc[o];
            const int slot = v & kSlot;
            const Det<W> d = tile_det(slot);
            const int64_t p0v = tpop[slot * R], p1v = R > 1 ? tpop[slot * R + 1] : 0;
            const int64_t dst = base + o;
            const bool fresh = (v & kNew) != 0 && dst < b.cap;
            const uint32_t nb = __ballot_sync(__activemask(), fresh);
            if (fresh) {
                const int leader = __ffs(nb) - 1;
                uint32_t at = 0;
                if ((threadIdx.x & 31) == leader) at = atomicAdd(&s_nnew, (uint32_t)__popc(nb));
                at = __shfl_sync(nb, at, leader);
                newo[at + __popc(nb & lanemask_lt())] = (uint16_t)o;
            }
            if (dst < b.cap) {
                store_det<W>(odets, dst, d);
                opops[dst * R] = p0v;
                if (R > 1) opops[dst * R + 1] = p1v;
                if (!(v & kNew)) okii[dst] = mkii[ia + slot];
                ap0 += p0v < 0 ? -p0v : p0v;
                ap1 += p1v < 0 ? -p1v : p1v;
            }
        }
        __syncthreads();
        // K_ii of the new determinants (insert_new_walker, src/annihilation.f90:855),
        // consecutive threads on consecutive new determinants, so that every lane
        // of a warp runs the same pair sums
        const int nnew = (int)s_nnew;
        for (int k = threadIdx.x; k < nnew; k += kBlock) {
            const int o = newo[k];
            okii[base + o] = kii_of<W>(s, tile_det(osrc[o] & kSlot), tb);
        }
        __syncthreads();
    }
    const int64_t r0 = block_reduce_sum<int64_t>(ap0);
    const int64_t r1 = block_reduce_sum<int64_t>(ap1);
    const int64_t rbn = block_reduce_sum<int64_t>(bn);
    const int64_t rbt = block_reduce_sum<int64_t>(btot);
    if (threadIdx.x == 0) {
        b.part_i[blockIdx.x * 4 + 0] = r0;
        b.part_i[blockIdx.x * 4 + 1] = r1;
        if (rbn) {
            atomicAdd((unsigned long long *)&st->bloom_n, (unsigned long long)rbn);
            atomicAdd((unsigned long long *)&st->bloom_tot, (unsigned long long)rbt);
        }
    }
    if (bmax) atomicMax((unsigned long long *)&st->bloom_max, (unsigned long long)bmax);
}

// Dynamic shared memory of k_annihilate.
__host__ __forceinline__ size_t ann_smem_bytes(size_t fx_bytes, int R, bool initiator, int tile) {
    return fx_bytes + sizeof(int64_t) * (size_t)tile * (R + (initiator ? 1 : 0));
}

template <int W>
static void annihilation_w(const DevBuffers &b, int R, int cur, cudaStream_t st, const PhaseMarks *pm = nullptr) {
    DevState *S = b.state;
    k_clamp_spawns<<<1, 1, 0, st>>>(S, b.scap);
    // radix sort (hgpu_sort.cuh): pass 0 reads the ranks, or the spawned list itself
    const int rows = b.binom_rows, cols = b.binom_cols;
    const size_t hist_smem = sizeof(uint32_t) * kMaxPasses * kRadix +
                             (b.use_rank ? sizeof(uint64_t) * (size_t)rows * cols : 0);
    const int kw = b.key_words == 2 ? 2 : 1;
    // twice the streaming grid: the rank computation is latency-bound at four
    // blocks per SM (the 64-orbital sort phase is 1.6 % shorter with eight)
    const int hist_grid = 2 * b.grid;
    if (b.sort_packed == 1 && kw == 1) k_sort_hist<W, 1, true, 1><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    else if (b.sort_packed == 2 && kw == 1) k_sort_hist<W, 1, true, 2><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    else if (b.sort_packed == 2) k_sort_hist<W, 2, true, 2><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    else if (b.use_rank && kw == 2) k_sort_hist<W, 2, true, 0><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    else if (b.use_rank) k_sort_hist<W, 1, true, 0><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    else k_sort_hist<W, W, false, 0><<<hist_grid, kBlock, hist_smem, st>>>(b, rows, cols);
    k_sort_offsets<<<1, kRadix, 0, st>>>(b);
    const uint64_t *kin = b.use_rank ? b.skeys : b.sdets;
    const uint32_t *iin = nullptr;
    int o = 0;
    if (b.sort_packed) {
        // packed records: the pass reads records of 16 bytes while the remaining
        // key and the index need two words, then of 8; the last pass writes the
        // index alone
        const int ib = b.sort_ibits;
        const void *in = b.skeys;
        for (int p = 0; p < b.sort_passes; p++) {
            const bool in128 = b.sort_key_bits - kRadixBits * p + ib > 64;
            const bool last = p == b.sort_passes - 1;
            const bool out128 = !last && b.sort_key_bits - kRadixBits * (p + 1) + ib > 64;
            void *out = last ? (void *)b.idx[o] : (void *)b.keys[o];
            if (in128) {
                const P128 *ip = static_cast<const P128 *>(in);
                const size_t sm = PKConf<P128>::smem;
                if (last) k_onesweep_pk<P128, uint32_t><<<b.sort_grid, kOSThreads, sm, st>>>(b, p, ip, (uint32_t *)out, ib);
                else if (out128) k_onesweep_pk<P128, P128><<<b.sort_grid, kOSThreads, sm, st>>>(b, p, ip, (P128 *)out, ib);
                else k_onesweep_pk<P128, P64><<<b.sort_grid, kOSThreads, sm, st>>>(b, p, ip, (P64 *)out, ib);
            } else {
                const P64 *ip = static_cast<const P64 *>(in);
                const size_t sm = PKConf<P64>::smem;
                if (last) k_onesweep_pk<P64, uint32_t><<<b.sort_grid, kOSThreads, sm, st>>>(b, p, ip, (uint32_t *)out, ib);
                else k_onesweep_pk<P64, P64><<<b.sort_grid, kOSThreads, sm, st>>>(b, p, ip, (P64 *)out, ib);
            }
            in = out;
            if (last) iin = b.idx[o];
            o ^= 1;
        }
        kin = nullptr;  // the annihilation reads the determinants through the indices
    }
    for (int p = 0; p < (b.sort_packed ? 0 : b.sort_passes); p++) {
        if (b.key32)
            k_onesweep<uint32_t, 1><<<b.sort_grid, kOSThreads, OSConf<uint32_t, 1>::smem, st>>>(
                b, p, reinterpret_cast<const uint32_t *>(kin), iin, reinterpret_cast<uint32_t *>(b.keys[o]),
                b.idx[o]);
        else if (b.key_words == 1)
            k_onesweep<uint64_t, 1><<<b.sort_grid, kOSThreads, OSConf<uint64_t, 1>::smem, st>>>(
                b, p, kin, iin, b.keys[o], b.idx[o]);
        else
            k_onesweep<uint64_t, 2><<<b.sort_grid, kOSThreads, OSConf<uint64_t, 2>::smem, st>>>(
                b, p, kin, iin, b.keys[o], b.idx[o]);
        kin = b.keys[o];
        iin = b.idx[o];
        o ^= 1;
    }
    if (pm) cudaEventRecord(pm->ev[4], st);
    // merge-path cuts at group boundaries, then one pass over the merged
    // sequence; the second pass runs only after an overflow of the main list
    const size_t ann_smem = ann_smem_bytes(b.fx_smem_bytes, R, b.sflag != nullptr, ann_tile<W>());
    if (b.use_rank) {
        k_ann_splits<W, true><<<b.splits_grid, kBlock, 0, st>>>(b, cur, kin, iin);
        if (pm) cudaEventRecord(pm->ev[5], st);
        for (int mode = 0; mode < 2; mode++)
            k_annihilate<W, true><<<b.grid, kBlock, ann_smem, st>>>(b, R, cur, kin, iin, mode);
    } else {
        k_ann_splits<W, false><<<b.splits_grid, kBlock, 0, st>>>(b, cur, kin, iin);
        if (pm) cudaEventRecord(pm->ev[5], st);
        for (int mode = 0; mode < 2; mode++)
            k_annihilate<W, false><<<b.grid, kBlock, ann_smem, st>>>(b, R, cur, kin, iin, mode);
    }
    if (pm) cudaEventRecord(pm->ev[6], st);
}

void launch_sort_annihilate(const DevBuffers &b, int W, int R, int cur, cudaStream_t st, const PhaseMarks *pm) {
    if (W == 1) annihilation_w<1>(b, R, cur, st, pm);
    else annihilation_w<2>(b, R, cur, st, pm);
}

int set_annihilate_attributes(const DevBuffers &b) {
    if (cudaFuncSetAttribute(k_onesweep_pk<P128, uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PKConf<P128>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep_pk<P128, P128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PKConf<P128>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep_pk<P128, P64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PKConf<P128>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep_pk<P64, uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PKConf<P64>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep_pk<P64, P64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PKConf<P64>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep<uint32_t, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)OSConf<uint32_t, 1>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep<uint64_t, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)OSConf<uint64_t, 1>::smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_onesweep<uint64_t, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)OSConf<uint64_t, 2>::smem) != cudaSuccess)
        return 1;
    // The largest staged table (32 KB; larger ones are read from global memory)
    // with two spaces and initiator flags, so that handles of different systems
    // in one process never lower the limit another handle's captured graph
    // relies on.
    const int fx_max = 32768;
    if (b.fx_smem_bytes > (size_t)fx_max) return 1;
    const int max_bytes = (int)ann_smem_bytes((size_t)fx_max, 2, true, ann_tile<1>());
    const void *fns[4] = {(const void *)k_annihilate<1, true>, (const void *)k_annihilate<1, false>,
                          (const void *)k_annihilate<2, true>, (const void *)k_annihilate<2, false>};
    for (const void *f : fns)
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, max_bytes) != cudaSuccess) return 1;
    return 0;
}

}  // namespace hgpu
