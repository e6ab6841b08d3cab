// hgpu_sort.cuh -- stable LSD radix sort of the spawned list.
//
// HANDE sorts the spawned list by determinant (qsort, src/sort.f90:213-395,
// called from annihilate_wrapper_spawn_t_single, src/spawn_data.F90:359-421)
// before summing repeated determinants.  Here the sort key of a determinant is
// its colexicographic rank, sum_k C(p_k, k) over its occupied orbitals p_1 <
// ... < p_nel (the combinatorial number system): a bijection onto
// [0, C(nbasis, nel)) that orders determinants exactly as HANDE's comparison
// does (unsigned, last word most significant), in ceil(log2 C(nbasis, nel))
// bits instead of nbasis -- 34 instead of 52 bits for 52 spin orbitals and 10
// electrons.  Systems whose rank does not fit 64 bits sort the raw words.
//
// One pass per 8-bit digit.  Digit histograms of all passes are counted in one
// read of the list (k_sort_hist); each pass (k_onesweep) then ranks a tile of
// keys in shared memory and finds the tile's global offsets by decoupled
// look-back over the preceding tiles (Merrill and Garland, "Single-pass
// parallel prefix scan with decoupled look-back", 2016; Adinets and Merrill,
// "Onesweep", 2022), so a pass reads and writes each key once.  Tiles are taken
// in ticket order, so a tile only ever waits on tiles that running blocks
// hold; every wait is bounded and a timeout raises HGPU_FLAG_TIMEOUT.
#pragma once

namespace hgpu {

constexpr int kSpinLimit = 1 << 22;  // polls of one look-back wait before it gives up
constexpr int kOSLook = 8;           // predecessor tiles read per look-back round trip

// look-back status word: [63:62] flag, [61:32] epoch of the pass, [31:0] count
constexpr uint64_t kOSAggregate = 1, kOSPrefix = 2;
__device__ __forceinline__ uint64_t os_word(uint64_t flag, uint32_t epoch, uint32_t count) {
    return (flag << 62) | ((uint64_t)(epoch & 0x3FFFFFFFu) << 32) | count;
}

// Epoch of pass p of the current sort: never 0, so zeroed memory is never valid.
__device__ __forceinline__ uint32_t os_epoch(uint32_t base, int pass) {
    return (uint32_t)((base + (uint32_t)pass) % 0x3FFFFFFFu) + 1u;
}

template <int KW>
__device__ __forceinline__ uint32_t os_digit(const uint64_t *k, int shift) {
    return (uint32_t)((k[shift >> 6] >> (shift & 63)) & (kRadix - 1));
}
template <int KW>
__device__ __forceinline__ uint32_t os_digit(const uint32_t *k, int shift) {
    return (k[shift >> 5] >> (shift & 31)) & (kRadix - 1);
}

// Packed records of the rank sort.  A record holds the key bits that earlier
// passes have not consumed, shifted down so that the digit of the next pass is
// its lowest byte, and the entry's index in the top `ib` bits: one 64-bit word
// (P64) or two (P128, low word first).  k_sort_hist writes the first records
// (rank and index); a pass ranks the lowest byte and writes the record shifted
// by one digit -- the consumed bits are not moved again -- or, after the last
// pass, the index alone.  The host picks P64 once the remaining key and the
// index fit one word, so later passes move 8 bytes per entry instead of 16.
struct P64 {
    uint64_t v;
};
struct P128 {
    uint64_t lo, hi;
};
__device__ __forceinline__ uint32_t pk_digit(const P64 &r) { return (uint32_t)r.v & (kRadix - 1); }
__device__ __forceinline__ uint32_t pk_digit(const P128 &r) { return (uint32_t)r.lo & (kRadix - 1); }
__device__ __forceinline__ void pk_out(const P64 &r, int ib, uint32_t &o) { o = (uint32_t)(r.v >> (64 - ib)); }
__device__ __forceinline__ void pk_out(const P128 &r, int ib, uint32_t &o) { o = (uint32_t)(r.hi >> (64 - ib)); }
__device__ __forceinline__ void pk_out(const P64 &r, int ib, P64 &o) {
    const uint64_t km = ~0ull >> ib;  // key bits of the word
    o.v = ((r.v & km) >> kRadixBits) | (r.v & ~km);
}
__device__ __forceinline__ void pk_out(const P128 &r, int ib, P128 &o) {
    const uint64_t km = ~0ull >> ib;
    const uint64_t hk = r.hi & km;
    o.lo = (r.lo >> kRadixBits) | (hk << (64 - kRadixBits));
    o.hi = (hk >> kRadixBits) | (r.hi & ~km);
}
// the remaining key fits below the index (the host's choice of P64)
__device__ __forceinline__ void pk_out(const P128 &r, int ib, P64 &o) {
    const uint64_t km = ~0ull >> ib;
    o.v = (r.lo >> kRadixBits) | ((r.hi & km) << (64 - kRadixBits)) | (r.hi & ~km);
}

// Lanes of `mask` whose 8-bit digit equals this lane's: one ballot per digit
// bit (cheaper on this GPU than match.any).
__device__ __forceinline__ uint32_t warp_peers8(uint32_t mask, uint32_t d) {
    uint32_t peers = mask;
#pragma unroll
    for (int bit = 0; bit < kRadixBits; bit++) {
        uint32_t bb = __ballot_sync(mask, (d >> bit) & 1u);
        peers &= ((d >> bit) & 1u) ? bb : ~bb;
    }
    return peers;
}

// Spin-resolved rank of a determinant among those with na alpha (even) and nb
// beta (odd) spin orbitals: the number of such determinants below it in the
// list order (unsigned, last word most significant).  A smaller determinant
// agrees above some occupied spin orbital p, leaves p empty and places below p
// the ka alpha and kb beta electrons that the determinant holds at or below p:
// C(alpha orbitals below p, ka) C(beta orbitals below p, kb) ways, summed over
// p.  mode 1: tab[(ka (nb + 1) + kb) * cols + p] holds that product; mode 2:
// tab[k * cols + n] = C(n, k).  A determinant with other electron counts sets
// bad (its key is then 0).  det_rank128: mode 2 with 128-bit products and sum,
// for ranks above 64 bits (two key words, low word first).
template <int W>
__device__ __forceinline__ uint64_t det_rank(const Det<W> &f, const uint64_t *tab, int cols, int mode, int na,
                                             int nb, bool &bad) {
    int ca = 0, cb = 0;
#pragma unroll
    for (int w = 0; w < W; w++) {
        ca += __popcll(f.w[w] & 0x5555555555555555ull);
        cb += __popcll(f.w[w] & 0xAAAAAAAAAAAAAAAAull);
    }
    if (ca != na || cb != nb) {
        bad = true;
        return 0;
    }
    uint64_t r = 0;
    if (mode == 1) {
        // row (ka, kb) of the product table, advanced by one alpha or one beta row per electron
        const uint64_t *row = tab;
        const int sa = (nb + 1) * cols, sb = cols;
#pragma unroll
        for (int h = 0; h < 2 * W; h++) {
            uint32_t x = (uint32_t)(f.w[h >> 1] >> (32 * (h & 1)));
            while (x) {
                const int p = 32 * h + __ffs((int)x) - 1;
                x &= x - 1;
                row += (p & 1) ? sb : sa;
                r += row[p];
            }
        }
        return r;
    }
    int ka = 0, kb = 0;
#pragma unroll
    for (int w = 0; w < W; w++) {
        uint64_t x = f.w[w];
        while (x) {
            const int p = 64 * w + __ffsll((long long)x) - 1;
            x &= x - 1;
            if (p & 1) kb++;
            else ka++;
            r += tab[ka * cols + ((p + 1) >> 1)] * tab[kb * cols + (p >> 1)];
        }
    }
    return r;
}

template <int W>
__device__ __forceinline__ unsigned __int128 det_rank128(const Det<W> &f, const uint64_t *tab, int cols, int na,
                                                         int nb, bool &bad) {
    int ca = 0, cb = 0;
#pragma unroll
    for (int w = 0; w < W; w++) {
        ca += __popcll(f.w[w] & 0x5555555555555555ull);
        cb += __popcll(f.w[w] & 0xAAAAAAAAAAAAAAAAull);
    }
    if (ca != na || cb != nb) {
        bad = true;
        return 0;
    }
    unsigned __int128 r = 0;
    int ka = 0, kb = 0;
#pragma unroll
    for (int w = 0; w < W; w++) {
        uint64_t x = f.w[w];
        while (x) {
            const int p = 64 * w + __ffsll((long long)x) - 1;
            x &= x - 1;
            if (p & 1) kb++;
            else ka++;
            r += (unsigned __int128)tab[ka * cols + ((p + 1) >> 1)] * tab[kb * cols + (p >> 1)];
        }
    }
    return r;
}

// Sort keys of the spawned list (ranks into b.skeys, when ranks are used) and
// the digit histograms of every pass, added into b.ghist[pass][digit].
// PACK 1 / 2: the ranks are written as P64 / P128 records with the index i.
template <int W, int KW, bool RANK, int PACK>
__global__ void __launch_bounds__(kBlock) k_sort_hist(DevBuffers b, int rows, int cols) {
    extern __shared__ uint64_t hist_smem[];
    uint32_t *h = reinterpret_cast<uint32_t *>(hist_smem);  // [passes][kRadix]
    uint64_t *binom = hist_smem + (kMaxPasses * kRadix) / 2;
    const int passes = b.sort_passes;
    for (int k = threadIdx.x; k < passes * kRadix; k += blockDim.x) h[k] = 0;
    if (RANK)
        for (int k = threadIdx.x; k < rows * cols; k += blockDim.x) binom[k] = b.binom[k];
    __syncthreads();
    const int64_t n = b.state->n_spawn;
    bool bad = false;
    // kHistUnroll entries per thread and round, their loads issued together
    // (the loop is otherwise bound by the latency of one load per thread)
    constexpr int kHistUnroll = 4;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += stride * kHistUnroll) {
        Det<W> fs[kHistUnroll];
#pragma unroll
        for (int r = 0; r < kHistUnroll; r++) {
            const int64_t i = i0 + r * stride;
            if (i < n) fs[r] = load_det<W>(b.sdets, i);
        }
#pragma unroll
        for (int r = 0; r < kHistUnroll; r++) {
            const int64_t i = i0 + r * stride;
            if (i >= n) break;
            const Det<W> &f = fs[r];
            uint64_t key[KW];
            if (PACK) {
                uint64_t lo, hi = 0;
                if (KW == 2) {
                    const unsigned __int128 r = det_rank128<W>(f, binom, cols, b.sort_na, b.sort_nb, bad);
                    lo = (uint64_t)r;
                    hi = (uint64_t)(r >> 64);
                } else {
                    lo = det_rank<W>(f, binom, cols, b.use_rank, b.sort_na, b.sort_nb, bad);
                }
                key[0] = lo;
                key[KW - 1] = KW == 2 ? hi : lo;
                const uint64_t ix = (uint64_t)i << (64 - b.sort_ibits);
                if (PACK == 1) {
                    b.skeys[i] = lo | ix;
                } else {
                    b.skeys[2 * i] = lo;
                    b.skeys[2 * i + 1] = hi | ix;
                }
            } else if (RANK && KW == 2) {
                const unsigned __int128 r = det_rank128<W>(f, binom, cols, b.sort_na, b.sort_nb, bad);
                key[0] = (uint64_t)r;
                key[KW - 1] = (uint64_t)(r >> 64);
                b.skeys[2 * i] = key[0];
                b.skeys[2 * i + 1] = key[KW - 1];
            } else if (RANK) {
                key[0] = det_rank<W>(f, binom, cols, b.use_rank, b.sort_na, b.sort_nb, bad);
                if (b.key32) reinterpret_cast<uint32_t *>(b.skeys)[i] = (uint32_t)key[0];
                else b.skeys[i] = key[0];
            } else {
#pragma unroll
                for (int w = 0; w < KW; w++) key[w] = f.w[w];
            }
            // Digits of the top passes take few values (ranks are far below 2^64):
            // those are counted with one ballot per value, the others with plain
            // shared-memory atomics (spread over 256 counters)
            const uint32_t active = __activemask();
            const int lane = threadIdx.x & 31;
            for (int p = 0; p < passes; p++) {
                uint32_t dd = os_digit<KW>(key, p * kRadixBits);
                const int nv = p < b.sort_few_from ? kRadix : b.sort_few_values[p];
                if (nv > 32) {
                    atomicAdd(&h[p * kRadix + dd], 1u);
                } else {
                    for (int v = 0; v < nv; v++) {
                        uint32_t c = __popc(__ballot_sync(active, dd == (uint32_t)v));
                        if (lane == __ffs(active) - 1 && c) atomicAdd(&h[p * kRadix + v], c);
                    }
                }
            }
        }
    }
    if (bad) atomicOr(&b.state->error_flags, HGPU_FLAG_BAD_DET);
    __syncthreads();
    for (int k = threadIdx.x; k < passes * kRadix; k += blockDim.x)
        if (h[k]) atomicAdd(&b.ghist[k], h[k]);
}

// Global digit offsets of every pass; clears the histograms for the next sort,
// the tile tickets and advances the look-back epoch.
__global__ void __launch_bounds__(kRadix) k_sort_offsets(DevBuffers b) {
    const int passes = b.sort_passes;
    for (int p = 0; p < passes; p++) {
        uint32_t c = b.ghist[p * kRadix + threadIdx.x];
        uint32_t tot;
        uint32_t ex = block_exclusive_scan<uint32_t>(c, &tot);
        b.gofs[p * kRadix + threadIdx.x] = ex;
        b.ghist[p * kRadix + threadIdx.x] = 0;
    }
    if (threadIdx.x < kMaxPasses) b.state->os_ticket[threadIdx.x] = 0;
    if (threadIdx.x == 0) *b.os_epoch += (uint32_t)kMaxPasses;
}

// One stable pass on digit `pass`: keys (KW words of type K) and 32-bit
// indices (the identity when idx_in is null).
template <typename K, int KW>
__global__ void __launch_bounds__(kOSThreads, 4) k_onesweep(DevBuffers b, int pass, const K *keys_in,
                                                         const uint32_t *idx_in, K *keys_out, uint32_t *idx_out) {
    constexpr int ITEMS = OSConf<K, KW>::items;
    constexpr int TILE = OSConf<K, KW>::tile;
    constexpr int NW = kOSThreads / 32;
    extern __shared__ uint64_t os_smem[];
    K *skey = reinterpret_cast<K *>(os_smem);                      // [TILE][KW]
    uint32_t *sidx = reinterpret_cast<uint32_t *>(skey + TILE * KW);  // [TILE]
    __shared__ uint32_t wcnt[NW][kRadix];
    __shared__ uint32_t lstart[kRadix], gbase[kRadix];
    __shared__ uint32_t s_tile;
    DevState *st = b.state;
    const int64_t n = st->n_spawn;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    const uint32_t epoch = os_epoch(*b.os_epoch, pass);
    const int shift = pass * kRadixBits;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int d = threadIdx.x;  // digit owned in the look-back
    uint64_t *status = b.lookback;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->os_ticket[pass], 1u);
#pragma unroll
        for (int w = 0; w < NW; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t tile = s_tile;
        if (tile >= ntiles) break;
        const int64_t t0 = tile * TILE;
        K kv[ITEMS][KW];
        uint32_t iv[ITEMS], off[ITEMS], dg[ITEMS];
        // stable ranking: element t0 + (warp*ITEMS + r)*32 + lane
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            int64_t e = t0 + (int64_t)(warp * ITEMS + r) * 32 + lane;
            bool valid = e < n;
            uint32_t mask = __ballot_sync(FULL_MASK, valid);
            dg[r] = 0xFFFFFFFFu;
            if (valid) {
#pragma unroll
                for (int w = 0; w < KW; w++) kv[r][w] = keys_in[e * KW + w];
                iv[r] = idx_in ? idx_in[e] : (uint32_t)e;
                uint32_t dd = os_digit<KW>(kv[r], shift);
                dg[r] = dd;
                uint32_t peers = warp_peers8(mask, dd);
                int leader = __ffs(peers) - 1;
                uint32_t old = 0;
                if (lane == leader) {
                    old = wcnt[warp][dd];
                    wcnt[warp][dd] = old + __popc(peers);
                }
                old = __shfl_sync(mask, old, leader);
                off[r] = old + __popc(peers & lanemask_lt());
            }
            __syncwarp();
        }
        __syncthreads();
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = cnt;
            cnt += c;
        }
        // publish this tile's count of digit d, then look back for its prefix
        volatile uint64_t *my = status + tile * kRadix + d;
        uint32_t excl = 0;
        if (tile == 0) {
            *my = os_word(kOSPrefix, epoch, cnt);
        } else {
            *my = os_word(kOSAggregate, epoch, cnt);
            // walk back kOSLook tiles per round trip: the loads of a round are
            // independent, so a long run of tiles that have only published their
            // aggregates costs one memory latency per kOSLook tiles
            int64_t k = tile - 1;
            int spins = 0;
            bool done = false;
            while (!done) {
                uint64_t v[kOSLook];
#pragma unroll
                for (int u = 0; u < kOSLook; u++)
                    v[u] = k - u >= 0 ? *(volatile uint64_t *)(status + (k - u) * kRadix + d) : 0;
                int u = 0;
                for (; u < kOSLook && k - u >= 0; u++) {
                    uint32_t ve = (uint32_t)(v[u] >> 32) & 0x3FFFFFFFu;
                    uint64_t fl = v[u] >> 62;
                    if (ve != (epoch & 0x3FFFFFFFu) || fl == 0) break;  // not published yet
                    excl += (uint32_t)v[u];
                    if (fl == kOSPrefix) {
                        done = true;
                        break;
                    }
                }
                if (done) break;
                k -= u;  // resume at the first tile that was not ready
                if (u == 0) {
                    if (++spins > kSpinLimit) {
                        atomicOr(&st->error_flags, HGPU_FLAG_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            *my = os_word(kOSPrefix, epoch, excl + cnt);
        }
        gbase[d] = b.gofs[pass * kRadix + d] + excl;
        uint32_t ltot;
        lstart[d] = block_exclusive_scan<uint32_t>(cnt, &ltot);
        __syncthreads();
        // stage in digit order, then write each digit's run contiguously
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (dg[r] != 0xFFFFFFFFu) {
                uint32_t lp = lstart[dg[r]] + wcnt[warp][dg[r]] + off[r];
#pragma unroll
                for (int w = 0; w < KW; w++) skey[lp * KW + w] = kv[r][w];
                sidx[lp] = iv[r];
            }
        }
        __syncthreads();
        const int tn = (int)min((int64_t)TILE, n - t0);
        for (int j = threadIdx.x; j < tn; j += kOSThreads) {
            K k[KW];
#pragma unroll
            for (int w = 0; w < KW; w++) k[w] = skey[j * KW + w];
            uint32_t dd = os_digit<KW>(k, shift);
            int64_t pos = (int64_t)gbase[dd] + (j - (int64_t)lstart[dd]);
            if (pos < n) {
#pragma unroll
                for (int w = 0; w < KW; w++) keys_out[pos * KW + w] = k[w];
                idx_out[pos] = sidx[j];
            }
        }
        __syncthreads();
    }
}

// One stable pass over packed records (see P64 / P128): the digit is the
// record's lowest byte; OUT is the next pass's record or, after the last pass,
// the 32-bit index.  Look-back as in k_onesweep.  Tiles of 48 KB of records
// (24 eight-byte or 12 sixteen-byte records per thread, two blocks per SM at
// up to 128 registers): twice k_onesweep's, which halves the look-backs,
// block scans and barriers per record and gives each digit of a tile twice
// as long a contiguous run to write.  Ranking within a warp: each lane sets
// its bit in a shared word per digit, and the word read back is the set of
// lanes with its digit -- one shared-memory atomic instead of a ballot per
// digit bit (16 % faster passes than tiles of 24 KB ranked by ballots, 21 %
// with this ranking, on the 64-orbital replica lists).
constexpr int kPKMinBlocks = 2;
template <typename IN>
struct PKConf {
    static constexpr int items = sizeof(IN) == 8 ? 24 : 12;
    static constexpr int tile = kOSThreads * items;
    static constexpr size_t smem = (size_t)tile * sizeof(IN);
};

template <typename IN, typename OUT>
__global__ void __launch_bounds__(kOSThreads, kPKMinBlocks) k_onesweep_pk(DevBuffers b, int pass, const IN *recs_in,
                                                                       OUT *recs_out, int ib) {
    constexpr int ITEMS = PKConf<IN>::items;
    constexpr int TILE = PKConf<IN>::tile;
    constexpr int NW = kOSThreads / 32;
    extern __shared__ uint64_t os_smem[];
    IN *srec = reinterpret_cast<IN *>(os_smem);  // [TILE], in digit order
    __shared__ uint32_t wcnt[NW][kRadix];
    __shared__ uint32_t wmatch[NW][kRadix];  // lanes of a warp per digit, zero between items
    __shared__ uint32_t lstart[kRadix], gbase[kRadix];
    __shared__ uint32_t s_tile;
    DevState *st = b.state;
    const int64_t n = st->n_spawn;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    const uint32_t epoch = os_epoch(*b.os_epoch, pass);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int d = threadIdx.x;  // digit owned in the look-back
    uint64_t *status = b.lookback;
#pragma unroll
    for (int w = 0; w < NW; w++) wmatch[w][threadIdx.x] = 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->os_ticket[pass], 1u);
#pragma unroll
        for (int w = 0; w < NW; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t tile = s_tile;
        if (tile >= ntiles) break;
        const int64_t t0 = tile * TILE;
        IN rv[ITEMS];
        uint32_t dgo[ITEMS];  // digit << 16 | rank of the record in its warp and digit
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const int64_t e = t0 + (int64_t)(warp * ITEMS + r) * 32 + lane;
            if (e < n) rv[r] = recs_in[e];
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const int64_t e = t0 + (int64_t)(warp * ITEMS + r) * 32 + lane;
            const bool valid = e < n;
            const uint32_t mask = __ballot_sync(FULL_MASK, valid);
            dgo[r] = 0xFFFFFFFFu;
            // peers of equal digit: every lane sets its bit in its digit's word
            const uint32_t dd = pk_digit(rv[r]);
            if (valid) atomicOr(&wmatch[warp][dd], 1u << lane);
            __syncwarp();
            uint32_t peers = 0;
            if (valid) peers = wmatch[warp][dd];
            __syncwarp();
            if (valid) {
                const int leader = __ffs(peers) - 1;
                uint32_t old = 0;
                if (lane == leader) {
                    old = wcnt[warp][dd];
                    wcnt[warp][dd] = old + __popc(peers);
                    wmatch[warp][dd] = 0;
                }
                old = __shfl_sync(mask, old, leader);
                dgo[r] = (dd << 16) | (old + __popc(peers & lanemask_lt()));
            }
            __syncwarp();
        }
        __syncthreads();
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = cnt;
            cnt += c;
        }
        volatile uint64_t *my = status + tile * kRadix + d;
        uint32_t excl = 0;
        if (tile == 0) {
            *my = os_word(kOSPrefix, epoch, cnt);
        } else {
            *my = os_word(kOSAggregate, epoch, cnt);
            int64_t k = tile - 1;
            int spins = 0;
            bool done = false;
            while (!done) {
                uint64_t v[kOSLook];
#pragma unroll
                for (int u = 0; u < kOSLook; u++)
                    v[u] = k - u >= 0 ? *(volatile uint64_t *)(status + (k - u) * kRadix + d) : 0;
                int u = 0;
                for (; u < kOSLook && k - u >= 0; u++) {
                    const uint32_t ve = (uint32_t)(v[u] >> 32) & 0x3FFFFFFFu;
                    const uint64_t fl = v[u] >> 62;
                    if (ve != (epoch & 0x3FFFFFFFu) || fl == 0) break;  // not published yet
                    excl += (uint32_t)v[u];
                    if (fl == kOSPrefix) {
                        done = true;
                        break;
                    }
                }
                if (done) break;
                k -= u;
                if (u == 0) {
                    if (++spins > kSpinLimit) {
                        atomicOr(&st->error_flags, HGPU_FLAG_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            *my = os_word(kOSPrefix, epoch, excl + cnt);
        }
        gbase[d] = b.gofs[pass * kRadix + d] + excl;
        uint32_t ltot;
        lstart[d] = block_exclusive_scan<uint32_t>(cnt, &ltot);
        __syncthreads();
#pragma unroll
        for (int r = 0; r < ITEMS; r++)
            if (dgo[r] != 0xFFFFFFFFu) {
                const uint32_t dd = dgo[r] >> 16;
                srec[lstart[dd] + wcnt[warp][dd] + (dgo[r] & 0xFFFFu)] = rv[r];
            }
        __syncthreads();
        const int tn = (int)min((int64_t)TILE, n - t0);
        for (int j = threadIdx.x; j < tn; j += kOSThreads) {
            const IN rec = srec[j];
            const uint32_t dd = pk_digit(rec);
            const int64_t pos = (int64_t)gbase[dd] + (j - (int64_t)lstart[dd]);
            if (pos < n) {
                OUT o;
                pk_out(rec, ib, o);
                recs_out[pos] = o;
            }
        }
        __syncthreads();
    }
}

}  // namespace hgpu
