// hgpu_rdm.cu -- replica sampling of the two-body reduced density matrix
// (src/replica_rdm.F90) on the device.
//
// With density_matrices, every allowed spawning attempt of replica s also
// draws spawn_rdm's unweighted amount (src/spawning.F90:664-671) and records
// (parent, child, amount) (create_spawned_particle_replica_rdm).  After the
// annihilation of each cycle, update_rdm_from_spawns (src/replica_rdm.F90:84-159)
// adds, for every recorded pair whose child is occupied, N_child^(other
// replica) x amount / 2 to the RDM elements of the excitation child -> parent,
// and every occupied determinant adds N^(1) N^(2) to its diagonal pairs.  The
// reference first sums equal (parent, child) entries; the sum is linear, so
// here every entry is added on its own (atomic FP64 additions: the RDM agrees
// with the reference's to rounding).  At a report's end calc_rdm_energy
// (src/replica_rdm.F90:215-264) contracts the RDM with the integrals: one block
// per row, rows summed in a fixed order.
#include "hgpu_common.cuh"

namespace hgpu {

// tri_ind_distinct_reorder (lib/local/utils.F90:579-611), 0-based orbitals and index.
__device__ __forceinline__ int64_t tri_pair(int p, int q) {
    const int64_t hi = p > q ? p : q, lo = p > q ? q : p;
    return hi * (hi - 1) / 2 + lo;
}

// orbs_from_index (lib/local/utils.F90:613-628), 0-based: pair ind -> p < q.
__device__ __forceinline__ void orbs_of_pair(int64_t ind, int &p, int &q) {
    const int64_t i1 = ind + 1;
    int qq = (int)(1.50 + sqrt((double)(2 * i1) - 1.750));
    while ((int64_t)qq * (qq - 1) / 2 < i1) qq++;
    while ((int64_t)(qq - 1) * (qq - 2) / 2 >= i1) qq--;
    p = (int)(i1 - (int64_t)(qq - 1) * (qq - 2) / 2) - 1;
    q = qq - 1;
}

// Open-addressing hash table of the new main list (index per slot, linear
// probing), so that each RDM spawn finds its child with about two memory
// accesses instead of a binary search of the whole list.  The index needs the
// low bits of a slot (the fewest that hold the list's capacity); the bits above
// it hold a tag from the high word of the determinant's hash, so that a probe
// loads a determinant only when the tags agree (three tag bits at a capacity of
// 3e8 skip 7 in 8 of the loads that would not match).  Probe sequences are
// bounded by the table size; a full sweep (impossible below a load of one)
// raises HGPU_FLAG_INTERNAL.
constexpr uint32_t kHashEmpty = 0xFFFFFFFFu;

template <int W>
__device__ __forceinline__ uint64_t det_hash(const Det<W> &f) {
    uint64_t x = 0x9E3779B97F4A7C15ull;
#pragma unroll
    for (int w = 0; w < W; w++) x = (x ^ f.w[w]) * 0xBF58476D1CE4E5B9ull;
    // murmur3 finaliser
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return x;
}

__global__ void __launch_bounds__(kBlock) k_rdm_hash_clear(DevBuffers b) {
    if (!b.state->rdm_on) return;
    uint4 *t = reinterpret_cast<uint4 *>(b.rdm_hash);
    const int64_t n = (b.rdm_hash_mask + 1) / 4;
    const uint4 e = make_uint4(kHashEmpty, kHashEmpty, kHashEmpty, kHashEmpty);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        t[k] = e;
}

template <int W>
__global__ void __launch_bounds__(kBlock) k_rdm_hash_insert(DevBuffers b, int cur) {
    DevState *st = b.state;
    if (!st->rdm_on) return;
    const int64_t N = st->n_main;
    const uint64_t *dets = b.dets[cur];
    const uint64_t mask = (uint64_t)b.rdm_hash_mask;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t hx = det_hash<W>(load_det<W>(dets, i));
        const uint32_t entry = ((uint32_t)(hx >> 32) & b.rdm_hash_tagmask) | (uint32_t)i;
        uint64_t h = hx & mask;
        uint64_t probes = 0;
        while (atomicCAS(&b.rdm_hash[h], kHashEmpty, entry) != kHashEmpty) {
            h = (h + 1) & mask;
            if (++probes > mask) {
                atomicOr(&st->error_flags, HGPU_FLAG_INTERNAL);
                break;
            }
        }
    }
}

// The cycle's RDM spawns against the new main list (buffer cur).  A double
// adds one element; a single adds one per other occupied orbital of the child,
// done by the warp's lanes together (lane l tests orbitals l, l + 32, ...) for
// each single of the warp in turn, so that the few singles among a warp's
// spawns do not hold the others through their loops.
template <int W>
__global__ void __launch_bounds__(kBlock) k_rdm_spawns(DevBuffers b, int R, int cur) {
    DevState *st = b.state;
    if (!st->rdm_on) return;
    const int64_t n = st->n_rdm < b.scap ? st->n_rdm : b.scap;
    const uint64_t *dets = b.dets[cur];
    const int64_t *pops = b.pops[cur];
    const int nel = b.sys->nel;
    const int64_t np = b.npairs;
    const double inv_rf = 1.0 / (double)b.sys->real_factor;  // exact: a power of two
    const uint64_t mask = (uint64_t)b.rdm_hash_mask;
    const uint32_t tagmask = b.rdm_hash_tagmask;
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t k = base + lane;
        bool single = false;
        double matel = 0.0;
        int p = 0, q = 0;
        Det<W> fc;
#pragma unroll
        for (int w = 0; w < W; w++) fc.w[w] = 0;
        if (k < n) {
            // the parent from the cycle's old main list (buffer 1 - cur, unchanged by
            // the annihilation, which wrote the new list into buffer cur)
            const Det<W> fp = load_det<W>(b.dets[1 - cur], b.rdm_sparent[k]);
            fc = load_det<W>(b.rdm_schild, k);
            const uint64_t hx = det_hash<W>(fc);
            const uint32_t tag = (uint32_t)(hx >> 32) & tagmask;
            uint64_t h = hx & mask;
            int64_t pos = -1;
            for (uint64_t probes = 0; probes <= mask; probes++) {
                const uint32_t v = b.rdm_hash[h];
                if (v == kHashEmpty) break;
                if ((v & tagmask) == tag && det_eq<W>(load_det<W>(dets, v & ~tagmask), fc)) {
                    pos = v & ~tagmask;
                    break;
                }
                h = (h + 1) & mask;
            }
            if (pos >= 0) {
                const int s = b.rdm_sspace[k];
                // pops(other replica, child) / real_factor x amount / real_factor / 2
                const double pop1 = (double)pops[pos * R + (1 - s)] * inv_rf;
                const double pop2 = (double)b.rdm_spops[k] * inv_rf;
                matel = pop1 * pop2 / 2.0;
                // update_rdm (src/replica_rdm.F90:12-82) for the child and its parent
                const Excit e = get_excitation<W>(fc, fp, nel);
                if (e.perm) matel = -matel;
                if (e.nexcit == 2) {
                    atomicAdd(&b.rdm[tri_pair(e.to[0], e.to[1]) * np + tri_pair(e.from[0], e.from[1])], matel);
                } else if (e.nexcit == 1) {
                    single = true;
                    p = e.to[0];
                    q = e.from[0];
                }
            }
        }
        for (uint32_t m = __ballot_sync(FULL_MASK, single); m; m &= m - 1) {
            const int src = __ffs(m) - 1;
            Det<W> g;
#pragma unroll
            for (int w = 0; w < W; w++) g.w[w] = __shfl_sync(FULL_MASK, fc.w[w], src);
            const double v = __shfl_sync(FULL_MASK, matel, src);
            const int pp = __shfl_sync(FULL_MASK, p, src), qq = __shfl_sync(FULL_MASK, q, src);
#pragma unroll
            for (int c = 0; c < 2 * W; c++) {
                const int orb = 32 * c + lane;
                if (((g.w[c >> 1] >> (orb & 63)) & 1ull) == 0 || orb == qq) continue;
                if (orb < pp && orb < qq) atomicAdd(&b.rdm[tri_pair(orb, pp) * np + tri_pair(orb, qq)], v);
                else if (orb > pp && orb > qq) atomicAdd(&b.rdm[tri_pair(orb, pp) * np + tri_pair(qq, orb)], v);
                else atomicAdd(&b.rdm[tri_pair(pp, orb) * np + tri_pair(orb, qq)], -v);
            }
        }
    }
}

// The diagonal: N^(1) N^(2) of every occupied determinant on each of its
// occupied pairs, summed per block in shared memory.  A warp loads 32
// determinants and runs those occupied in both spaces one after the other,
// its lanes on the determinant's pairs: lane l holds the l-th occupied orbital,
// and pair k of the pair table (x, y), x < y, is added by lane k mod 32 from
// the orbitals of lanes x and y -- the same work for every determinant, so
// the lanes stay busy whatever mix of determinants a warp meets.  Up to 32
// electrons (a table of at most 496 pairs); more take one determinant per lane.
constexpr int kDiagMaxPairs = 32 * 31 / 2;

template <int W>
__global__ void __launch_bounds__(kBlock) k_rdm_diag(DevBuffers b, int R, int cur) {
    extern __shared__ double dsm[];  // [npairs]
    __shared__ uint16_t ptab[kDiagMaxPairs];  // x | y << 8
    const DevState *st = b.state;
    if (!st->rdm_on) return;
    const int64_t np = b.npairs;
    const int nel = b.sys->nel;
    const int nep = nel * (nel - 1) / 2;
    for (int64_t k = threadIdx.x; k < np; k += blockDim.x) dsm[k] = 0.0;
    if (nel <= 32)
        for (int k = threadIdx.x; k < nep; k += blockDim.x) {
            int y = 1;
            while ((y + 1) * y / 2 <= k) y++;
            ptab[k] = (uint16_t)((k - y * (y - 1) / 2) | (y << 8));
        }
    __syncthreads();
    const int64_t N = st->n_main;
    const uint64_t *dets = b.dets[cur];
    const int64_t *pops = b.pops[cur];
    const double inv_rf = 1.0 / (double)b.sys->real_factor;
    const int lane = threadIdx.x & 31;
    if (nel <= 32) {
        const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
        for (int64_t base = warp * 32; base < N; base += nwarps * 32) {
            const int64_t i = base + lane;
            int64_t p0 = 0, p1 = 0;
            Det<W> f;
#pragma unroll
            for (int w = 0; w < W; w++) f.w[w] = 0;
            if (i < N) {
                p0 = pops[i * R];
                p1 = pops[i * R + 1];
                f = load_det<W>(dets, i);
            }
            const double matel = (double)p0 * inv_rf * ((double)p1 * inv_rf) / 1.0;
            for (uint32_t m = __ballot_sync(FULL_MASK, p0 != 0 && p1 != 0); m; m &= m - 1) {
                const int src = __ffs(m) - 1;
                Det<W> g;
#pragma unroll
                for (int w = 0; w < W; w++) g.w[w] = __shfl_sync(FULL_MASK, f.w[w], src);
                const double v = __shfl_sync(FULL_MASK, matel, src);
                const int occ = lane < nel ? select_det<W>(g.w, lane) : 0;
                for (int k0 = 0; k0 < nep; k0 += 32) {
                    const int k = k0 + lane;
                    const uint16_t xy = k < nep ? ptab[k] : 0;
                    const int a = __shfl_sync(FULL_MASK, occ, xy & 0xFF), c = __shfl_sync(FULL_MASK, occ, xy >> 8);
                    if (k < nep) atomicAdd(&dsm[tri_pair(c, a)], v);
                }
            }
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
            const int64_t p0 = pops[i * R], p1 = pops[i * R + 1];
            if (p0 == 0 || p1 == 0) continue;
            const double matel = (double)p0 * inv_rf * ((double)p1 * inv_rf) / 1.0;
            const Det<W> f = load_det<W>(dets, i);
#pragma unroll
            for (int wx = 0; wx < W; wx++) {
                for (uint64_t x = f.w[wx]; x; x &= x - 1) {
                    const int px = 64 * wx + __ffsll((long long)x) - 1;
                    for (uint64_t y = x & (x - 1); y; y &= y - 1)
                        atomicAdd(&dsm[tri_pair(64 * wx + __ffsll((long long)y) - 1, px)], matel);
#pragma unroll
                    for (int wy = wx + 1; wy < W; wy++)
                        for (uint64_t y = f.w[wy]; y; y &= y - 1)
                            atomicAdd(&dsm[tri_pair(64 * wy + __ffsll((long long)y) - 1, px)], matel);
                }
            }
        }
    }
    __syncthreads();
    for (int64_t k = threadIdx.x; k < np; k += blockDim.x)
        if (dsm[k] != 0.0) atomicAdd(&b.rdm[k * np + k], dsm[k]);
}

// get_two_e_int_mol (src/hamiltonian_molecular.f90:579-597): <ij||ab> with the
// spin and symmetry checks of get_two_body_int_mol.
__device__ __forceinline__ double rdm_two_e(const DevSys &s, int i, int j, int a, int b) {
    const bool sym_ok = ((s.orbsym[i] ^ s.orbsym[j] ^ s.orbsym[a] ^ s.orbsym[b]) & (s.nsym - 1)) == 0;
    double x = 0.0, y = 0.0;
    if (sym_ok && ((i ^ a) & 1) == 0 && ((j ^ b) & 1) == 0) x = Ints<double>::v2(s, i, j, a, b);
    if (sym_ok && ((i ^ b) & 1) == 0 && ((j ^ a) & 1) == 0) y = Ints<double>::v2(s, i, j, b, a);
    return x - y;
}

// get_one_e_int_mol (src/hamiltonian_molecular.f90:599-617).
__device__ __forceinline__ double rdm_one_e(const DevSys &s, int i, int j) {
    if (s.orbsym[i] != s.orbsym[j] || ((i ^ j) & 1) != 0) return 0.0;
    return s.h1[(i >> 1) * s.norb + (j >> 1)];
}

// calc_rdm_energy, one row per block iteration: the row's contribution and
// its diagonal element into rdm_rows.
__global__ void __launch_bounds__(kBlock) k_rdm_rows(DevBuffers b) {
    __shared__ DevSys s;
    __shared__ double red[kBlock];
    stage_sys(s, b.sys);
    __syncthreads();
    if (!b.state->rdm_on) return;
    const int64_t np = b.npairs;
    const double nm1 = (double)(s.nel - 1);
    for (int64_t row = blockIdx.x; row < np; row += gridDim.x) {
        int a, bb;
        orbs_of_pair(row, a, bb);
        double e = 0.0;
        for (int64_t j = threadIdx.x; j < np; j += blockDim.x) {
            const double r = b.rdm[row * np + j];
            if (fabs(r) < 1.0e-12) continue;  // depsilon (lib/local/const.F90)
            int c, d;
            orbs_of_pair(j, c, d);
            e = e + r * rdm_two_e(s, a, bb, c, d);
            if (a == c) e = e + r * rdm_one_e(s, bb, d) / nm1;
            if (bb == d) e = e + r * rdm_one_e(s, a, c) / nm1;
            if (a == d) e = e - r * rdm_one_e(s, bb, c) / nm1;
            if (bb == c) e = e - r * rdm_one_e(s, a, d) / nm1;
        }
        red[threadIdx.x] = e;
        __syncthreads();
        for (int w = kBlock / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] = red[threadIdx.x] + red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            b.rdm_rows[row] = red[0];
            b.rdm_rows[np + row] = b.rdm[row * np + row];
        }
        __syncthreads();
    }
}

// The rows' sums in a fixed order: energy and trace (src/replica_rdm.F90:250-262).
__global__ void __launch_bounds__(1024) k_rdm_final(DevBuffers b) {
    __shared__ double re[1024], rt[1024];
    DevState *st = b.state;
    if (!st->rdm_on) return;
    const int64_t np = b.npairs;
    double e = 0.0, t = 0.0;
    for (int64_t k = threadIdx.x; k < np; k += blockDim.x) {
        e = e + b.rdm_rows[k];
        t = t + b.rdm_rows[np + k];
    }
    re[threadIdx.x] = e;
    rt[threadIdx.x] = t;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            re[threadIdx.x] = re[threadIdx.x] + re[threadIdx.x + w];
            rt[threadIdx.x] = rt[threadIdx.x] + rt[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const DevSys *s = b.sys;
        double energy = re[0] * (double)s->nel * (double)(s->nel - 1) * 0.5;
        energy = energy + (s->ecore - s->H00) * rt[0];
        st->rdm_energy = energy;
        st->rdm_trace = rt[0];
    }
}

// The diagonal (every occupied determinant) does not depend on the RDM spawns:
// it runs on the second stream while the hash table is built and the spawns
// are added (both only add into the RDM), joined before the cycle ends.  Half
// the streaming grid (two blocks per SM, one wave) leaves room on every SM for
// the spawns' blocks: 4.5 % shorter cycles on the 64-orbital replica list than
// with the full grid (three resident blocks per SM and a second wave), and
// 6 % shorter than with a third of it.
void launch_rdm_cycle(const DevBuffers &b, int W, int R, int cur, cudaStream_t st) {
    const size_t dsm = sizeof(double) * (size_t)b.npairs;
    const int dgrid = (b.grid + 1) / 2;
    cudaEventRecord(b.rdm_fork, st);
    cudaStreamWaitEvent(b.rdm_aux, b.rdm_fork, 0);
    if (W == 1) k_rdm_diag<1><<<dgrid, kBlock, dsm, b.rdm_aux>>>(b, R, cur);
    else k_rdm_diag<2><<<dgrid, kBlock, dsm, b.rdm_aux>>>(b, R, cur);
    cudaEventRecord(b.rdm_join, b.rdm_aux);
    k_rdm_hash_clear<<<b.grid, kBlock, 0, st>>>(b);
    if (W == 1) {
        k_rdm_hash_insert<1><<<b.grid, kBlock, 0, st>>>(b, cur);
        k_rdm_spawns<1><<<b.grid, kBlock, 0, st>>>(b, R, cur);
    } else {
        k_rdm_hash_insert<2><<<b.grid, kBlock, 0, st>>>(b, cur);
        k_rdm_spawns<2><<<b.grid, kBlock, 0, st>>>(b, R, cur);
    }
    cudaStreamWaitEvent(st, b.rdm_join, 0);
}

void launch_rdm_energy(const DevBuffers &b, int W, cudaStream_t st) {
    (void)W;
    const int rows = (int)(b.npairs < 4 * kMaxBlocks ? b.npairs : 4 * kMaxBlocks);
    k_rdm_rows<<<rows > 0 ? rows : 1, kBlock, 0, st>>>(b);
    k_rdm_final<<<1, 1024, 0, st>>>(b);
}

int set_rdm_attributes() {
    // 128 spin orbitals: 8128 pairs
    const int max_bytes = (int)sizeof(double) * (128 * 127 / 2);
    if (cudaFuncSetAttribute(k_rdm_diag<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_bytes) != cudaSuccess ||
        cudaFuncSetAttribute(k_rdm_diag<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_bytes) != cudaSuccess)
        return 1;
    return 0;
}

}  // namespace hgpu
