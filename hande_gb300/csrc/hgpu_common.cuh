// hgpu_common.cuh -- device helpers shared by the kernels of a cycle: warp
// and block scans and reductions, staging of the system in shared memory,
// determinant loads and stores, stochastic rounding.
#pragma once

#include "hgpu_kernels.cuh"

namespace hgpu {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint2 operator+(uint2 a, uint2 b) { return make_uint2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ uint2 operator-(uint2 a, uint2 b) { return make_uint2(a.x - b.x, a.y - b.y); }

template <typename T>
__device__ __forceinline__ T zero_of();
template <>
__device__ __forceinline__ int64_t zero_of<int64_t>() { return 0; }
template <>
__device__ __forceinline__ uint2 zero_of<uint2>() { return make_uint2(0, 0); }
template <>
__device__ __forceinline__ uint32_t zero_of<uint32_t>() { return 0u; }
template <>
__device__ __forceinline__ uint64_t zero_of<uint64_t>() { return 0ull; }

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int d);
template <>
__device__ __forceinline__ int64_t shfl_up<int64_t>(int64_t v, int d) {
    return __shfl_up_sync(FULL_MASK, (long long)v, d);
}
template <>
__device__ __forceinline__ uint32_t shfl_up<uint32_t>(uint32_t v, int d) {
    return __shfl_up_sync(FULL_MASK, v, d);
}
template <>
__device__ __forceinline__ uint64_t shfl_up<uint64_t>(uint64_t v, int d) {
    return __shfl_up_sync(FULL_MASK, (unsigned long long)v, d);
}
template <>
__device__ __forceinline__ uint2 shfl_up<uint2>(uint2 v, int d) {
    return make_uint2(__shfl_up_sync(FULL_MASK, v.x, d), __shfl_up_sync(FULL_MASK, v.y, d));
}

// Inclusive warp scan, then block scan through shared memory.  Returns the
// exclusive prefix of v within the block and the block total in *tot.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *tot) {
    __shared__ T wsum[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T y = shfl_up<T>(x, d);
        if (lane >= d) x = x + y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int nw = blockDim.x >> 5;
    if (warp == 0) {
        T w = lane < nw ? wsum[lane] : zero_of<T>();
        T s = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T y = shfl_up<T>(s, d);
            if (lane >= d) s = s + y;
        }
        if (lane < nw) wsum[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    T before = warp > 0 ? wsum[warp - 1] : zero_of<T>();
    *tot = wsum[nw - 1];
    __syncthreads();
    // exclusive = inclusive - v
    return before + x - v;
}

__device__ __forceinline__ double shfl_down_any(double v, int d) { return __shfl_down_sync(FULL_MASK, v, d); }
__device__ __forceinline__ uint32_t shfl_down_any(uint32_t v, int d) { return __shfl_down_sync(FULL_MASK, v, d); }
__device__ __forceinline__ int64_t shfl_down_any(int64_t v, int d) {
    return (int64_t)__shfl_down_sync(FULL_MASK, (long long)v, d);
}

template <typename T>
__device__ __forceinline__ T block_reduce_sum(T v) {
    __shared__ T red[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += shfl_down_any(v, d);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    T r = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < nw; k++) r += red[k];
    __syncthreads();
    return r;  // valid in thread 0
}

__device__ __forceinline__ void chunk_range(int64_t n, int64_t &begin, int64_t &end) {
    int64_t G = gridDim.x;
    int64_t chunk = (n + G - 1) / G;
    chunk = (chunk + 255) & ~(int64_t)255;
    begin = (int64_t)blockIdx.x * chunk;
    end = begin + chunk < n ? begin + chunk : n;
    if (begin > n) begin = n;
}

// ---------------------------------------------------------------------------
// Shared-memory staging of the system
// ---------------------------------------------------------------------------
__device__ __forceinline__ void stage_sys(DevSys &dst, const DevSys *src) {
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (int k = threadIdx.x; k < (int)(sizeof(DevSys) / 4); k += blockDim.x) d[k] = s[k];
}

__device__ __forceinline__ HubTables stage_hub(const DevSys *src, uint8_t *smem) {
    HubTables t;
    int nk = src->nk;
    t.nk = nk;
    if (src->kind == HGPU_SYS_HUB_K) {
        for (int k = threadIdx.x; k < nk * nk; k += blockDim.x) smem[k] = src->sym_table[k];
        for (int k = threadIdx.x; k < nk; k += blockDim.x) smem[nk * nk + k] = src->inv_sym[k];
    }
    t.sym = smem;
    t.inv = smem + nk * nk;
    return t;
}

template <int W>
__device__ __forceinline__ Det<W> load_det(const uint64_t *p, int64_t i) {
    Det<W> d;
#pragma unroll
    for (int k = 0; k < W; k++) d.w[k] = p[i * W + k];
    return d;
}

template <int W>
__device__ __forceinline__ void store_det(uint64_t *p, int64_t i, const Det<W> &d) {
#pragma unroll
    for (int k = 0; k < W; k++) p[i * W + k] = d.w[k];
}

// first index in [0, n) whose determinant is not less than x
template <int W>
__device__ __forceinline__ int64_t lower_bound_det(const uint64_t *list, int64_t n, const Det<W> &x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        Det<W> m = load_det<W>(list, mid);
        if (det_less<W>(m, x)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Sign helpers and stochastic rounding of the annihilation
// ---------------------------------------------------------------------------
__device__ __forceinline__ int sgn3(int64_t x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }
__device__ __forceinline__ int sgn1(int64_t x) { return x >= 0 ? 1 : -1; }
// Fortran sign(1, int(x)): int() keeps the low 32 bits of an int64.
__device__ __forceinline__ int sign1_int32(int64_t x) { return (int32_t)(uint32_t)(uint64_t)x >= 0 ? 1 : -1; }

// stochastic_round_int_64 (src/stoch_utils.f90:51-85) of one entry's pops.
__device__ __forceinline__ void round_pops(const DevSys &s, int64_t *p, int R, uint32_t purpose, int64_t idx,
                                           uint64_t iter) {
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (q >= R) break;
        int64_t v = p[q];
        int64_t av = v < 0 ? -v : v;
        if (av < s.real_factor && v != 0) {
            RStream rs;
            rs.init(s.seed, purpose, q, idx, 0, iter);
            // (double)av > u * real_factor with real_factor = 2^31 and u = k 2^-53,
            // both sides exact: av * 2^22 > k in integers
            uint64_t k = rs.next_k();
            p[q] = (((uint64_t)av << 22) > k) ? isign64(s.real_factor, v) : 0;
        }
    }
}

}  // namespace hgpu
