// hgpu_fixed.h -- exact fixed-point accumulation of diagonal matrix elements.
//
// <D|H|D> (slater_condon0, src/hamiltonian_molecular.f90:73-139 and
// src/hamiltonian_hub_k.f90:91-132) is a sum of O(nel^2) integrals.  The engine
// accumulates the same terms exactly, as signed 128-bit integers in units of
// 2^-96 (each term rounded once to that grid, ties to even), and rounds the
// total once to double.  The result is the correctly rounded exact sum of the
// terms; summing left to right in FP64 (as the reference does) differs from it
// by at most a few ulps.  Integer accumulation runs on the integer pipes, which
// on this GPU have 64x the throughput of the FP64 pipe, and its result does not
// depend on the summation order.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define HGPU_HD __host__ __device__ __forceinline__
#else
#define HGPU_HD inline
#endif

namespace hgpu {

typedef __int128 fx128;
typedef unsigned __int128 ufx128;

constexpr int kFxShift = 96;

HGPU_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

HGPU_HD int clz128(ufx128 u) {
    uint64_t hi = (uint64_t)(u >> 64);
    if (hi) return clz64(hi);
    return 64 + clz64((uint64_t)u);
}

// round(x * 2^96) to the nearest integer, ties to even; |x| < 2^31.
inline fx128 fx_from_double(double x) {
    if (x == 0.0) return 0;
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    bool neg = bits >> 63;
    int e = (int)((bits >> 52) & 0x7FF);
    uint64_t m = bits & ((1ull << 52) - 1);
    if (e == 0) {
        e = 1;  // subnormal
    } else {
        m |= 1ull << 52;
    }
    // x = m * 2^(e - 1075); x * 2^96 = m * 2^(e - 979)
    int sh = e - 1075 + kFxShift;
    ufx128 v;
    if (sh >= 0) {
        v = (ufx128)m << sh;
    } else {
        int s = -sh;
        if (s > 64) {
            v = 0;  // below 2^-96 / 2: rounds to zero
            if (s == 65 && m > (1ull << 63)) v = 1;  // unreachable for m < 2^53
        } else {
            uint64_t q = s == 64 ? 0 : (m >> s);
            uint64_t rem = s == 64 ? m : (m & ((1ull << s) - 1));
            uint64_t half = 1ull << (s - 1);
            if (rem > half || (rem == half && (q & 1))) q++;
            v = q;
        }
    }
    return neg ? -(fx128)v : (fx128)v;
}

// Nearest double to v * 2^-96 (ties to even).
HGPU_HD double fx_to_double(fx128 v) {
    if (v == 0) return 0.0;
    bool neg = v < 0;
    ufx128 u = neg ? (ufx128)(-v) : (ufx128)v;
    int msb = 127 - clz128(u);
    uint64_t m;
    int sh;  // value = m * 2^(sh - 96), m in [2^52, 2^53)
    if (msb <= 52) {
        m = (uint64_t)u << (52 - msb);
        sh = msb - 52;
    } else {
        int s = msb - 52;
        ufx128 q = u >> s;
        ufx128 rem = u & (((ufx128)1 << s) - 1);
        ufx128 half = (ufx128)1 << (s - 1);
        if (rem > half || (rem == half && (q & 1))) q++;
        if (q == ((ufx128)1 << 53)) {
            q >>= 1;
            s++;
        }
        m = (uint64_t)q;
        sh = s;
    }
    int exp2 = sh - kFxShift + 52;  // unbiased exponent of the result
    uint64_t bits = ((uint64_t)(exp2 + 1023) << 52) | (m & ((1ull << 52) - 1));
    if (neg) bits |= 1ull << 63;
    double d;
#if defined(__CUDA_ARCH__)
    d = __longlong_as_double((long long)bits);
#else
    std::memcpy(&d, &bits, 8);
#endif
    return d;
}

}  // namespace hgpu
