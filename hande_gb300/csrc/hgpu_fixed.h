// hgpu_fixed.h -- exact fixed-point accumulation of diagonal matrix elements.
//
// <D|H|D> (slater_condon0, src/hamiltonian_molecular.f90:73-139 and
// src/hamiltonian_hub_k.f90:91-132) is a sum of O(nel^2) integrals.  The engine
// rounds each term once to the grid 2^-s (ties to even) and accumulates the
// terms exactly in 64-bit integers; the total is rounded once to double.  The
// scale s is fixed per system so that the sum of the magnitudes of every term
// that can occur, B, satisfies 2 B 2^s < 2^62: no determinant's sum, nor the
// difference of two, can overflow.  The result does not depend on the order of
// the terms; summing left to right in FP64, as the reference does, differs from
// it by a few ulps.  The integer pipes that do the work have 64x the throughput
// of this GPU's FP64 pipe.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define HGPU_HD __host__ __device__ __forceinline__
#else
#define HGPU_HD inline
#endif

namespace hgpu {

// Scale exponent from the exact integer bound B = sum of ceil(|term|).
inline int fx_scale_for_bound(int64_t B) {
    int bits = 0;
    while (bits < 63 && (B >> bits) != 0) bits++;
    int s = 61 - bits;
    if (s > 60) s = 60;
    if (s < 0) s = 0;
    return s;
}

inline int64_t fx_ceil_abs(double x) { return (int64_t)std::ceil(std::fabs(x)); }

// round(x * 2^s), ties to even (the default rounding mode of rint).
inline int64_t fx_from_double(double x, int s) { return (int64_t)std::rint(std::ldexp(x, s)); }

// Nearest double to v * 2^-s: one rounding (int64 -> double), then an exact
// scaling by a power of two.
HGPU_HD double fx_to_double(int64_t v, double inv_scale) {
#if defined(__CUDA_ARCH__)
    return __ll2double_rn((long long)v) * inv_scale;
#else
    return (double)v * inv_scale;
#endif
}

}  // namespace hgpu
