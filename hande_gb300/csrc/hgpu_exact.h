// hgpu_exact.h -- integer forms of FP64 expressions of the spawning path.
//
// GB300 executes two FP64 operations per clock per SM, and the generators are
// full of small FP64 expressions on a uniform u = k 2^-53 (k < 2^53): int(u*n),
// u < p, the fractional part of p_spawn.  Each function here returns exactly
// what IEEE-754 binary64 arithmetic with round-to-nearest-even returns for the
// expression it names (the argument is given with it), computed on the integer
// pipes instead.  tests/test_exact_forms.py checks them against the FP64
// expressions on the host.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define HGPU_XD __host__ __device__ __forceinline__
#else
#define HGPU_XD inline
#endif

namespace hgpu {

HGPU_XD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

HGPU_XD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// RN(P) to 53 significant bits, ties to even, returned as q * 2^e (q <= 2^53).
HGPU_XD uint64_t rn53(uint64_t P, int &e) {
    if (P < (1ull << 53)) {
        e = 0;
        return P;
    }
    int sh = 11 - clz64(P);  // bits beyond 53 (1..11)
    uint64_t q = P >> sh, r = P & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (r > half || (r == half && (q & 1))) q++;
    e = sh;
    return q;
}

// (int)(u * n) for u = k 2^-53 and an integer n < 2^11 (also (int)(n * u)).
HGPU_XD int floor_un(uint64_t k, uint32_t n) {
    int e;
    uint64_t q = rn53(k * n, e);  // RN(u n) = q 2^(e-53)
    return (int)(q >> (53 - e));
}

// (int)(u * a * b / 2.0) for u = k 2^-53 and integers a, b < 2^11, evaluated
// left to right (choose_ij_mol's index, src/excit_gen_mol.f90:641).
HGPU_XD int floor_uab_half(uint64_t k, uint32_t a, uint32_t b) {
    int e1, e2;
    uint64_t q1 = rn53(k * a, e1);   // RN(u a) = q1 2^(e1-53)
    uint64_t q2 = rn53(q1 * b, e2);  // RN(RN(u a) b) = q2 2^(e1+e2-53)
    return (int)(q2 >> (54 - e1 - e2));
}

// (int)(u * a * b) for u = k 2^-53 and integers a, b < 2^11, left to right.
HGPU_XD int floor_uab(uint64_t k, uint32_t a, uint32_t b) {
    int e1, e2;
    uint64_t q1 = rn53(k * a, e1);
    uint64_t q2 = rn53(q1 * b, e2);
    return (int)(q2 >> (53 - e1 - e2));
}

// u < p for u = k 2^-53, with t = ceil(p 2^53) precomputed (0 <= p <= 1).
HGPU_XD bool u_less(uint64_t k, uint64_t t) { return k < t; }

// x > 0.0 for a double given by its bits (x not NaN).
HGPU_XD bool positive(uint64_t xb) { return (int64_t)xb > 0; }

// a < b for doubles given by their bits, both >= +0 and not NaN.
HGPU_XD bool less_nonneg(uint64_t ab, uint64_t bb) { return ab < bb; }

// The large-amplitude branch of stochastic_round_spawned_particle
// (src/stoch_utils.f90:87-136) for pspawn >= 0 finite, pspawn < 2^63:
//   n = (int64)pspawn; if (pspawn - (double)n > u) n = n + 1,  u = k 2^-53.
HGPU_XD int64_t round_up_frac(uint64_t pb, uint64_t k) {
    int expf = (int)((pb >> 52) & 0x7FF);
    uint64_t m = pb & ((1ull << 52) - 1);
    int E;
    if (expf == 0) {
        E = -1022;
    } else {
        E = expf - 1023;
        m |= 1ull << 52;
    }
    // pspawn = m 2^(E-52)
    if (E >= 52) return (int64_t)(m << (E - 52));  // no fraction: 0 > u is false
    if (E >= 0) {
        int64_t n = (int64_t)(m >> (52 - E));
        uint64_t frac = m & ((1ull << (52 - E)) - 1);  // fraction = frac 2^(E-52)
        return (frac << (E + 1)) > k ? n + 1 : n;      // frac 2^(E-52) > k 2^-53
    }
    // 0 <= pspawn < 1: n = 0 and the fraction is pspawn: m 2^(E-52) > k 2^-53
    int t = -E - 1;  // >= 0:  m > k 2^t
    bool up;
    if (t >= 64) up = k == 0 && m > 0;
    else if (t > 0 && (k >> (64 - t)) != 0) up = false;
    else up = m > (k << t);
    return up ? 1 : 0;
}

}  // namespace hgpu
