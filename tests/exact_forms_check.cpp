// Checks the integer forms of hande_gb300/csrc/hgpu_exact.h against the FP64
// expressions they stand for, on random and boundary inputs.  Built and run by
// tests/test_exact_forms.py; prints the number of mismatches and exits 1 if any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include "../hande_gb300/csrc/hgpu_exact.h"

using namespace hgpu;

static double udbl(uint64_t k) { return (double)k * 0x1p-53; }  // exact: k < 2^53

int main(int argc, char **argv) {
    long n = argc > 1 ? atol(argv[1]) : 2000000;
    std::mt19937_64 g(12345);
    long bad = 0;
    auto randk = [&](int mode) -> uint64_t {
        uint64_t k = g() >> 11;
        if (mode == 1) k = g() & 0xFF;                   // tiny u
        if (mode == 2) k = (1ull << 53) - 1 - (g() & 0xFF);  // u just below 1
        return k;
    };
    for (long it = 0; it < n; it++) {
        uint64_t k = randk((int)(it % 7 == 0) + (int)(it % 11 == 0));
        double u = udbl(k);
        uint32_t a = 1 + (uint32_t)(g() % 200), b = 1 + (uint32_t)(g() % 200);
        // int(u * n)
        if ((int)(u * (double)a) != floor_un(k, a)) bad++;
        if ((int)((double)a * u) != floor_un(k, a)) bad++;
        // int(u * a * b / 2.0) and int(u * a * b)
        if ((int)(u * (double)a * (double)b / 2.0) != floor_uab_half(k, a, b)) bad++;
        if ((int)(u * (double)a * (double)b) != floor_uab(k, a, b)) bad++;
        // u < p
        double p = (double)(g() >> 11) * 0x1p-53;
        if (it % 5 == 0) p = udbl(k);                 // equality boundary
        if (it % 13 == 0) p = std::nextafter(udbl(k), 1.0);
        uint64_t t = (uint64_t)std::ceil(std::ldexp(p, 53));
        if ((u < p) != u_less(k, t)) bad++;
        // stochastic rounding, large branch
        double ps;
        switch (it % 6) {
            case 0: ps = std::ldexp((double)(g() >> 11), -(int)(g() % 60)); break;  // wide range incl. < 1
            case 1: ps = (double)(g() % 100000) + udbl(g() >> 11); break;
            case 2: ps = udbl(k); break;                                          // fraction equal to u
            case 3: ps = std::ldexp(1.0, -(int)(g() % 1100)); break;                // tiny, subnormal
            case 4: ps = (double)(g() >> 20); break;                                 // integers
            default: ps = std::ldexp((double)(g() >> 11), (int)(g() % 10)); break;  // up to 2^62
        }
        int64_t ref = (int64_t)ps;
        if (ps - (double)ref > u) ref = ref + 1;
        if (ref != round_up_frac(dbits(ps), k)) bad++;
        // sign and order tests
        double x = std::ldexp((double)(int64_t)(g() >> 12) - (double)(1ll << 51), -(int)(g() % 40));
        if ((x > 0.0) != positive(dbits(x))) bad++;
        double y = std::fabs(x), z = std::fabs(std::ldexp((double)(g() >> 11), -(int)(g() % 40)));
        if ((y < z) != less_nonneg(dbits(y), dbits(z))) bad++;
    }
    std::printf("%ld mismatches in %ld cases\n", bad, n);
    return bad ? 1 : 0;
}
