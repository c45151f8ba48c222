// Cube root built only from correctly rounded IEEE-754 double operations
// (add, multiply, divide, explicit fma), so a CPU build without FMA
// contraction and a GPU build compiled with --fmad=false produce the same
// bits. Used by the LULESH_FP64_EXACT path for the hourglass coefficient
// (reference lulesh.cc:1068, which calls libm cbrt).
//
// Method: split x = m * 2^(3k) with m in [1, 8) by exponent arithmetic,
// start from a least-squares quadratic fit of m^(1/3) on [1, 8] (max
// relative error 4.7e-2), refine with four Halley steps
// y <- y (y^3 + 2m) / (2 y^3 + m) (cubic convergence), finish with one
// Newton step whose residual y^3 - m is formed from error-free products, and
// rescale by 2^k exactly. tests/test_host.py checks the result against libm.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LULESH_HD __host__ __device__
#else
#define LULESH_HD
#endif

namespace lulesh {

LULESH_HD inline double bits_to_double(uint64_t b) {
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
}

LULESH_HD inline uint64_t double_to_bits(double d) {
    uint64_t b;
    memcpy(&b, &d, sizeof b);
    return b;
}

LULESH_HD inline double cbrt_portable(double x) {
    if (!(x > 0.0)) {
        if (x < 0.0) return -cbrt_portable(-x);
        return x;  // +-0 and NaN
    }
    uint64_t bits = double_to_bits(x);
    int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0x7ff) return x;  // inf
    if (ex == 0) {
        // subnormal: scale by 2^54 (exact), take the root, scale by 2^-18
        return cbrt_portable(x * 18014398509481984.0) * 3.814697265625e-06;
    }
    int e = ex - 1023;
    int k = (e >= 0) ? e / 3 : -((2 - e) / 3);  // floor(e / 3)
    int r = e - 3 * k;                           // 0, 1 or 2
    double m = bits_to_double((bits & 0x000fffffffffffffULL) | ((uint64_t)(1023 + r) << 52));
    double y = 0.8209 + m * (0.2374 - m * 0.01159);
    for (int it = 0; it < 4; ++it) {
        double y3 = y * y * y;
        y = y * (y3 + 2.0 * m) / (2.0 * y3 + m);
    }
    // Newton step y - (y^3 - m) / (3 y^2) with the residual y^3 - m formed
    // from error-free products (t + e1 = y^2, u + e2 = t y) and u - m exact
    // (Sterbenz), so the last rounding dominates the error.
    const double t = y * y;
    const double e1 = fma(y, y, -t);
    const double u = t * y;
    const double e2 = fma(t, y, -u);
    const double res = (u - m) + (e2 + e1 * y);
    y = y - res / (3.0 * t);
    return y * bits_to_double((uint64_t)(1023 + k) << 52);
}

}  // namespace lulesh
