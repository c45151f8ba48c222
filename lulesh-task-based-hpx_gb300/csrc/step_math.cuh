// Element, node and material arithmetic shared by the step kernels.
//
// Every function lives in namespace lulesh::LULESH_VARIANT, so the three
// translation units that include this header (fast double, exact double
// compiled with --fmad=false, mixed) never share an out-of-line copy compiled
// with another contraction setting.
//
// Geometry functions are templated on the real type R (double for the double
// paths, float for the mixed path's temporaries) and keep the reference's
// operand order and parenthesisation (esa-tu-darmstadt/lulesh-task-based-hpx
// lulesh.cc), which is what makes the exact double variant round every
// operation as the reference does.
#pragma once

#include "fp64_emu.cuh"
#include "lulesh_dev.h"
#include "portable_cbrt.h"

#ifndef LULESH_VARIANT
#error "define LULESH_VARIANT"
#endif

namespace lulesh {
namespace LULESH_VARIANT {

#define LD(p) __ldg(p)

// A product for the FP64-bound kernels. Fast variants: double multiplies run
// on the integer pipes (dmul_ipipe, the same bits as a * b), beside the FP64
// pipe's adds and multiply-adds; a product written with pmul is never fused
// into a multiply-add. Exact variant: the plain multiply, rounded on its own
// as there every operation is. Float products stay plain.
#if LULESH_EXACT
__device__ __forceinline__ double pmul(double a, double b) { return a * b; }
#else
__device__ __forceinline__ double pmul(double a, double b) { return dmul_ipipe(a, b); }
#endif
__device__ __forceinline__ float pmul(float a, float b) { return a * b; }

__device__ __forceinline__ void raise_error(StepResult* r, int elem, int phase) {
    if (atomicCAS(&r->err, 0, LULESH_EVOLUME) == 0) {
        r->err_elem = elem;
        r->err_phase = phase;
    }
}

__device__ __forceinline__ void load_nodelist(const int32_t* nodelist, int i, int nl[8]) {
    const int4* p = reinterpret_cast<const int4*>(nodelist + 8 * (size_t)i);
    const int4 a = __ldg(p), b = __ldg(p + 1);
    nl[0] = a.x; nl[1] = a.y; nl[2] = a.z; nl[3] = a.w;
    nl[4] = b.x; nl[5] = b.y; nl[6] = b.z; nl[7] = b.w;
}

__device__ __forceinline__ void gather8(const double* __restrict__ f, const int nl[8], double o[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = LD(f + nl[k]);
}

// --- element geometry -------------------------------------------------------

// TRIPLE_PRODUCT of lulesh.cc:649-651, arguments in the macro's order.
template <class R>
__device__ __forceinline__ R triple(R x1, R y1, R z1, R x2, R y2, R z2, R x3, R y3, R z3) {
#if LULESH_EXACT
    return x1 * (y2 * z3 - z2 * y3) + x2 * (z1 * y3 - y1 * z3) + x3 * (y1 * z2 - z1 * y2);
#else
    // the first product of each pair and of the sum on the integer pipes
    return fma(x3, fma(-z1, y2, pmul(y1, z2)),
               fma(x2, fma(-y1, z3, pmul(z1, y3)), pmul(x1, fma(-z2, y3, pmul(y2, z3)))));
#endif
}

// CalcElemVolume (lulesh.cc:592-665).
template <class R>
__device__ __forceinline__ R hex_volume(const R x[8], const R y[8], const R z[8]) {
    const R twelveth = R(1.0) / R(12.0);
    R dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    R dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    R dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    R dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    R dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    R dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    R dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    R dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    R dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    R dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    R dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    R dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
    R vol = triple(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
            triple(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
            triple(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
    return pmul(vol, twelveth);
}

// Centre Jacobian of CalcElemShapeFunctionDerivatives (lulesh.cc:277-305).
template <class R>
struct Jac {
    R fjxxi, fjxet, fjxze, fjyxi, fjyet, fjyze, fjzxi, fjzet, fjzze;
};

template <class R>
__device__ __forceinline__ Jac<R> jacobian(const R x[8], const R y[8], const R z[8]) {
    const R c = R(.125);
    Jac<R> j;
    j.fjxxi = c * ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    j.fjxet = c * ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    j.fjxze = c * ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    j.fjyxi = c * ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    j.fjyet = c * ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    j.fjyze = c * ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    j.fjzxi = c * ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    j.fjzet = c * ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    j.fjzze = c * ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    return j;
}

// Determinant only (lulesh.cc:308-373 without the B matrix).
template <class R>
__device__ __forceinline__ R jac_det(const Jac<R>& j) {
    const R cjxet = -(j.fjyxi * j.fjzze) + (j.fjzxi * j.fjyze);
    const R cjyet = (j.fjxxi * j.fjzze) - (j.fjzxi * j.fjxze);
    const R cjzet = -(j.fjxxi * j.fjyze) + (j.fjyxi * j.fjxze);
    return R(8.) * (j.fjxet * cjxet + j.fjyet * cjyet + j.fjzet * cjzet);
}

#if !LULESH_EXACT
// Direction sums of one coordinate (or velocity component) v from the four
// body diagonals: d[0], d[1], d[2] along xi, eta, zeta are 8 times the centre
// Jacobian entries fj?xi, fj?et, fj?ze (lulesh.cc:287-305) and 4 times the
// Q-gradient differences d?i, d?j, d?k (lulesh.cc:1341-1349). Linear in v.
template <class R>
__device__ __forceinline__ void dirs(const R v[8], R d[3]) {
    const R d60 = v[6] - v[0], d53 = v[5] - v[3], d71 = v[7] - v[1], d42 = v[4] - v[2];
    const R u = d60 - d42, w = d53 - d71;
    d[0] = u + w;
    d[1] = u - w;
    d[2] = (d60 + d42) + (d53 + d71);
}

// Cofactors c[a][b] of the 3x3 matrix J[a][b] (a = coordinate, b = direction;
// c[0][0] is the reference's cjxxi, c[0][1] its cjxet, ...).
template <class R>
__device__ __forceinline__ void cofactors(const R J[3][3], R c[3][3]) {
    // a * b - c * d as fma(-c, d, a * b), the first product on the integer pipes
    c[0][0] = fma(-J[2][1], J[1][2], pmul(J[1][1], J[2][2]));
    c[0][1] = fma(-J[1][0], J[2][2], pmul(J[2][0], J[1][2]));
    c[0][2] = fma(-J[2][0], J[1][1], pmul(J[1][0], J[2][1]));
    c[1][0] = fma(-J[0][1], J[2][2], pmul(J[2][1], J[0][2]));
    c[1][1] = fma(-J[2][0], J[0][2], pmul(J[0][0], J[2][2]));
    c[1][2] = fma(-J[0][0], J[2][1], pmul(J[2][0], J[0][1]));
    c[2][0] = fma(-J[1][1], J[0][2], pmul(J[0][1], J[1][2]));
    c[2][1] = fma(-J[0][0], J[1][2], pmul(J[1][0], J[0][2]));
    c[2][2] = fma(-J[1][0], J[0][1], pmul(J[0][0], J[1][1]));
}
#endif

// zero tests of the compare helpers below (declared here for jacobian_singular)
__device__ __forceinline__ bool f_is_zero(double x);
__device__ __forceinline__ bool f_is_zero(float x);

// The reference's zero test on the centre Jacobian determinant of the force
// phase (lulesh.cc:817-821). The fast variants test the determinant of 8
// times the Jacobian in another summation order: zero for the same collapsed
// elements, though a near-singular element may round differently.
template <class R>
__device__ __forceinline__ bool jacobian_singular(const R x[8], const R y[8], const R z[8]) {
#if LULESH_EXACT
    return jac_det(jacobian(x, y, z)) == R(0);
#else
    R J[3][3];
    dirs(x, J[0]);
    dirs(y, J[1]);
    dirs(z, J[2]);
    const R det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) +
                  J[0][1] * (J[2][0] * J[1][2] - J[1][0] * J[2][2]) +
                  J[0][2] * (J[1][0] * J[2][1] - J[2][0] * J[1][1]);
    return f_is_zero(det);
#endif
}

// Shape-function derivatives b[a][0..3] (b[a][4..7] are their negatives,
// lulesh.cc:337-364) and the determinant.
template <class R>
__device__ __forceinline__ R shape_derivs(const Jac<R>& j, R b[3][4]) {
    const R cjxxi = (j.fjyet * j.fjzze) - (j.fjzet * j.fjyze);
    const R cjxet = -(j.fjyxi * j.fjzze) + (j.fjzxi * j.fjyze);
    const R cjxze = (j.fjyxi * j.fjzet) - (j.fjzxi * j.fjyet);
    const R cjyxi = -(j.fjxet * j.fjzze) + (j.fjzet * j.fjxze);
    const R cjyet = (j.fjxxi * j.fjzze) - (j.fjzxi * j.fjxze);
    const R cjyze = -(j.fjxxi * j.fjzet) + (j.fjzxi * j.fjxet);
    const R cjzxi = (j.fjxet * j.fjyze) - (j.fjyet * j.fjxze);
    const R cjzet = -(j.fjxxi * j.fjyze) + (j.fjyxi * j.fjxze);
    const R cjzze = (j.fjxxi * j.fjyet) - (j.fjyxi * j.fjxet);
    b[0][0] = -cjxxi - cjxet - cjxze;
    b[0][1] = cjxxi - cjxet - cjxze;
    b[0][2] = cjxxi + cjxet - cjxze;
    b[0][3] = -cjxxi + cjxet - cjxze;
    b[1][0] = -cjyxi - cjyet - cjyze;
    b[1][1] = cjyxi - cjyet - cjyze;
    b[1][2] = cjyxi + cjyet - cjyze;
    b[1][3] = -cjyxi + cjyet - cjyze;
    b[2][0] = -cjzxi - cjzet - cjzze;
    b[2][1] = cjzxi - cjzet - cjzze;
    b[2][2] = cjzxi + cjzet - cjzze;
    b[2][3] = -cjzxi + cjzet - cjzze;
    return R(8.) * (j.fjxet * cjxet + j.fjyet * cjyet + j.fjzet * cjzet);
}

// Division helpers. x / refdens is x itself when refdens is 1 (the
// reference's value), so that case skips the divide and stays bit-exact.
// a / sqrt(b) uses the reciprocal square root in the fast variants (one
// rounding more, a few FP64-pipe slots fewer) and the reference's divide and
// square root in the exact one.
template <bool UNIT_RHO>
__device__ __forceinline__ double over_rho(double x, const lulesh_params& P) {
    return UNIT_RHO ? x : x / P.refdens;
}

// Reciprocal and quotient. Exact variant: IEEE 1/x and a/b. Fast variants:
// the hardware's approximate double reciprocal y (rcp.approx.ftz.f64, which
// issues on the multi-function unit, not the FP64 pipe; its relative error
// measured at most 2^-19.95 over 4M inputs spanning 2^-100..2^100) and one
// third-order correction from the series 1/x = y / (1 - e) = y (1 + e + e^2
// + ...) with e = 1 - x y: three multiply-adds, truncation below 2^-57, so
// within about 1 ulp of 1/x for finite, nonzero, normal x (every divisor of
// the step is such a number). a/b becomes a * (1/b), one rounding more. This
// saves FP64-pipe slots over the IEEE divide.
__device__ __forceinline__ double rcp(double x) {
#if LULESH_EXACT
    return 1.0 / x;
#else
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
#endif
}
__device__ __forceinline__ float rcp(float x) { return 1.0f / x; }

template <class R>
__device__ __forceinline__ R quot(R a, R b) {
#if LULESH_EXACT
    return a / b;
#else
    return pmul(a, rcp(b));
#endif
}

// a / b for the relative volume: the fast variants add one correction with
// the exact residual a - b q (two multiply-adds), which rounds as the IEEE
// divide in all but rare cases and gives exactly 1 when a == b, so an
// element that has not moved keeps v = 1 and delv = 0 as in the reference
// (a delv of -1 ulp would send its EOS passes down the compressing branch).
__device__ __forceinline__ double quot_refined(double a, double b) {
#if LULESH_EXACT
    return a / b;
#else
    const double y = rcp(b);
    const double q = pmul(a, y);
    return fma(fma(-b, q, a), y, q);
#endif
}

// Comparisons. On GB300 a double compare (DSETP) occupies the FP64 pipe,
// which issues at 1/60 the integer rate. The fast variants compare the
// doubles' bit patterns on the integer pipe instead: positive doubles order
// like their 64-bit patterns, negative ones in reverse. For non-NaN inputs
// these give the IEEE results, except that -0 may compare below +0 (a test
// that then stores the constant turns a -0 into +0). The exact variant keeps
// the IEEE compares.
#if LULESH_EXACT
__device__ __forceinline__ bool f_lt(double x, double c) { return x < c; }
__device__ __forceinline__ bool f_le(double x, double c) { return x <= c; }
__device__ __forceinline__ bool f_neg(double x) { return x < 0.0; }
__device__ __forceinline__ double nonneg_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ bool f_gt(double x, double c) { return x > c; }
__device__ __forceinline__ bool f_ge(double x, double c) { return x >= c; }
__device__ __forceinline__ bool f_abs_lt(double x, double c) { return fabs(x) < c; }
__device__ __forceinline__ bool f_is_zero(double x) { return x == 0.0; }
#else
constexpr long long kMag = 0x7fffffffffffffffLL;
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool f_lt(double x, double c) {
    const long long bx = dbits(x), bc = dbits(c);
    return bc >= 0 ? bx < bc : (bx < 0 && (bx & kMag) > (bc & kMag));
}
__device__ __forceinline__ bool f_le(double x, double c) {
    const long long bx = dbits(x), bc = dbits(c);
    return bc >= 0 ? bx <= bc : (bx < 0 && (bx & kMag) >= (bc & kMag));
}
__device__ __forceinline__ bool f_gt(double x, double c) { return !f_le(x, c); }
__device__ __forceinline__ bool f_ge(double x, double c) { return !f_lt(x, c); }
__device__ __forceinline__ bool f_abs_lt(double x, double c) { return (dbits(x) & kMag) < dbits(c); }
__device__ __forceinline__ bool f_is_zero(double x) { return (dbits(x) & kMag) == 0; }
// x < 0 as IEEE (-0 is not negative)
__device__ __forceinline__ bool f_neg(double x) { return dbits(x) < 0 && (dbits(x) & kMag) != 0; }
// min of two non-negative, non-NaN doubles: their bit patterns order alike
__device__ __forceinline__ double nonneg_min(double a, double b) {
    return __longlong_as_double(min(dbits(a), dbits(b)));
}
#endif
// two variables (the limiter); floats compare on the float pipe
__device__ __forceinline__ bool f_vlt(double a, double b) {
#if LULESH_EXACT
    return a < b;
#else
    const long long ba = dbits(a), bb = dbits(b);
    const long long ka = ba ^ ((ba >> 63) & kMag), kb = bb ^ ((bb >> 63) & kMag);
    return ka < kb;
#endif
}
__device__ __forceinline__ bool f_vlt(float a, float b) { return a < b; }
__device__ __forceinline__ bool f_lt(float x, float c) { return x < c; }
__device__ __forceinline__ bool f_gt(float x, float c) { return x > c; }
__device__ __forceinline__ bool f_is_zero(float x) { return x == 0.0f; }

// Conversions between double and float on the integer pipe (conversion
// instructions occupy the FP64 pipe on GB300). narrow rounds a double to
// float, round to nearest even: add half a unit of the 29 dropped bits (just
// under half when the kept last bit is even), clear them, and a carry moves
// into the exponent as rounding does; bit for bit the conversion's result
// for magnitudes whose float is normal (overflow gives the infinity). widen
// is exact for zeros and normal floats. Zeros keep their sign; other inputs
// take the conversion instruction in a function of its own (inlined, the
// compiler would evaluate it for every input and select).
__device__ __forceinline__ unsigned long long round_to_float_bits(unsigned long long b) {
    return (b + 0x0FFFFFFFull + ((b >> 29) & 1ull)) & ~((1ull << 29) - 1ull);
}
__device__ __forceinline__ float float_from_rounded(unsigned long long b) {
    const unsigned e = unsigned(b >> 52) & 0x7ffu;
    return __uint_as_float((unsigned(b >> 32) & 0x80000000u) | ((e - 896u) << 23) |
                           (unsigned(b >> 29) & 0x7fffffu));
}
__device__ __noinline__ float narrow_convert(double v) { return __double2float_rn(v); }
__device__ __noinline__ double widen_convert(float f) { return double(f); }
__device__ __forceinline__ float narrow(double v) {
    const unsigned long long b = __double_as_longlong(v);
    const unsigned e = unsigned(b >> 52) & 0x7ffu;
    if ((b << 1) == 0ull) return __uint_as_float(unsigned(b >> 32));  // +-0
    if (e < 897u || e > 1150u) return narrow_convert(v);
    return float_from_rounded(round_to_float_bits(b));
}
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if ((u << 1) == 0u) return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(u) << 32));
    if (e == 0u || e == 0xffu) return widen_convert(f);
    return __longlong_as_double(static_cast<long long>(
        (static_cast<unsigned long long>(u & 0x80000000u) << 32) |
        (static_cast<unsigned long long>(e + 896u) << 52) | (static_cast<unsigned long long>(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double recip_sqrt(double b) { return rsqrt(b); }
__device__ __forceinline__ float recip_sqrt(float b) { return rsqrtf(b); }

#if !LULESH_EXACT
// Reciprocal cube root of a positive double (fast variants). Seed: the float
// reciprocal cube root y of x rounded to float (documented within 1 float
// ulp), so the residual r = 1 - x y^3 is below 2^-21 in magnitude. One
// third-order correction from the binomial series
//   x^(-1/3) = y (1 - r)^(-1/3) = y (1 + r/3 + 2 r^2/9 + 14 r^3/81 + ...)
// leaves a truncation error below 2^-62; y^2 is exact (y has 24 significant
// bits), so the result is within about one double ulp. Outside the float's
// normal range the double library function is used instead.
__device__ __forceinline__ double rcbrt_pos(double x) {
    const float xf = __double2float_rn(x);
    if (!(xf >= 1.17549435e-38f && xf <= 3.0e38f)) return rcbrt(x);
    const double y = double(rcbrtf(xf));
    const double r = fma(-x, (y * y) * y, 1.0);
    return fma(y, r * fma(r, 2.0 / 9.0, 1.0 / 3.0), y);
}

// Square root of a positive normal double in the fast variants: x times the
// library's reciprocal square root, one rounding more than sqrt (within
// about one ulp; the probe test measures it) for fewer FP64-pipe slots.
__device__ __forceinline__ double sqrt_fast(double x) { return pmul(x, rsqrt(x)); }
#endif

template <class R>
__device__ __forceinline__ R div_sqrt(R a, R b) {
#if LULESH_EXACT
    return a / sqrt(b);
#else
    return pmul(a, recip_sqrt(b));
#endif
}

// One face's area vector added to its four corners (SumElemFaceNormal,
// lulesh.cc:378-409); A..D are the face corners in the reference's order.
// The reference's factors 0.5 (bisectors) and 0.25 (area) are left out: the
// normals come out scaled by exactly 16, and callers scale the stress by
// 1/16 instead. Powers of two commute with rounding, so this is bit-exact.
template <int A, int B, int C, int D, class R>
__device__ __forceinline__ void face_normal(R nx[8], R ny[8], R nz[8], const R x[8], const R y[8],
                                            const R z[8]) {
    const R bisX0 = (x[D] + x[C] - x[B] - x[A]);
    const R bisY0 = (y[D] + y[C] - y[B] - y[A]);
    const R bisZ0 = (z[D] + z[C] - z[B] - z[A]);
    const R bisX1 = (x[C] + x[B] - x[D] - x[A]);
    const R bisY1 = (y[C] + y[B] - y[D] - y[A]);
    const R bisZ1 = (z[C] + z[B] - z[D] - z[A]);
    const R ax = (bisY0 * bisZ1 - bisZ0 * bisY1);
    const R ay = (bisZ0 * bisX1 - bisX0 * bisZ1);
    const R az = (bisX0 * bisY1 - bisY0 * bisX1);
    const int c[4] = {A, B, C, D};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        nx[c[k]] += ax;
        ny[c[k]] += ay;
        nz[c[k]] += az;
    }
}

#if !LULESH_EXACT
// Half the bisector cross product of face A..D: with the diagonals
// s = C - A and t = D - B the bisectors are s + t and s - t, and
// (s + t) x (s - t) = 2 t x s.
template <int A, int B, int C, int D, class R>
__device__ __forceinline__ void face_txs(const R x[8], const R y[8], const R z[8], R a[3]) {
    const R sx = x[C] - x[A], sy = y[C] - y[A], sz = z[C] - z[A];
    const R tx = x[D] - x[B], ty = y[D] - y[B], tz = z[D] - z[B];
    a[0] = fma(-tz, sy, pmul(ty, sz));
    a[1] = fma(-tx, sz, pmul(tz, sx));
    a[2] = fma(-ty, sx, pmul(tx, sy));
}
#endif

// Scale of node_normals' result relative to the reference's normals; the
// stress is multiplied by its inverse (a power of two).
constexpr double kInvNormalScale = LULESH_EXACT ? 0.0625 : 0.125;

#if !LULESH_EXACT
// Component c of the corner sums of the six faces' t x s (faces in the
// reference's order 0123, 0451, 1562, 2673, 3740, 4765): each corner adds its
// three faces, and the four face pairs that two corners share are added
// once (corners 0,1 share faces 0123 and 0451, corners 2,3 faces 0123 and
// 2673, corners 4,5 faces 0451 and 4765, corners 6,7 faces 2673 and 4765).
template <class R>
__device__ __forceinline__ void corner_sums(const R fa[6][3], int c, R n[8]) {
    const R p01 = fa[0][c] + fa[1][c], p03 = fa[0][c] + fa[3][c];
    const R p15 = fa[1][c] + fa[5][c], p35 = fa[3][c] + fa[5][c];
    n[0] = p01 + fa[4][c];
    n[1] = p01 + fa[2][c];
    n[2] = p03 + fa[2][c];
    n[3] = p03 + fa[4][c];
    n[4] = p15 + fa[4][c];
    n[5] = p15 + fa[2][c];
    n[6] = p35 + fa[2][c];
    n[7] = p35 + fa[4][c];
}
#endif

// CalcElemNodeNormals (lulesh.cc:413-451). Exact variant: faces in the
// reference's order, 16 times the reference's normals (see face_normal).
// Fast variants: 8 times the normals, the corner sums of the faces' t x s.
template <class R>
__device__ __forceinline__ void node_normals(R nx[8], R ny[8], R nz[8], const R x[8], const R y[8],
                                             const R z[8]) {
#if LULESH_EXACT
#pragma unroll
    for (int k = 0; k < 8; ++k) nx[k] = ny[k] = nz[k] = R(0.0);
    face_normal<0, 1, 2, 3>(nx, ny, nz, x, y, z);
    face_normal<0, 4, 5, 1>(nx, ny, nz, x, y, z);
    face_normal<1, 5, 6, 2>(nx, ny, nz, x, y, z);
    face_normal<2, 6, 7, 3>(nx, ny, nz, x, y, z);
    face_normal<3, 7, 4, 0>(nx, ny, nz, x, y, z);
    face_normal<4, 7, 6, 5>(nx, ny, nz, x, y, z);
#else
    R fa[6][3];
    face_txs<0, 1, 2, 3>(x, y, z, fa[0]);
    face_txs<0, 4, 5, 1>(x, y, z, fa[1]);
    face_txs<1, 5, 6, 2>(x, y, z, fa[2]);
    face_txs<2, 6, 7, 3>(x, y, z, fa[3]);
    face_txs<3, 7, 4, 0>(x, y, z, fa[4]);
    face_txs<4, 7, 6, 5>(x, y, z, fa[5]);
    corner_sums(fa, 0, nx);
    corner_sums(fa, 1, ny);
    corner_sums(fa, 2, nz);
#endif
}

// VoluDer (lulesh.cc:468-491) for corner K from the corners P0..P5.
template <int K, int P0, int P1, int P2, int P3, int P4, int P5, class R>
__device__ __forceinline__ void volu_der(R dvdx[8], R dvdy[8], R dvdz[8], const R x[8],
                                         const R y[8], const R z[8]) {
    const R twelfth = R(1.0) / R(12.0);
    const R x0 = x[P0], x1 = x[P1], x2 = x[P2], x3 = x[P3], x4 = x[P4], x5 = x[P5];
    const R y0 = y[P0], y1 = y[P1], y2 = y[P2], y3 = y[P3], y4 = y[P4], y5 = y[P5];
    const R z0 = z[P0], z1 = z[P1], z2 = z[P2], z3 = z[P3], z4 = z[P4], z5 = z[P5];
    const R dx = (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) + (y0 + y4) * (z3 + z4) -
                 (y3 + y4) * (z0 + z4) - (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    const R dy = -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) - (x0 + x4) * (z3 + z4) +
                 (x3 + x4) * (z0 + z4) + (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    const R dz = -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) - (y0 + y4) * (x3 + x4) +
                 (y3 + y4) * (x0 + x4) + (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
#if LULESH_EXACT
    dvdx[K] = dx * twelfth;
    dvdy[K] = dy * twelfth;
    dvdz[K] = dz * twelfth;
#else
    // fast variants: 12 x the derivative; hourgam_all folds 1/12 into volinv
    (void)twelfth;
    dvdx[K] = dx;
    dvdy[K] = dy;
    dvdz[K] = dz;
#endif
}

// CalcElemVolumeDerivative (lulesh.cc:495-523).
template <class R>
__device__ __forceinline__ void volume_derivs(R dvdx[8], R dvdy[8], R dvdz[8], const R x[8],
                                              const R y[8], const R z[8]) {
    volu_der<0, 1, 2, 3, 4, 5, 7>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<3, 0, 1, 2, 7, 4, 6>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<2, 3, 0, 1, 6, 7, 5>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<1, 2, 3, 0, 5, 6, 4>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<4, 7, 6, 5, 0, 3, 1>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<5, 4, 7, 6, 1, 0, 2>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<6, 5, 4, 7, 2, 1, 3>(dvdx, dvdy, dvdz, x, y, z);
    volu_der<7, 6, 5, 4, 3, 2, 0>(dvdx, dvdy, dvdz, x, y, z);
}

// Flanagan-Belytschko hourglass base vector M at corner k (lulesh.cc:921-954):
//   {1,1,-1,-1,-1,-1,1,1} {1,-1,-1,1,-1,1,1,-1} {1,-1,1,-1,1,-1,1,-1} {-1,1,-1,1,1,-1,1,-1}
__host__ __device__ constexpr int gamma_sign(int M, int k) {
    return (M == 0)   ? ((k == 2 || k == 3 || k == 4 || k == 5) ? -1 : 1)
           : (M == 1) ? ((k == 1 || k == 2 || k == 4 || k == 7) ? -1 : 1)
           : (M == 2) ? ((k & 1) ? -1 : 1)
                      : ((k == 0 || k == 2 || k == 5 || k == 7) ? -1 : 1);
}

// Sum_k v[k] * gamma[M][k] in the reference's left-to-right order
// (lulesh.cc:972-986); the products by +-1 are exact.
template <int M, class R>
__device__ __forceinline__ R hourmod(const R v[8]) {
    return v[0] * R(gamma_sign(M, 0)) + v[1] * R(gamma_sign(M, 1)) + v[2] * R(gamma_sign(M, 2)) +
           v[3] * R(gamma_sign(M, 3)) + v[4] * R(gamma_sign(M, 4)) + v[5] * R(gamma_sign(M, 5)) +
           v[6] * R(gamma_sign(M, 6)) + v[7] * R(gamma_sign(M, 7));
}

// All four mode sums of one coordinate with shared pair sums and differences
// (18 adds instead of 28); a different summation order than the reference,
// so fast variants only.
template <class R>
__device__ __forceinline__ void hourmod4(const R v[8], R h[4]) {
    const R a01 = v[0] + v[1], a23 = v[2] + v[3], a45 = v[4] + v[5], a67 = v[6] + v[7];
    const R d01 = v[0] - v[1], d23 = v[2] - v[3], d45 = v[4] - v[5], d67 = v[6] - v[7];
    const R p = d01 + d23, q = d45 + d67;
    h[0] = (a01 - a23) - (a45 - a67);  // (+ + - - - - + +)
    h[1] = (d01 - d23) - (d45 - d67);  // (+ - - + - + + -)
    h[2] = p + q;                      // (+ - + - + - + -)
    h[3] = q - p;                      // (- + - + + - + -)
}

#if !LULESH_EXACT
// dirs(v, d) and hourmod4(v, h) together as a three-stage Walsh-Hadamard
// transform over the corners' (xi, eta, zeta) signs: 23 adds for the 7
// non-constant coefficients instead of 11 + 18.
template <class R>
__device__ __forceinline__ void walsh7(const R v[8], R d[3], R h[4]) {
    // xi pairs of the four (eta, zeta) edges: corners (0,1), (3,2), (4,5), (7,6)
    const R p00 = v[1] + v[0], m00 = v[1] - v[0], p10 = v[2] + v[3], m10 = v[2] - v[3];
    const R p01 = v[5] + v[4], m01 = v[5] - v[4], p11 = v[6] + v[7], m11 = v[6] - v[7];
    // eta, per zeta layer
    const R pp0 = p10 + p00, pm0 = p10 - p00, mp0 = m10 + m00, mm0 = m10 - m00;
    const R pp1 = p11 + p01, pm1 = p11 - p01, mp1 = m11 + m01, mm1 = m11 - m01;
    // zeta
    d[0] = mp1 + mp0;  // xi
    d[1] = pm1 + pm0;  // eta
    d[2] = pp1 - pp0;  // zeta
    h[0] = pm1 - pm0;  // eta zeta
    h[1] = mp1 - mp0;  // zeta xi
    h[2] = mm1 + mm0;  // xi eta
    h[3] = mm1 - mm0;  // xi eta zeta
}
#endif

#if !LULESH_EXACT
// 192 times the gradient of the element volume with respect to each corner
// (fast variants). With the body-diagonal sums A_d = sum_k s_dk x_k (the
// columns of J = dirs, s_dk = xi, eta, zeta of corner k) and the hourglass
// mode sums H_m = sum_k t_mk x_k (hourmod4's modes eta zeta, zeta xi, xi eta),
// the trilinear hexahedron's volume, its integral of det(dx/dxi) over the
// reference cube, is
//   64 V = det(A1, A2, A3) + (det(A1, H3, H2) + det(H3, A2, H1) + det(H2, H1, A3)) / 3,
// the value of the reference's CalcElemVolume (lulesh.cc:592-665) in another
// form. Its gradient at corner k is sum_d s_dk dV/dA_d + sum_m t_mk dV/dH_m:
// six vectors of cross products (c holds cof(J), whose column d is
// A_{d+1} x A_{d+2}) and a sign transform over the corners, in place of
// VoluDer's six products per component and corner (lulesh.cc:468-523).
template <class R>
__device__ __forceinline__ void cross_acc(const R u[3], const R v[3], R w[3]) {  // w += u x v
    w[0] = fma(u[1], v[2], fma(-u[2], v[1], w[0]));
    w[1] = fma(u[2], v[0], fma(-u[0], v[2], w[1]));
    w[2] = fma(u[0], v[1], fma(-u[1], v[0], w[2]));
}
template <class R>
__device__ __forceinline__ void volume_gradient(const R J[3][3], const R c[3][3], const R hx[4],
                                                const R hy[4], const R hz[4], R gx[8], R gy[8],
                                                R gz[8]) {
    const R A[3][3] = {{J[0][0], J[1][0], J[2][0]}, {J[0][1], J[1][1], J[2][1]}, {J[0][2], J[1][2], J[2][2]}};
    const R H[3][3] = {{hx[0], hy[0], hz[0]}, {hx[1], hy[1], hz[1]}, {hx[2], hy[2], hz[2]}};
    R g[6][3];  // dV/dA_1..3, dV/dH_1..3, times 192
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g[0][a] = pmul(R(3), c[a][0]);
        g[1][a] = pmul(R(3), c[a][1]);
        g[2][a] = pmul(R(3), c[a][2]);
        g[3][a] = g[4][a] = g[5][a] = R(0);
    }
    cross_acc(H[2], H[1], g[0]);
    cross_acc(H[0], H[2], g[1]);
    cross_acc(H[1], H[0], g[2]);
    cross_acc(H[2], A[1], g[3]);
    cross_acc(A[2], H[1], g[3]);
    cross_acc(A[0], H[2], g[4]);
    cross_acc(H[0], A[2], g[4]);
    cross_acc(H[1], A[0], g[5]);
    cross_acc(A[1], H[0], g[5]);
    R* out[3] = {gx, gy, gz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // f = xi g1 + eta g2 + zeta g3 + eta zeta g4 + zeta xi g5 + xi eta g6 at the corners
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // zeta = -1 (corners 0-3), +1 (corners 4-7)
            const R bx = h ? g[0][a] + g[4][a] : g[0][a] - g[4][a];
            const R by = h ? g[1][a] + g[3][a] : g[1][a] - g[3][a];
            const R p = bx + by, q = bx - by;
            const R sv = h ? g[5][a] + g[2][a] : g[5][a] - g[2][a];  // xi eta g6 + zeta g3, xi = eta
            const R tv = h ? g[2][a] - g[5][a] : -g[2][a] - g[5][a];  // xi = -eta
            out[a][4 * h + 0] = sv - p;  // (-1, -1)
            out[a][4 * h + 1] = tv + q;  // ( 1, -1)
            out[a][4 * h + 2] = sv + p;  // ( 1,  1)
            out[a][4 * h + 3] = tv - q;  // (-1,  1)
        }
    }
}
#endif

// Hourglass shape vectors of mode M (lulesh.cc:988-1023) from the mode sums
// hx, hy, hz of the coordinates, already multiplied by volinv: three
// multiply-adds per corner.
template <int M, class R>
__device__ __forceinline__ void hourgam_mode_h(R hg[8][4], R hx, R hy, R hz, const R dvdx[8],
                                               const R dvdy[8], const R dvdz[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
        hg[k][M] = R(gamma_sign(M, k)) - dvdx[k] * hx - dvdy[k] * hy - dvdz[k] * hz;
}

// Hourglass shape vectors of mode M (lulesh.cc:988-1023).
template <int M, class R>
__device__ __forceinline__ void hourgam_mode(R hg[8][4], const R x[8], const R y[8], const R z[8],
                                             const R dvdx[8], const R dvdy[8], const R dvdz[8],
                                             R volinv) {
    const R hx = hourmod<M>(x), hy = hourmod<M>(y), hz = hourmod<M>(z);
#pragma unroll
    for (int k = 0; k < 8; ++k)
        hg[k][M] = R(gamma_sign(M, k)) - volinv * (dvdx[k] * hx + dvdy[k] * hy + dvdz[k] * hz);
}

// volinv = 1 / (volo v); in the fast variants the volume derivatives come
// 12 times too large (volu_der) and the 1/12 is applied here, once.
template <class R>
__device__ __forceinline__ void hourgam_all(R hg[8][4], const R x[8], const R y[8], const R z[8],
                                            const R dvdx[8], const R dvdy[8], const R dvdz[8],
                                            R volinv) {
#if LULESH_EXACT
    hourgam_mode<0>(hg, x, y, z, dvdx, dvdy, dvdz, volinv);
    hourgam_mode<1>(hg, x, y, z, dvdx, dvdy, dvdz, volinv);
    hourgam_mode<2>(hg, x, y, z, dvdx, dvdy, dvdz, volinv);
    hourgam_mode<3>(hg, x, y, z, dvdx, dvdy, dvdz, volinv);
#else
    volinv = volinv * (R(1.0) / R(12.0));
    R hx[4], hy[4], hz[4];
    hourmod4(x, hx);
    hourmod4(y, hy);
    hourmod4(z, hz);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        hx[m] *= volinv;
        hy[m] *= volinv;
        hz[m] *= volinv;
    }
    hourgam_mode_h<0>(hg, hx[0], hy[0], hz[0], dvdx, dvdy, dvdz);
    hourgam_mode_h<1>(hg, hx[1], hy[1], hz[1], dvdx, dvdy, dvdz);
    hourgam_mode_h<2>(hg, hx[2], hy[2], hz[2], dvdx, dvdy, dvdz);
    hourgam_mode_h<3>(hg, hx[3], hy[3], hz[3], dvdx, dvdy, dvdz);
#endif
}

// CalcElemFBHourglassForce for one axis (lulesh.cc:527-562).
template <class R>
__device__ __forceinline__ void fb_force_axis(const R hg[8][4], const R vel[8], R coefficient,
                                              R out[8]) {
    R h[4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
        h[m] = hg[0][m] * vel[0] + hg[1][m] * vel[1] + hg[2][m] * vel[2] + hg[3][m] * vel[3] +
               hg[4][m] * vel[4] + hg[5][m] * vel[5] + hg[6][m] * vel[6] + hg[7][m] * vel[7];
#if LULESH_EXACT
#pragma unroll
    for (int k = 0; k < 8; ++k)
        out[k] = coefficient * (hg[k][0] * h[0] + hg[k][1] * h[1] + hg[k][2] * h[2] + hg[k][3] * h[3]);
#else
    // fast variants: the coefficient scales the 4 mode amplitudes, not the 8 corners
#pragma unroll
    for (int m = 0; m < 4; ++m) h[m] *= coefficient;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        out[k] = hg[k][0] * h[0] + hg[k][1] * h[1] + hg[k][2] * h[2] + hg[k][3] * h[3];
#endif
}

#if !LULESH_EXACT
// fb_force_axis added to init[k] (the corner's stress force): four
// multiply-adds per corner.
template <class R>
__device__ __forceinline__ void fb_force_axis_plus(const R hg[8][4], const R vel[8], R coefficient,
                                                   const R init[8], R out[8]) {
    R h[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        R d = pmul(hg[0][m], vel[0]);
#pragma unroll
        for (int k = 1; k < 8; ++k) d = fma(hg[k][m], vel[k], d);
        h[m] = pmul(d, coefficient);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
        out[k] = init[k] + hg[k][0] * h[0] + hg[k][1] * h[1] + hg[k][2] * h[2] + hg[k][3] * h[3];
}
#endif

// AreaFace (lulesh.cc:678-692) of the face with corners A..D.
template <int A, int B, int C, int D, class R>
__device__ __forceinline__ R face_area(const R x[8], const R y[8], const R z[8]) {
    const R fx = (x[C] - x[A]) - (x[D] - x[B]);
    const R fy = (y[C] - y[A]) - (y[D] - y[B]);
    const R fz = (z[C] - z[A]) - (z[D] - z[B]);
    const R gx = (x[C] - x[A]) + (x[D] - x[B]);
    const R gy = (y[C] - y[A]) + (y[D] - y[B]);
    const R gz = (z[C] - z[A]) + (z[D] - z[B]);
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) -
           (fx * gx + fy * gy + fz * gz) * (fx * gx + fy * gy + fz * gz);
}

template <class R>
__device__ __forceinline__ R max_ref(R a, R cl) {
    return (a < cl) ? cl : a;  // std::max(a, cl)
}

#if !LULESH_EXACT
// max of two non-negative values; doubles on the integer pipe
__device__ __forceinline__ double nonneg_max(double a, double b) {
    return __longlong_as_double(max(dbits(a), dbits(b)));
}
__device__ __forceinline__ float nonneg_max(float a, float b) { return fmaxf(a, b); }

// |s x t|^2 for the face diagonals s = C - A, t = D - B: a quarter of the
// reference's face measure (with f = s - t, g = s + t, Lagrange's identity
// gives |f|^2 |g|^2 - (f.g)^2 = |f x g|^2 = 4 |s x t|^2).
template <int A, int B, int C, int D, class R>
__device__ __forceinline__ R face_cross2(const R x[8], const R y[8], const R z[8]) {
    const R sx = x[C] - x[A], sy = y[C] - y[A], sz = z[C] - z[A];
    const R tx = x[D] - x[B], ty = y[D] - y[B], tz = z[D] - z[B];
    const R cx = sy * tz - sz * ty, cy = sz * tx - sx * tz, cz = sx * ty - sy * tx;
    return cx * cx + cy * cy + cz * cz;
}
#endif

// Characteristic length 4 V / sqrt(largest face measure)
// (CalcElemCharacteristicLength, lulesh.cc:696-729).
template <class R>
__device__ __forceinline__ R max_face_area(const R x[8], const R y[8], const R z[8]);

template <class R>
__device__ __forceinline__ R char_length(const R x[8], const R y[8], const R z[8], R volume) {
#if LULESH_EXACT
    return div_sqrt(R(4.0) * volume, max_face_area(x, y, z));
#else
    R cl = face_cross2<0, 1, 2, 3>(x, y, z);
    cl = nonneg_max(cl, face_cross2<4, 5, 6, 7>(x, y, z));
    cl = nonneg_max(cl, face_cross2<0, 1, 5, 4>(x, y, z));
    cl = nonneg_max(cl, face_cross2<1, 2, 6, 5>(x, y, z));
    cl = nonneg_max(cl, face_cross2<2, 3, 7, 6>(x, y, z));
    cl = nonneg_max(cl, face_cross2<3, 0, 4, 7>(x, y, z));
    return div_sqrt(R(2.0) * volume, cl);  // 4 V / sqrt(4 cl)
#endif
}

// Largest face measure of CalcElemCharacteristicLength (lulesh.cc:696-729);
// the characteristic length is 4 V / sqrt(of it).
template <class R>
__device__ __forceinline__ R max_face_area(const R x[8], const R y[8], const R z[8]) {
    R cl = R(0.0);
    cl = max_ref(face_area<0, 1, 2, 3>(x, y, z), cl);
    cl = max_ref(face_area<4, 5, 6, 7>(x, y, z), cl);
    cl = max_ref(face_area<0, 1, 5, 4>(x, y, z), cl);
    cl = max_ref(face_area<1, 2, 6, 5>(x, y, z), cl);
    cl = max_ref(face_area<2, 3, 7, 6>(x, y, z), cl);
    cl = max_ref(face_area<3, 0, 4, 7>(x, y, z), cl);
    return cl;
}

// Monotonic-Q gradients of CalcMonotonicQGradientsForElemsTask
// (lulesh.cc:1341-1416). vol = volo * vnew. Outputs
// g[0..2] = delv_xi, delv_eta, delv_zeta and g[3..5] = delx_xi, delx_eta, delx_zeta.
template <class R>
__device__ __forceinline__ void q_gradients(const R x[8], const R y[8], const R z[8], const R xv[8],
                                            const R yv[8], const R zv[8], R vol, R g[6]) {
    const R ptiny = R(1.e-36);
    const R q = R(0.25), mq = R(-0.25);
    const R norm = rcp(vol + ptiny);
    const R dxj = mq * ((x[0] + x[1] + x[5] + x[4]) - (x[3] + x[2] + x[6] + x[7]));
    const R dyj = mq * ((y[0] + y[1] + y[5] + y[4]) - (y[3] + y[2] + y[6] + y[7]));
    const R dzj = mq * ((z[0] + z[1] + z[5] + z[4]) - (z[3] + z[2] + z[6] + z[7]));
    const R dxi = q * ((x[1] + x[2] + x[6] + x[5]) - (x[0] + x[3] + x[7] + x[4]));
    const R dyi = q * ((y[1] + y[2] + y[6] + y[5]) - (y[0] + y[3] + y[7] + y[4]));
    const R dzi = q * ((z[1] + z[2] + z[6] + z[5]) - (z[0] + z[3] + z[7] + z[4]));
    const R dxk = q * ((x[4] + x[5] + x[6] + x[7]) - (x[0] + x[1] + x[2] + x[3]));
    const R dyk = q * ((y[4] + y[5] + y[6] + y[7]) - (y[0] + y[1] + y[2] + y[3]));
    const R dzk = q * ((z[4] + z[5] + z[6] + z[7]) - (z[0] + z[1] + z[2] + z[3]));
    R ax, ay, az, dxv, dyv, dzv;

    // zeta: i cross j
    ax = dyi * dzj - dzi * dyj;
    ay = dzi * dxj - dxi * dzj;
    az = dxi * dyj - dyi * dxj;
    g[5] = div_sqrt(vol, ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = q * ((xv[4] + xv[5] + xv[6] + xv[7]) - (xv[0] + xv[1] + xv[2] + xv[3]));
    dyv = q * ((yv[4] + yv[5] + yv[6] + yv[7]) - (yv[0] + yv[1] + yv[2] + yv[3]));
    dzv = q * ((zv[4] + zv[5] + zv[6] + zv[7]) - (zv[0] + zv[1] + zv[2] + zv[3]));
    g[2] = ax * dxv + ay * dyv + az * dzv;

    // xi: j cross k
    ax = dyj * dzk - dzj * dyk;
    ay = dzj * dxk - dxj * dzk;
    az = dxj * dyk - dyj * dxk;
    g[3] = div_sqrt(vol, ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = q * ((xv[1] + xv[2] + xv[6] + xv[5]) - (xv[0] + xv[3] + xv[7] + xv[4]));
    dyv = q * ((yv[1] + yv[2] + yv[6] + yv[5]) - (yv[0] + yv[3] + yv[7] + yv[4]));
    dzv = q * ((zv[1] + zv[2] + zv[6] + zv[5]) - (zv[0] + zv[3] + zv[7] + zv[4]));
    g[0] = ax * dxv + ay * dyv + az * dzv;

    // eta: k cross i
    ax = dyk * dzi - dzk * dyi;
    ay = dzk * dxi - dxk * dzi;
    az = dxk * dyi - dyk * dxi;
    g[4] = div_sqrt(vol, ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = mq * ((xv[0] + xv[1] + xv[5] + xv[4]) - (xv[3] + xv[2] + xv[6] + xv[7]));
    dyv = mq * ((yv[0] + yv[1] + yv[5] + yv[4]) - (yv[3] + yv[2] + yv[6] + yv[7]));
    dzv = mq * ((zv[0] + zv[1] + zv[5] + zv[4]) - (zv[3] + zv[2] + zv[6] + zv[7]));
    g[1] = ax * dxv + ay * dyv + az * dzv;
}

// Trace of the velocity gradient at the half-step geometry
// (CalcElemVelocityGradient lulesh.cc:733-781, d[0]+d[1]+d[2] as
// lulesh.cc:1232). xh.. are the half-step coordinates.
template <class R>
__device__ __forceinline__ R vel_grad_trace(const R xh[8], const R yh[8], const R zh[8],
                                            const R xv[8], const R yv[8], const R zv[8]) {
    R b[3][4];
    const R detJ = shape_derivs(jacobian(xh, yh, zh), b);
    const R inv = rcp(detJ);
    const R dxx = inv * (b[0][0] * (xv[0] - xv[6]) + b[0][1] * (xv[1] - xv[7]) +
                         b[0][2] * (xv[2] - xv[4]) + b[0][3] * (xv[3] - xv[5]));
    const R dyy = inv * (b[1][0] * (yv[0] - yv[6]) + b[1][1] * (yv[1] - yv[7]) +
                         b[1][2] * (yv[2] - yv[4]) + b[1][3] * (yv[3] - yv[5]));
    const R dzz = inv * (b[2][0] * (zv[0] - zv[6]) + b[2][1] * (zv[1] - zv[7]) +
                         b[2][2] * (zv[2] - zv[4]) + b[2][3] * (zv[3] - zv[5]));
    return dxx + dyy + dzz;
}

#if !LULESH_EXACT
// gradients_vdov from the coordinates' direction sums X and their cofactors
// c = cof(X), computed by the caller (fast variants).
template <class R>
__device__ __forceinline__ R gradients_vdov_xc(const R X[3][3], const R cx[3][3], const R xv[8],
                                               const R yv[8], const R zv[8], R vol, R dt2, R g[6]) {
    R V[3][3], c[3][3];
    dirs(xv, V[0]);
    dirs(yv, V[1]);
    dirs(zv, V[2]);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) c[a][d] = cx[a][d];
    const R pt = R(256.0) * R(1.e-36);
    const R vol16 = pmul(R(16.0), vol);
    const R n64 = pmul(rcp(vol + R(1.e-36)), R(0.015625));
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        g[3 + d] = pmul(vol16, recip_sqrt(fma(c[2][d], c[2][d], fma(c[1][d], c[1][d], pmul(c[0][d], c[0][d]))) + pt));
        g[d] = pmul(fma(c[2][d], V[2][d], fma(c[1][d], V[1][d], pmul(c[0][d], V[0][d]))), n64);
    }
    R J[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) J[a][d] = X[a][d] - dt2 * V[a][d];
    cofactors(J, c);
    const R det = fma(J[0][2], c[0][2], fma(J[0][1], c[0][1], pmul(J[0][0], c[0][0])));
    R num = pmul(c[0][0], V[0][0]);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (a + d > 0) num = num + c[a][d] * V[a][d];
    return quot(num, det);
}
#endif

// Q gradients g (as q_gradients) and vdov, the trace of the velocity
// gradient at the half-step geometry x - dt2 v (lulesh.cc:1221-1232), of one
// element. Exact variant: the reference's two computations. Fast variants,
// from the 18 direction sums X = dirs(x, y, z) and V = dirs(xv, yv, zv):
//  * the Q-gradient cross products of directions i x j, j x k, k x i are the
//    cofactor columns of X, and the sums are 4 times the reference's
//    differences, so with C = cof(X) = 16 a: delx = 16 vol / sqrt(|C|^2 +
//    256 ptiny) and delv = (C . V) / (64 (vol + ptiny));
//  * the half-step Jacobian is J = X - dt2 V (dirs is linear) and the trace
//    of V J^-1 is sum(cof(J) * V) / det(J); the 8x scale of J cancels.
template <class R>
__device__ __forceinline__ R gradients_vdov(const R x[8], const R y[8], const R z[8], const R xv[8],
                                            const R yv[8], const R zv[8], R vol, R dt2, R g[6]) {
#if LULESH_EXACT
    q_gradients(x, y, z, xv, yv, zv, vol, g);
    R xh[8], yh[8], zh[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        xh[k] = x[k] - dt2 * xv[k];
        yh[k] = y[k] - dt2 * yv[k];
        zh[k] = z[k] - dt2 * zv[k];
    }
    return vel_grad_trace(xh, yh, zh, xv, yv, zv);
#else
    R X[3][3], c[3][3];
    dirs(x, X[0]);
    dirs(y, X[1]);
    dirs(z, X[2]);
    cofactors(X, c);
    return gradients_vdov_xc(X, c, xv, yv, zv, vol, dt2, g);
#endif
}



// --- material ------------------------------------------------------------

// Monotonic limiter of one direction (lulesh.cc:1464-1531, repeated for eta
// and zeta): dv is the direction's velocity gradient, bm/bp the minus/plus
// face BC bits, nm/np the face neighbours.
template <class R>
__device__ __forceinline__ R limiter(const R* __restrict__ dv, int i, int bm, int bp, int symm_m,
                                     int comm_m, int nm, int symm_p, int comm_p, int np, R mult,
                                     R max_slope) {
    const R ptiny = R(1.e-36);
    const R self = LD(dv + i);
    const R norm = rcp(self + ptiny);
    R delvm, delvp;
    if (bm == comm_m || bm == 0) delvm = LD(dv + nm);
    else if (bm == symm_m) delvm = self;
    else delvm = R(0.0);  // free surface (and malformed masks, lulesh.cc:1477-1480)
    if (bp == comm_p || bp == 0) delvp = LD(dv + np);
    else if (bp == symm_p) delvp = self;
    else delvp = R(0.0);
    delvm = pmul(delvm, norm);
    delvp = pmul(delvp, norm);
    R phi = pmul(R(.5), delvm + delvp);
    delvm = pmul(delvm, mult);
    delvp = pmul(delvp, mult);
    if (f_vlt(delvm, phi)) phi = delvm;
    if (f_vlt(delvp, phi)) phi = delvp;
    if (f_lt(phi, R(0.))) phi = R(0.);
    if (f_gt(phi, max_slope)) phi = max_slope;
    return phi;
}

// Linear and quadratic q of one element (lulesh.cc:1448-1656). dv/dx are the
// six gradient arrays.
template <class R>
__device__ __forceinline__ void q_terms(const Mesh& m, int i, const R* dvxi, const R* dveta,
                                        const R* dvzeta, const R* dxxi, const R* dxeta,
                                        const R* dxzeta, double vnew, double vdov, double& ql,
                                        double& qq) {
    const lulesh_params& P = m.prm;
    const int bc = LD(m.elemBC + i);
    const R mult = R(P.monoq_limiter_mult), slope = R(P.monoq_max_slope);
    const R phixi = limiter(dvxi, i, bc & XI_M, bc & XI_P, XI_M_SYMM, XI_M_COMM, LD(m.lxim + i),
                            XI_P_SYMM, XI_P_COMM, LD(m.lxip + i), mult, slope);
    const R phieta = limiter(dveta, i, bc & ETA_M, bc & ETA_P, ETA_M_SYMM, ETA_M_COMM,
                             LD(m.letam + i), ETA_P_SYMM, ETA_P_COMM, LD(m.letap + i), mult, slope);
    const R phizeta = limiter(dvzeta, i, bc & ZETA_M, bc & ZETA_P, ZETA_M_SYMM, ZETA_M_COMM,
                              LD(m.lzetam + i), ZETA_P_SYMM, ZETA_P_COMM, LD(m.lzetap + i), mult,
                              slope);
    if (f_gt(vdov, 0.)) {
        ql = 0.;
        qq = 0.;
        return;
    }
    R dxi = pmul(LD(dvxi + i), LD(dxxi + i));
    R deta = pmul(LD(dveta + i), LD(dxeta + i));
    R dzeta = pmul(LD(dvzeta + i), LD(dxzeta + i));
    if (f_gt(dxi, R(0.))) dxi = R(0.);
    if (f_gt(deta, R(0.))) deta = R(0.);
    if (f_gt(dzeta, R(0.))) dzeta = R(0.);
    const R rho = R(quot(LD(m.elemMass + i), pmul(LD(m.volo + i), vnew)));
    const R qlin = pmul(pmul(-R(P.qlc_monoq), rho),
                        pmul(dxi, R(1.) - phixi) + pmul(deta, R(1.) - phieta) + pmul(dzeta, R(1.) - phizeta));
    const R qquad = pmul(pmul(R(P.qqc_monoq), rho),
                         pmul(pmul(dxi, dxi), R(1.) - pmul(phixi, phixi)) +
                         pmul(pmul(deta, deta), R(1.) - pmul(phieta, phieta)) +
                         pmul(pmul(dzeta, dzeta), R(1.) - pmul(phizeta, phizeta)));
    ql = double(qlin);
    qq = double(qquad);
}

// CalcPressureForElemsTask for one element (lulesh.cc:1671-1690).
__device__ __forceinline__ double eos_pressure(double& bvc, double& pbvc, double e, double comp,
                                               double vnewc, const lulesh_params& P) {
    const double cls = 2.0 / 3.0;
    bvc = cls * (comp + 1.0);
    pbvc = cls;
    double nv = bvc * e;
    if (f_abs_lt(nv, P.p_cut) || f_ge(vnewc, P.eosvmax)) nv = 0.0;
    if (f_lt(nv, P.pmin)) nv = P.pmin;
    return nv;
}

__device__ __forceinline__ double ss_guard(double ssc) {
#if LULESH_EXACT
    return f_le(ssc, .1111111e-36) ? .3333333e-18 : sqrt(ssc);
#else
    return f_le(ssc, .1111111e-36) ? .3333333e-18 : sqrt_fast(ssc);
#endif
}

// Square root of the q terms' sound-speed expression (ss_guard's guard and
// value). The mixed variant forms the linear and quadratic q coefficients
// (ql, qq) in float, so its q terms take a float square root of the double
// expression (two conversions and a float reciprocal square root instead of
// the double sequence); the sound speed saved for the dt constraints stays
// double.
#ifndef LULESH_FLOAT_Q
#define LULESH_FLOAT_Q 0
#endif
__device__ __forceinline__ double q_sound(double ssc) {
#if LULESH_FLOAT_Q
    if (f_le(ssc, .1111111e-36)) return .3333333e-18;
    const float f = float(ssc);
    return double(f * rsqrtf(f));
#else
    return ss_guard(ssc);
#endif
}

// rep evaluations of EvalEOSAllInOneTask (lulesh.cc:1692-1871) for element i,
// each from the saved state, then the sound speed and the save of
// CalcSoundSpeedForElemsAndSaveTask (lulesh.cc:1873-1904). Returns ss.
// UNIT_RHO: refdens == 1, so the divisions by it are identities.
#if LULESH_EXACT
// The reference's "+ 0.5 * work" terms add 0.5 * 0 (work is zero,
// lulesh.cc:1749); adding +0 only turns a -0 into +0, so the fast variants
// leave them out.
#define LULESH_PLUS_ZERO_WORK +0.5 * 0.0
template <bool UNIT_RHO>
__device__ __forceinline__ double eos_body(const Mesh& m, int i, double vnewc, int rep) {
    const lulesh_params& P = m.prm;
    double e_new = 0., p_new = 0., q_new = 0., bvc = 0., pbvc = 0.;
    const bool vmin_on = !f_is_zero(P.eosvmin), vmax_on = !f_is_zero(P.eosvmax);
    for (int r = 0; r < rep; ++r) {
        // Each evaluation re-reads its inputs from memory as the reference's
        // EvalEOSInit does (lulesh.cc:1720-1727), and vnewc is made opaque,
        // so the compiler can hoist no part of the evaluation out of the
        // repeat loop: the repeat count stays real work.
        asm volatile("" ::: "memory");
        asm volatile("" : "+d"(vnewc));
        const double e_old = m.e[i], delvc = m.delv[i], q_old = m.q[i];
        double p_old = m.p[i];
        const double qq_old = m.qq[i], ql_old = m.ql[i];
        double comp = rcp(vnewc) - 1.;
        const double vchalf = vnewc - delvc * .5;
        double compHalf = rcp(vchalf) - 1.;
        if (vmin_on && f_le(vnewc, P.eosvmin)) compHalf = comp;
        if (vmax_on && f_ge(vnewc, P.eosvmax)) {
            p_old = 0.;
            comp = 0.;
            compHalf = 0.;
        }
        // predictor
        e_new = e_old - 0.5 * delvc * (p_old + q_old) LULESH_PLUS_ZERO_WORK;
        if (f_lt(e_new, P.emin)) e_new = P.emin;
        const double pHalf = eos_pressure(bvc, pbvc, e_new, compHalf, vnewc, P);
        const double vhalf = rcp(1. + compHalf);
        if (f_gt(delvc, 0.)) {
            q_new = 0.;
        } else {
            const double ssc = ss_guard(over_rho<UNIT_RHO>((pbvc * e_new + vhalf * vhalf * bvc * pHalf), P));
            q_new = (ssc * ql_old + qq_old);
        }
        e_new = e_new + 0.5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (pHalf + q_new));
        e_new = e_new LULESH_PLUS_ZERO_WORK;
        if (f_abs_lt(e_new, P.e_cut)) e_new = 0.0;
        if (f_lt(e_new, P.emin)) e_new = P.emin;
        p_new = eos_pressure(bvc, pbvc, e_new, comp, vnewc, P);
        // corrector
        {
            const double sixth = 1.0 / 6.0;
            double q_tilde;
            if (f_gt(delvc, 0.)) {
                q_tilde = 0.;
            } else {
                const double ssc = ss_guard(over_rho<UNIT_RHO>((pbvc * e_new + vnewc * vnewc * bvc * p_new), P));
                q_tilde = (ssc * ql_old + qq_old);
            }
            e_new = e_new -
                    (7.0 * (p_old + q_old) - 8.0 * (pHalf + q_new) + (p_new + q_tilde)) * delvc * sixth;
            if (f_abs_lt(e_new, P.e_cut)) e_new = 0.;
            if (f_lt(e_new, P.emin)) e_new = P.emin;
        }
        p_new = eos_pressure(bvc, pbvc, e_new, comp, vnewc, P);
        if (f_le(delvc, 0.)) {
            const double ssc = ss_guard(over_rho<UNIT_RHO>((pbvc * e_new + vnewc * vnewc * bvc * p_new), P));
            q_new = (ssc * ql_old + qq_old);
            if (f_abs_lt(q_new, P.q_cut)) q_new = 0.;
        }
    }
    const double sst = ss_guard(over_rho<UNIT_RHO>((pbvc * e_new + vnewc * vnewc * bvc * p_new), P));
    m.ss[i] = sst;
    m.p[i] = p_new;
    m.e[i] = e_new;
    m.q[i] = q_new;
    return sst;
}

#else
// Fast variants. The pressure coefficient bvc = 2/3 (comp + 1) is 2/3 / v
// for comp = 1/v - 1, the reference's vhalf = 1 / (1 + compHalf) is vchalf
// itself, and the sound-speed term v^2 bvc p is 2/3 v p: each pass forms two
// reciprocals instead of three and each sound speed takes one multiply-add.
// The eosvmin override (compHalf = comp) makes the half step use vnewc, and
// the eosvmax override (comp = compHalf = 0) makes bvc = 2/3, vhalf = 1 and
// the full-step term 2/3 vnewc^2 p. The repeat loop stays real work as in
// the exact variant.
__device__ __forceinline__ double pressure(double bvc, double e, double vnewc, const lulesh_params& P) {
    double nv = pmul(bvc, e);
    if (f_abs_lt(nv, P.p_cut) || f_ge(vnewc, P.eosvmax)) nv = 0.0;
    if (f_lt(nv, P.pmin)) nv = P.pmin;
    return nv;
}

template <bool UNIT_RHO>
__device__ __forceinline__ double eos_body(const Mesh& m, int i, double vnewc, int rep) {
    const lulesh_params& P = m.prm;
    const double cls = 2.0 / 3.0;
    double e_new = 0., p_new = 0., q_new = 0., vf = vnewc;
    const bool vmin_on = !f_is_zero(P.eosvmin), vmax_on = !f_is_zero(P.eosvmax);
    for (int r = 0; r < rep; ++r) {
        asm volatile("" ::: "memory");
        asm volatile("" : "+d"(vnewc));
        const double e_old = m.e[i], delvc = m.delv[i], q_old = m.q[i];
        double p_old = m.p[i];
        const double qq_old = m.qq[i], ql_old = m.ql[i];
        const double vchalf = vnewc - delvc * .5;
        double bvcf = pmul(cls, rcp(vnewc)), bvch = pmul(cls, rcp(vchalf));
        double vh = vchalf;
        vf = vnewc;
        if (vmin_on && f_le(vnewc, P.eosvmin)) {
            bvch = bvcf;
            vh = vnewc;
        }
        if (vmax_on && f_ge(vnewc, P.eosvmax)) {
            p_old = 0.;
            bvcf = bvch = cls;
            vh = 1.0;
            vf = vnewc * vnewc;
        }
        const double pq_old = p_old + q_old;
        const double hdelv = pmul(0.5, delvc);
        // predictor
        e_new = fma(-hdelv, pq_old, e_old);
        if (f_lt(e_new, P.emin)) e_new = P.emin;
        const double pHalf = pressure(bvch, e_new, vnewc, P);
        if (f_gt(delvc, 0.)) q_new = 0.;
        else q_new = fma(q_sound(over_rho<UNIT_RHO>(pmul(cls, fma(vh, pHalf, e_new)), P)), ql_old, qq_old);
        const double pq_half = pHalf + q_new;
        e_new = fma(hdelv, fma(-4.0, pq_half, pmul(3.0, pq_old)), e_new);
        if (f_abs_lt(e_new, P.e_cut)) e_new = 0.0;
        if (f_lt(e_new, P.emin)) e_new = P.emin;
        p_new = pressure(bvcf, e_new, vnewc, P);
        // corrector
        double q_tilde;
        if (f_gt(delvc, 0.)) q_tilde = 0.;
        else q_tilde = fma(q_sound(over_rho<UNIT_RHO>(pmul(cls, fma(vf, p_new, e_new)), P)), ql_old, qq_old);
        e_new = fma(-(fma(-8.0, pq_half, pmul(7.0, pq_old)) + (p_new + q_tilde)), pmul(delvc, 1.0 / 6.0), e_new);
        if (f_abs_lt(e_new, P.e_cut)) e_new = 0.;
        if (f_lt(e_new, P.emin)) e_new = P.emin;
        p_new = pressure(bvcf, e_new, vnewc, P);
        if (f_le(delvc, 0.)) {
            q_new = fma(q_sound(over_rho<UNIT_RHO>(pmul(cls, fma(vf, p_new, e_new)), P)), ql_old, qq_old);
            if (f_abs_lt(q_new, P.q_cut)) q_new = 0.;
        }
    }
    const double sst = ss_guard(over_rho<UNIT_RHO>(pmul(cls, fma(vf, p_new, e_new)), P));
    m.ss[i] = sst;
    m.p[i] = p_new;
    m.e[i] = e_new;
    m.q[i] = q_new;
    return sst;
}
#endif

__device__ __forceinline__ double eos_element(const Mesh& m, int i, double vnewc, int rep) {
    return m.prm.refdens == 1.0 ? eos_body<true>(m, i, vnewc, rep) : eos_body<false>(m, i, vnewc, rep);
}

// Courant and hydro candidates of one element (lulesh.cc:1938-1974); false
// where vdov == 0 (the element does not constrain).
__device__ __forceinline__ bool dt_candidates(const lulesh_params& P, double ss, double vdov,
                                              double arealg, double& courant, double& hydro) {
    if (f_is_zero(vdov)) return false;
    const double qqc2 = 64.0 * P.qqc * P.qqc;
#if LULESH_EXACT
    double dtf = ss * ss;
    if (f_lt(vdov, 0.0)) dtf += qqc2 * arealg * arealg * vdov * vdov;
#else
    double dtf = pmul(ss, ss);
    if (f_lt(vdov, 0.0)) dtf = fma(pmul(qqc2, pmul(arealg, arealg)), pmul(vdov, vdov), dtf);
#endif
    courant = div_sqrt(arealg, dtf);  // arealg / sqrt(dtf)
    hydro = quot(P.dvovmax, fabs(vdov) + 1.e-20);
    return true;
}

// The same constraints folded into running minima (the candidates of the
// step's own state are non-negative: ss, arealg >= 0).
__device__ __forceinline__ void dt_constraints(const lulesh_params& P, double ss, double vdov,
                                               double arealg, double& dtc, double& dth) {
    double courant, hydro;
    if (!dt_candidates(P, ss, vdov, arealg, courant, hydro)) return;
    dtc = nonneg_min(dtc, courant);
    dth = nonneg_min(dth, hydro);
}

// Block-wide min of (a, b); the result is valid in thread 0.
__device__ __forceinline__ void block_min2(double& a, double& b) {
    __shared__ double sa[32], sb[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = fmin(a, __shfl_down_sync(0xffffffffu, a, o));
        b = fmin(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        a = lane < nw ? sa[lane] : 1.0e+20;
        b = lane < nw ? sb[lane] : 1.0e+20;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = fmin(a, __shfl_down_sync(0xffffffffu, a, o));
            b = fmin(b, __shfl_down_sync(0xffffffffu, b, o));
        }
    }
}

// Publishes this block's (dtc, dth) minima; the last block to arrive reduces
// all partials into m.result (with accumulate, into the minima already
// there: a launch over part of the elements) and re-arms the counter. One
// pass, no second launch. Every thread of the block must call it.
__device__ __forceinline__ void finish_dt_reduction(const Mesh& m, double dtc, double dth,
                                                    bool accumulate = false) {
    block_min2(dtc, dth);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        m.partials[blockIdx.x].dtc = dtc;
        m.partials[blockIdx.x].dth = dth;
        __threadfence();
        const unsigned ticket = atomicAdd(&m.result->blocks_done, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 1.0e+20, b = 1.0e+20;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        a = fmin(a, __ldcg(&m.partials[k].dtc));
        b = fmin(b, __ldcg(&m.partials[k].dth));
    }
    __syncthreads();  // block_min2's shared scratch is reused
    block_min2(a, b);
    if (threadIdx.x == 0) {
        m.result->dtcourant = accumulate ? fmin(a, m.result->dtcourant) : a;
        m.result->dthydro = accumulate ? fmin(b, m.result->dthydro) : b;
        m.result->blocks_done = 0u;
    }
}

// --- node update ------------------------------------------------------------

// Acceleration, symmetry-plane zeroing, velocity with u_cut and position of
// node n from its gathered force (lulesh.cc:1115-1158, 566-588).
// The positions advanced are m.x, m.y, m.z, or px, py, pz when given (the
// drop-in call's uploaded coordinates); the result goes to m.x, m.y, m.z.
__device__ __forceinline__ void node_update(const Mesh& m, int n, double fx, double fy, double fz,
                                            double dt, const double* __restrict__ px = nullptr,
                                            const double* __restrict__ py = nullptr,
                                            const double* __restrict__ pz = nullptr) {
    m.fx[n] = fx;
    m.fy[n] = fy;
    m.fz[n] = fz;
#if LULESH_EXACT
    const double mass = LD(m.nodalMass + n);
    double ax = fx / mass, ay = fy / mass, az = fz / mass;
#else
    // fast variants: the reciprocal nodal mass is precomputed once per handle
    const double im = LD(m.invMass + n);
    double ax = pmul(fx, im), ay = pmul(fy, im), az = pmul(fz, im);
#endif
    const unsigned sym = LD(m.nodeSymm + n);
    if (sym & 1u) ax = 0.0;
    if (sym & 2u) ay = 0.0;
    if (sym & 4u) az = 0.0;
    m.xdd[n] = ax;
    m.ydd[n] = ay;
    m.zdd[n] = az;
    const double u_cut = m.prm.u_cut;
    double vx = m.xd[n] + ax * dt;
    if (f_abs_lt(vx, u_cut)) vx = 0.0;
    double vy = m.yd[n] + ay * dt;
    if (f_abs_lt(vy, u_cut)) vy = 0.0;
    double vz = m.zd[n] + az * dt;
    if (f_abs_lt(vz, u_cut)) vz = 0.0;
    m.xd[n] = vx;
    m.yd[n] = vy;
    m.zd[n] = vz;
    const double x0 = px ? LD(px + n) : m.x[n];
    const double y0 = py ? LD(py + n) : m.y[n];
    const double z0 = pz ? LD(pz + n) : m.z[n];
    m.x[n] = x0 + vx * dt;
    m.y[n] = y0 + vy * dt;
    m.z[n] = z0 + vz * dt;
}

// CheckAndUpdateVolumeForElems (lulesh.cc:1252-1272): checks the old v, then
// stores vnew snapped to 1 within v_cut.
__device__ __forceinline__ void update_volume(const Mesh& m, int i, double vold, double relv) {
    const lulesh_params& P = m.prm;
    double vc = vold;
    if (!f_is_zero(P.eosvmin) && f_lt(vc, P.eosvmin)) vc = P.eosvmin;
    if (!f_is_zero(P.eosvmax) && f_gt(vc, P.eosvmax)) vc = P.eosvmax;
    if (f_neg(vc)) raise_error(m.result, i, PHASE_KINEMATICS);
    double vn = relv;
    if (f_abs_lt(vn - 1.0, P.v_cut)) vn = 1.0;
    m.v[i] = vn;
}

}  // namespace LULESH_VARIANT
}  // namespace lulesh
