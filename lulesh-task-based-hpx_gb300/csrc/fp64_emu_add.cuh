// Double-precision add on the integer pipes, for the measurement probes only
// (liblulesh_probe.so): no step kernel uses it. Measured on this machine's
// GB300 it is exact (the FP64 pipe's bits) but slow: 2.4e11 adds/s alone,
// 4.7e11/s with half the chains on each pipe, below the FP64 pipe's 5.3e11/s
// alone, because its alignment, normalisation and rounding take several
// times the integer instructions of dmul_ipipe; the double force kernel's
// corner sums written with it ran 2.60 -> 3.04 ms at s=150.
#pragma once

#include "fp64_emu.cuh"

namespace lulesh {

// Double-precision add on the integer pipes: the IEEE 754 binary64 sum a + b
// rounded to nearest even, formed from the operands' bit patterns with 64-bit
// integer adds, shifts and a count of leading zeros: the same bits as the
// FP64 pipe's add (a NaN result may carry another NaN payload), the
// counterpart of dmul_ipipe for adds. Finite operands, subnormal ones included, take the inline path
// (a subnormal counts as exponent 1 without the leading bit, the encoding's
// own scale); an infinite or NaN operand goes to dadd_ipipe_special, out of
// line and also integer-only.
static __device__ __noinline__ double dadd_ipipe_special(double a, double b) {
    const unsigned long long A = dmul_bits(a), B = dmul_bits(b);
    const unsigned long long inf2 = 0xFFE0000000000000ull;  // an infinity's bits shifted left by one
    const bool a_nan = (A << 1) > inf2, b_nan = (B << 1) > inf2;
    const bool a_inf = (A << 1) == inf2, b_inf = (B << 1) == inf2;
    if (a_nan || b_nan || (a_inf && b_inf && ((A ^ B) & kDmulSign)))
        return __longlong_as_double(static_cast<long long>(0x7FFFFFFFFFFFFFFFull));  // NaN
    return a_inf ? a : b;  // the infinite operand (a finite other one does not change it)
}

static __device__ __forceinline__ double dadd_ipipe(double a, double b) {
    const unsigned long long A = dmul_bits(a), B = dmul_bits(b);
    const unsigned long long am = A & ~kDmulSign, bm = B & ~kDmulSign;  // magnitudes
    if (am >= 0x7FF0000000000000ull || bm >= 0x7FF0000000000000ull) return dadd_ipipe_special(a, b);
    // x: the operand of larger magnitude, whose sign the result takes unless it is zero
    const bool swap = bm > am;
    const unsigned long long X = swap ? B : A, xm = swap ? bm : am, ym = swap ? am : bm;
    const bool sub = ((A ^ B) & kDmulSign) != 0ull;
    const unsigned ex = unsigned(xm >> 52), ey = unsigned(ym >> 52);
    // significands with 10 bits below the last place (guard bits, the lowest a sticky bit)
    const unsigned long long mx = ((xm & kDmulFrac) | (ex ? kDmulHidden : 0ull)) << 10;
    const unsigned long long my = ((ym & kDmulFrac) | (ey ? kDmulHidden : 0ull)) << 10;
    int e = int(max(ex, 1u));
    const unsigned d = unsigned(e) - max(ey, 1u);
    // y aligned to x, the bits shifted out folded into the lowest bit
    unsigned long long yal;
    if (d == 0u) yal = my;
    else if (d < 64u) yal = (my >> d) | static_cast<unsigned long long>((my << (64u - d)) != 0ull);
    else yal = static_cast<unsigned long long>(my != 0ull);
    unsigned long long s = sub ? mx - yal : mx + yal;  // both below 2^63: no overflow
    if (s == 0ull)  // exact cancellation gives +0; -0 + -0 stays -0
        return __longlong_as_double(static_cast<long long>(sub ? 0ull : X));
    // leading bit to bit 62, or as far as exponent 1 allows (a subnormal sum)
    if (s >> 63) {
        s = (s >> 1) | (s & 1ull);
        ++e;
    } else {
        const int sh = min(__clzll(static_cast<long long>(s)) - 1, e - 1);
        s <<= sh;
        e -= sh;
    }
    // round to nearest, ties to even, at bit 10
    unsigned long long q = s >> 10;
    const unsigned r = unsigned(s) & 0x3FFu;
    q += static_cast<unsigned long long>((r > 0x200u) | ((r == 0x200u) & unsigned(q & 1ull)));
    const unsigned long long sign = X & kDmulSign;
    if (e >= 2047) return __longlong_as_double(static_cast<long long>(sign | 0x7FF0000000000000ull));
    // (e - 1) << 52 plus the significand with its leading bit: a rounding carry
    // moves into the exponent, and a subnormal sum (e = 1, no leading bit)
    // encodes as itself
    return __longlong_as_double(static_cast<long long>(sign | ((static_cast<unsigned long long>(e - 1) << 52) + q)));
}

}  // namespace lulesh
