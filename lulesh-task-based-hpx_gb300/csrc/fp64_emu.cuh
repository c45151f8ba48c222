// Double-precision multiply on the integer pipes.
//
// On GB300 the FP64 pipe issues about 600 G operations/s per GPU (1/64 of the
// float rate), while the integer pipes, nearly idle in the FP64-bound step
// kernels, issue 32 times that. dmul_ipipe forms the IEEE 754 binary64
// product rounded to nearest even from the operands' bit patterns with
// 32-bit integer multiply-adds, shifts and adds: the same bits as the FP64
// pipe's multiply (a NaN result may carry another NaN payload), so a kernel
// can move some of its multiplies there and run them beside the FP64 pipe's
// adds and multiply-adds. Measured on this machine's GB300: the FP64 pipe
// 5.0e11 multiplies/s, the integer form 4.8e11/s, both together 7.9e11/s;
// a 3x3 cofactor kernel with the first product of each cofactor on the
// integer pipes ran 1.37x faster.
//
// The common case (normal operands with a normal product, or a zero operand)
// is inline. Everything else (subnormal, infinite or NaN operands, products
// that overflow or underflow) goes to dmul_ipipe_rare, out of line and also
// integer-only, so no FP64 instruction is reachable from a call site.
#pragma once

namespace lulesh {

constexpr unsigned long long kDmulFrac = 0xFFFFFFFFFFFFFull;
constexpr unsigned long long kDmulHidden = 1ull << 52;
constexpr unsigned long long kDmulSign = 0x8000000000000000ull;

// The bit pattern of x through an opaque move: the optimizer cannot see that
// the integer tests below (zero, normal, exponent range) examine a double,
// so it cannot turn them back into floating-point compares, which would
// issue on the FP64 pipe (measured: about two per multiply without it).
static __device__ __forceinline__ unsigned long long dmul_bits(double x) {
    unsigned long long r;
    asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
    return r;
}

// 53-bit significands a, b -> their 106-bit product hi:lo.
static __device__ __forceinline__ void dmul_sig_product(unsigned long long a, unsigned long long b,
                                                        unsigned long long& hi, unsigned long long& lo) {
    lo = a * b;
    hi = __umul64hi(a, b);
}

// Rounds hi:lo (the product of two significands in [2^52, 2^53)) shifted
// right by `shift` bits, 52 <= shift <= 170, to the nearest integer, ties to
// even.
static __device__ __forceinline__ unsigned long long dmul_round_shift(unsigned long long hi, unsigned long long lo,
                                                                      unsigned shift) {
    unsigned long long q, rest;  // quotient and the remainder left-aligned in 64 bits
    bool sticky_below;           // remainder bits that did not fit in `rest`
    if (shift < 64u) {
        q = (hi << (64u - shift)) | (lo >> shift);
        rest = lo << (64u - shift);
        sticky_below = false;
    } else if (shift == 64u) {
        q = hi;
        rest = lo;
        sticky_below = false;
    } else if (shift < 128u) {
        const unsigned s = shift - 64u;
        q = hi >> s;
        rest = (hi << (64u - s)) | (lo >> s);
        sticky_below = (lo << (64u - s)) != 0ull;
    } else {  // the whole product is below half of the last place
        q = 0ull;
        rest = 0ull;
        sticky_below = (hi | lo) != 0ull;
    }
    const unsigned long long half = 0x8000000000000000ull;
    const bool up = rest > half || (rest == half && (sticky_below || (q & 1ull)));
    return q + (up ? 1ull : 0ull);
}

// The rare cases of dmul_ipipe, in integer arithmetic only.
static __device__ __noinline__ double dmul_ipipe_rare(double a, double b) {
    const unsigned long long A = dmul_bits(a), B = dmul_bits(b);
    const unsigned long long sign = (A ^ B) & kDmulSign;
    int ea = int(unsigned(A >> 52) & 0x7ffu), eb = int(unsigned(B >> 52) & 0x7ffu);
    unsigned long long ma = A & kDmulFrac, mb = B & kDmulFrac;
    const bool a_zero = ea == 0 && ma == 0ull, b_zero = eb == 0 && mb == 0ull;
    if (ea == 0x7ff || eb == 0x7ff) {
        if ((ea == 0x7ff && ma) || (eb == 0x7ff && mb) || (ea == 0x7ff && b_zero) || (eb == 0x7ff && a_zero))
            return __longlong_as_double(static_cast<long long>(0x7FFFFFFFFFFFFFFFull));  // NaN
        return __longlong_as_double(static_cast<long long>(sign | 0x7FF0000000000000ull));  // infinity
    }
    if (a_zero || b_zero) return __longlong_as_double(static_cast<long long>(sign));
    // significands in [2^52, 2^53); a subnormal's exponent becomes 1 - shift
    if (ea == 0) {
        const int s = __clzll(static_cast<long long>(ma)) - 11;
        ma <<= s;
        ea = 1 - s;
    } else {
        ma |= kDmulHidden;
    }
    if (eb == 0) {
        const int s = __clzll(static_cast<long long>(mb)) - 11;
        mb <<= s;
        eb = 1 - s;
    } else {
        mb |= kDmulHidden;
    }
    unsigned long long hi, lo;
    dmul_sig_product(ma, mb, hi, lo);
    const int sh = int(hi >> 41);
    const int e = ea + eb - 1023 + sh;  // biased exponent of the normalised result
    if (e >= 2047) return __longlong_as_double(static_cast<long long>(sign | 0x7FF0000000000000ull));
    if (e >= 1) {
        const unsigned long long m = dmul_round_shift(hi, lo, unsigned(52 + sh));
        // a rounding carry out of the significand moves into the exponent (2047: infinity)
        return __longlong_as_double(static_cast<long long>(sign | ((static_cast<unsigned long long>(e - 1) << 52) + m)));
    }
    // subnormal result: 1 - e more bits go below the last place; a rounding
    // carry into bit 52 gives the smallest normal number, as the encoding does
    const unsigned shift = unsigned(52 + sh + (1 - e));
    const unsigned long long m = shift > 170u ? 0ull : dmul_round_shift(hi, lo, shift);
    return __longlong_as_double(static_cast<long long>(sign | m));
}

static __device__ __forceinline__ double dmul_ipipe(double a, double b) {
    const unsigned long long A = dmul_bits(a), B = dmul_bits(b);
    const unsigned ea = unsigned(A >> 52) & 0x7ffu, eb = unsigned(B >> 52) & 0x7ffu;
    const unsigned long long sign = (A ^ B) & kDmulSign;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u) {  // a zero, subnormal, infinity or NaN
        if (((A << 1) == 0ull && eb != 0x7ffu) || ((B << 1) == 0ull && ea != 0x7ffu))
            return __longlong_as_double(static_cast<long long>(sign));  // 0 * finite
        return dmul_ipipe_rare(a, b);
    }
    // 53-bit significands and their 106-bit product hi:lo in [2^104, 2^106)
    unsigned long long hi, lo;
    dmul_sig_product((A & kDmulFrac) | kDmulHidden, (B & kDmulFrac) | kDmulHidden, hi, lo);
    const unsigned sh = unsigned(hi >> 41);  // 1 when the product is >= 2^105
    // the top 53 bits, and the bits below them left-aligned
    unsigned long long m = (hi << (12u - sh)) | (lo >> (52u + sh));
    const unsigned long long rest = lo << (12u - sh);
    // round to nearest, ties to even
    m += static_cast<unsigned long long>(rest > 0x8000000000000000ull) |
         (static_cast<unsigned long long>(rest == 0x8000000000000000ull) & (m & 1ull));
    const int e = int(ea) + int(eb) - 1023 + int(sh);  // biased exponent of the result
    if (e < 1 || e > 2046) return dmul_ipipe_rare(a, b);
    // (e - 1) << 52 plus the significand with its leading bit: a rounding
    // carry out of the significand moves into the exponent
    return __longlong_as_double(static_cast<long long>(sign | ((static_cast<unsigned long long>(e - 1) << 52) + m)));
}

}  // namespace lulesh
