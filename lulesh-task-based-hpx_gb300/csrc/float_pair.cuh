// The float-pair split of the mixed variant's node mirrors, shared by its
// kernels and by the accuracy probe that checks it bit for bit against the
// conversion instructions. Include after step_math.cuh (it uses that
// variant's round_to_float_bits / float_from_rounded).
#pragma once

namespace lulesh {
namespace LULESH_VARIANT {

// The float-pair mirror of v, (hi, lo) = (fl(v), fl(v - hi)) with fl the
// round-to-nearest-even conversion, on the integer pipe (narrow's rounding of
// the bit pattern; v - hi is one exact double subtraction). Bit for bit the
// conversions' result for |v| in [2^-74, float's largest], where lo is zero
// or a normal float; zeros map to zeros and other values take the conversion
// instructions out of line.
__device__ __noinline__ float2 split_convert(double v) {
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - double(hi)));
}

__device__ __forceinline__ float2 split(double v) {
    const unsigned long long b = __double_as_longlong(v);
    const unsigned e = unsigned(b >> 52) & 0x7ffu;
    if ((b << 1) == 0ull) return make_float2(__uint_as_float(unsigned(b >> 32)), 0.0f);  // +-0
    if (e < 949u || e > 1150u) return split_convert(v);
    const unsigned long long hb = round_to_float_bits(b);
    const unsigned long long lb = __double_as_longlong(v - __longlong_as_double(hb));
    return make_float2(float_from_rounded(hb), (lb << 1) == 0ull ? 0.0f : float_from_rounded(round_to_float_bits(lb)));
}

}  // namespace LULESH_VARIANT
}  // namespace lulesh
