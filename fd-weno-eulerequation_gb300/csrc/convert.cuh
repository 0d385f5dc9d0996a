// FP64 <-> FP32 conversions on the integer ALU.
//
// On GB300 the conversion instructions between FP64 and FP32 issue on the
// FP64 pipe, which runs at 1/64 of the FP32 rate (1.0 vs 73 TFLOP/s
// measured); the FP32 form converts every staged state value and every RHS
// value, so it does the conversions with bit operations instead.
//
//  f64_to_f32: rounds toward zero (error < 1 FP32 ulp); magnitudes below
//              2^-126 become signed zero, above the FP32 range infinity; NaN
//              stays NaN.  Used only where the FP32 form reads the state.
//  f32_to_f64: exact for every finite float (FP32 subnormals become zero),
//              infinity and NaN preserved.
#pragma once

namespace wenofd {
namespace dev {

__device__ __forceinline__ float f64_to_f32(double d) {
  const unsigned hi = unsigned(__double2hiint(d));
  const unsigned lo = unsigned(__double2loint(d));
  const unsigned mag = hi & 0x7fffffffu;
  // (hi, lo) << 3 keeps the low 9 exponent bits and the top 23 mantissa bits
  // in place for FP32; subtracting 0x180 << 23 rebiases the exponent
  // (1023 - 127 = 896 = 0x380, congruent to 0x180 modulo 2^9), which leaves
  // bit 31 clear for every in-range magnitude; the sign is put back.
  const unsigned bits = (__funnelshift_l(lo, hi, 3) - 0xC0000000u) | (hi & 0x80000000u);
  if (mag < 0x38100000u) return __uint_as_float(hi & 0x80000000u);  // zero, subnormal, below 2^-126
  if (mag >= 0x47f00000u) {                                           // beyond FP32 range, inf, NaN
    const bool nan = mag > 0x7ff00000u || (mag == 0x7ff00000u && lo != 0u);
    return __uint_as_float((hi & 0x80000000u) | 0x7f800000u | (nan ? 0x400000u : 0u));
  }
  return __uint_as_float(bits);
}

__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned m = b & 0x7fffffu;
  unsigned hi, lo;
  if (e == 0) {  // zero (FP32 subnormals flush to zero)
    hi = sign;
    lo = 0;
  } else if (e == 0xffu) {
    hi = sign | 0x7ff00000u | (m >> 3);
    lo = m << 29;
  } else {
    hi = sign | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double(int(hi), int(lo));
}

// x * 2^-K on the integer ALU: exact, except that results that would be
// subnormal (below 2^-1022 in magnitude) become signed zero; infinity and NaN
// pass through.
template <int K>
__device__ __forceinline__ double scale_pow2_down(double x) {
  static_assert(K >= 1 && K < 16, "small power-of-two scales only");
  const unsigned hi = unsigned(__double2hiint(x));
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e == 0x7ffu) return x;
  if (e <= unsigned(K)) return __hiloint2double(int(hi & 0x80000000u), 0);
  return __hiloint2double(int(hi - (unsigned(K) << 20)), __double2loint(x));
}

}  // namespace dev
}  // namespace wenofd
