// Float-float arithmetic for the mixed form.  A value is the unevaluated sum
// hi + lo of two floats (|lo| <= ulp(hi)), about 48 significant bits; sums
// and products use the error-free transformations of Knuth (TwoSum) and
// Dekker (TwoProduct, here with one fused multiply-add), as in the
// double-double literature (Dekker 1971; Hida, Li and Bailey 2001).  Every
// operation is written with the round-to-nearest intrinsics, which the
// compiler never contracts, so the transformations hold in translation
// units compiled with or without FMA contraction.
#pragma once
#include <cuda_runtime.h>

namespace mmh {

struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ FF ff_quick(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  FF s = ff_two_sum(a.hi, b.hi), t = ff_two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = ff_quick(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return ff_quick(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_quick(p, e);
}
// p2 a power of two: exact
__device__ __forceinline__ FF ff_scale(FF a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }
__device__ __forceinline__ FF ff_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(__dsub_rn(x, (double)h))};
}
__device__ __forceinline__ FF ff_div(FF a, FF b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const FF r = ff_sub(a, ff_mul({q1, 0.0f}, b));
  return ff_quick(q1, __fdiv_rn(r.hi, b.hi));
}

// x as a float-float pair from its bit pattern, with integer and FP32
// operations only: GB300 runs FP64 conversions at its FP64 rate (about two
// per clock per SM), so ff_of costs as much as three FP64 operations.  hi is
// x truncated to 24 significant bits (exact in a float), lo the remaining 29
// mantissa bits rounded to 24: |hi + lo - x| <= 2^-48 |x|.  |x| >= 2^-74 keeps
// both parts; 2^-126 <= |x| < 2^-74 keeps hi only (error < 2^-23 |x|); |x| <
// 2^-126 gives 0.  Inf and NaN give hi = Inf / NaN, lo = 0; |x| >= 2^128
// gives hi = Inf.
__device__ __forceinline__ FF ff_of_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const unsigned sign = h32 & 0x80000000u;
  const int E = (int)((h32 >> 20) & 0x7ffu);  // biased FP64 exponent
  if (E < 897) return {__uint_as_float(sign), 0.0f};
  if (E > 1150)
    return {__uint_as_float(sign | 0x7f800000u | ((E == 2047 && ((h32 & 0xfffffu) | l32)) ? 0x400000u : 0u)), 0.0f};
  const float hi = __uint_as_float(sign | ((unsigned)(E - 896) << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
  if (E < 949) return {hi, 0.0f};
  // the low 29 bits m as a float: both halves are exact (magic-number
  // conversion of integers below 2^23), their sum rounds once
  const unsigned m = l32 & 0x1fffffffu;
  const float mh = __fsub_rn(__uint_as_float(0x4b000000u | (m >> 23)), 8388608.0f);
  const float ml = __fsub_rn(__uint_as_float(0x4b000000u | (m & 0x7fffffu)), 8388608.0f);
  const float r = __fmaf_rn(mh, 8388608.0f, ml);
  // times 2^(E - 1075): a float with biased exponent E - 1075 + 127 >= 1
  const float lo = __fmul_rn(r, __uint_as_float((unsigned)(E - 948) << 23));
  return {hi, sign ? -lo : lo};
}
// x truncated to a float from its bit pattern (integer operations only):
// |x - f| < 2^-23 |x| + 2^-126.  Returns false (f = 0) for Inf, NaN and
// |x| >= 2^128.
__device__ __forceinline__ bool f32_trunc_bits(double x, float& f) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const int E = (int)((h32 >> 20) & 0x7ffu);
  if (E > 1150) {
    f = 0.0f;
    return false;
  }
  f = E < 897 ? __uint_as_float(h32 & 0x80000000u)
              : __uint_as_float((h32 & 0x80000000u) | ((unsigned)(E - 896) << 23) | ((h32 & 0xfffffu) << 3) |
                                (l32 >> 29));
  return true;
}
// a - b for two float-float values of like magnitude (neighbouring samples
// of a smooth field): TwoSum of the high parts, low parts added after.
// Error ~2^-48 max(|a|, |b|).
__device__ __forceinline__ FF ff_diff(FF a, FF b) {
  FF s = ff_two_sum(a.hi, -b.hi);
  s.lo = __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo));
  return ff_quick(s.hi, s.lo);
}
// a + b rounded to a float, for pairs of any magnitude (TwoSum of the high
// parts, then the low parts)
__device__ __forceinline__ float ff_sum_f(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return __fadd_rn(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// a - b rounded to a float (FP32 accuracy of the difference itself, however
// large a and b are against it)
__device__ __forceinline__ float ff_diff_f(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, -b.hi);
  return __fadd_rn(s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo)));
}

}  // namespace mmh
