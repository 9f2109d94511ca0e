// Double-float arithmetic (an unevaluated sum hi + lo of two FP32 values,
// 48-bit significand) and exact FP32 -> FP64 assembly without the FP64
// pipe, for the residuals and updates of the refinement kernels: GB300's FP64
// rate is 1/64 of its FP32 rate.
#pragma once
#include "tridi_device.cuh"

namespace tridi {

// Exact float -> double by assembling the IEEE-754 fields (normal numbers and
// zeros; subnormals, infinities and NaNs take the conversion instruction).
// Keeps the residual's conversions off the FP64 pipe.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return (double)f;
}

// The double nearest hi + lo (ties to even) for a normalised double-float
// pair (|lo| <= ulp_float(hi) / 2), without the FP64 pipe.  With u = hi's
// double ulp, k = lo / u rounded half to even is one exact FP32 scaling by a
// power of two and one float -> int conversion (|k| <= 2^28).  hi + lo stays
// in hi's binade (it cannot reach the next power of two, and cannot fall
// below hi's own unless hi is a power of two and lo has the opposite sign),
// so the result's bit pattern is hi's moved by k units, and as hi's double
// has 29 zero low bits, k's parity is the sum's: the ties go to even.  hi
// below 2^-75 (where 1/u leaves FP32's range), non-normal hi and a
// power-of-two hi under a negative lo take one FP64 add.
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  const unsigned uh = __float_as_uint(hi), ul = __float_as_uint(lo);
  const unsigned eh = (uh >> 23) & 0xffu;
  const bool pow2_down = ((uh ^ ul) >> 31) != 0u && (uh & 0x7fffffu) == 0u && (ul & 0x7fffffffu) != 0u;
  if (eh >= 52u && eh <= 254u && !pow2_down) {
    const float inv_u = __uint_as_float((306u - eh) << 23);  // 2^(52 - unbiased exponent of hi)
    const int k = __float2int_rn(__fmul_rn(lo, inv_u));
    if (k >= -(1 << 28) && k <= (1 << 28)) {
      const long long h = __double_as_longlong(f2d_exact(hi));
      return __longlong_as_double((int)uh < 0 ? h - k : h + k);
    }
  }
  return f2d_exact(hi) + f2d_exact(lo);
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}
// Dekker's FastTwoSum (|a| >= |b| or a == 0).
__device__ __forceinline__ float fast_two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
  return s;
}

// (hi, lo) + v for a normalised pair and an FP32 v: TwoSum of the high
// words, the low word added to the error, renormalised by FastTwoSum.
__device__ __forceinline__ float2 df_add(float2 x, float v) {
  float e;
  const float s = two_sum(x.x, v, e);
  float lo;
  const float hi = fast_two_sum(s, __fadd_rn(e, x.y), lo);
  return make_float2(hi, lo);
}

// d - a xm - b x0 - c xp for FP32 x, as an unevaluated sum s + t: the
// products exactly (TwoProd by FMA), summed with TwoSum, their rounding
// errors gathered in the FP32 term t.
__device__ __forceinline__ float2 residual_parts(float a, float b, float c, float d, float xm, float x0, float xp) {
  const float pb = __fmul_rn(b, x0), pa = __fmul_rn(a, xm), pc = __fmul_rn(c, xp);
  float t = -(fmaf(b, x0, -pb) + fmaf(a, xm, -pa) + fmaf(c, xp, -pc));
  float e;
  float s = two_sum(d, -pb, e);
  t += e;
  s = two_sum(s, -pa, e);
  t += e;
  s = two_sum(s, -pc, e);
  t += e;
  return make_float2(s, t);
}

// The same for FP32 x, rounded to FP32.
__device__ __forceinline__ float f_residual(float a, float b, float c, float d, float xm, float x0, float xp) {
  const float2 st = residual_parts(a, b, c, d, xm, x0, xp);
  return __fadd_rn(st.x, st.y);
}

// The same for double-float x (the low words' products added to t in FP32).
__device__ __forceinline__ float df_residual(float a, float b, float c, float d, float2 xm, float2 x0, float2 xp) {
  const float2 st = residual_parts(a, b, c, d, xm.x, x0.x, xp.x);
  float t = st.y;
  t = fmaf(-b, x0.y, t);
  t = fmaf(-a, xm.y, t);
  t = fmaf(-c, xp.y, t);
  return __fadd_rn(st.x, t);
}

// ---- the same on two independent rows at once ----------------------------
// Component-wise, operation for operation the scalar routines above, in the
// paired FP32 instructions of sm_100+ (FADD2 / FMUL2 / FFMA2, round to nearest
// like __fadd_rn / __fmul_rn / fmaf): bit-identical results, half the issue
// slots.
__device__ __forceinline__ float2 df2_neg(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ float2 two_sum2(float2 a, float2 b, float2& e) {
  const float2 s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, df2_neg(a));
  e = __fadd2_rn(__fadd2_rn(a, df2_neg(__fadd2_rn(s, df2_neg(bb)))), __fadd2_rn(b, df2_neg(bb)));
  return s;
}
// residual_parts for two rows.
__device__ __forceinline__ void residual_parts2(float2 a, float2 b, float2 c, float2 d, float2 xm, float2 x0,
                                                float2 xp, float2& s, float2& t) {
  const float2 pb = __fmul2_rn(b, x0), pa = __fmul2_rn(a, xm), pc = __fmul2_rn(c, xp);
  t = df2_neg(__fadd2_rn(__fadd2_rn(__ffma2_rn(b, x0, df2_neg(pb)), __ffma2_rn(a, xm, df2_neg(pa))),
                         __ffma2_rn(c, xp, df2_neg(pc))));
  float2 e;
  s = two_sum2(d, df2_neg(pb), e);
  t = __fadd2_rn(t, e);
  s = two_sum2(s, df2_neg(pa), e);
  t = __fadd2_rn(t, e);
  s = two_sum2(s, df2_neg(pc), e);
  t = __fadd2_rn(t, e);
}
// df_residual for two rows: x given as high words (xmh, x0h, xph) and low
// words (xml, x0l, xpl), each pair holding the two rows.
__device__ __forceinline__ float2 df_residual2(float2 a, float2 b, float2 c, float2 d, float2 xmh, float2 xml,
                                               float2 x0h, float2 x0l, float2 xph, float2 xpl) {
  float2 s, t;
  residual_parts2(a, b, c, d, xmh, x0h, xph, s, t);
  t = __ffma2_rn(df2_neg(b), x0l, t);
  t = __ffma2_rn(df2_neg(a), xml, t);
  t = __ffma2_rn(df2_neg(c), xpl, t);
  return __fadd2_rn(s, t);
}

}  // namespace tridi
