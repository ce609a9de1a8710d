// Double-float ("double-word") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The operations are the published error-free
// transformations and double-word algorithms:
//   * TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and Fast2Sum (Dekker 1971) give the
//     rounded sum and its exact error; 2Prod gives the rounded product and its
//     exact error with one FMA.
//   * Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
//     building blocks of double-word arithmetic", ACM TOMS 44(2), 2017:
//     DWPlusFP (Alg. 4), SloppyDWPlusDW (Alg. 5), DWTimesFP (Alg. 9),
//     DWTimesDW (Alg. 11).
//   * Sums of products accumulate the rounded head products with TwoSum and
//     every error term (product errors, cross terms, TwoSum errors) in one
//     float, normalised once at the end (the compensated dot product of Ogita,
//     Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6),
//     2005, Alg. 5.3, with double-word operands).  Its error is bounded by a
//     small multiple of 2^-48 times the sum of |x_i y_i|: the bound of an FP64
//     dot product with 2^-48 in place of 2^-53.
// The sums and differences are written with the _rn intrinsics so that no
// contraction or reordering can touch the error terms.  The exponent range is
// FP32's.
#pragma once

#include <cuda_runtime.h>

namespace tg {
namespace ff {

struct dfloat {
  float hi, lo;
};

__device__ __forceinline__ dfloat make(float hi, float lo) {
  dfloat r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// nearest double-float of a double (hi + lo carries 48 of its 53 bits)
__device__ __forceinline__ dfloat from_double(double d) {
  const float hi = __double2float_rn(d);
  return make(hi, __double2float_rn(d - (double)hi));
}
__device__ __forceinline__ double to_double(dfloat a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfloat from_float2(float2 v) { return make(v.x, v.y); }
__device__ __forceinline__ float2 to_float2(dfloat a) { return make_float2(a.hi, a.lo); }

// TwoSum: s = fl(a + b), e = a + b - s exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// Fast2Sum, valid when a == 0 or |a| >= |b|
__device__ __forceinline__ dfloat fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// DWPlusFP: (x + b), relative error <= 2 u^2
__device__ __forceinline__ dfloat add(dfloat x, float b) {
  float sh, sl;
  two_sum(x.hi, b, sh, sl);
  return fast_two_sum(sh, __fadd_rn(x.lo, sl));
}
// SloppyDWPlusDW: absolute error <= 3 u^2 (|x| + |y|), which is the bound the
// FP64 sums it replaces have (with u = 2^-24 squared in place of 2^-53)
__device__ __forceinline__ dfloat add(dfloat x, dfloat y) {
  float sh, sl;
  two_sum(x.hi, y.hi, sh, sl);
  return fast_two_sum(sh, __fadd_rn(sl, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ dfloat neg(dfloat x) { return make(-x.hi, -x.lo); }
__device__ __forceinline__ dfloat sub(dfloat x, dfloat y) { return add(x, neg(y)); }

// DWTimesFP: relative error <= 2 u^2
__device__ __forceinline__ dfloat mul(dfloat x, float y) {
  const float ch = __fmul_rn(x.hi, y);
  const float cl1 = __fmaf_rn(x.hi, y, -ch);
  return fast_two_sum(ch, __fmaf_rn(x.lo, y, cl1));
}
// DWTimesDW (FMA form): relative error <= 5 u^2
__device__ __forceinline__ dfloat mul(dfloat x, dfloat y) {
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl = __fmul_rn(x.hi, y.lo);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl);
  return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}

// Accumulator of a sum of double-float products (see the header comment):
// s carries the TwoSum chain of the head products, t every lower-order term.
struct Dot {
  float s, t;
};
__device__ __forceinline__ Dot dot_zero() {
  Dot d;
  d.s = 0.f;
  d.t = 0.f;
  return d;
}
__device__ __forceinline__ Dot dot_from(dfloat c) {
  Dot d;
  d.s = c.hi;
  d.t = c.lo;
  return d;
}
// d += x * y
__device__ __forceinline__ void dot_fma(Dot& d, dfloat x, dfloat y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float pe = __fmaf_rn(x.hi, y.hi, -p);
  const float cross = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.hi));
  float s, e;
  two_sum(d.s, p, s, e);
  d.s = s;
  d.t = __fadd_rn(d.t, __fadd_rn(__fadd_rn(pe, cross), e));
}
// d -= x * y
__device__ __forceinline__ void dot_fms(Dot& d, dfloat x, dfloat y) { dot_fma(d, neg(x), y); }
__device__ __forceinline__ dfloat dot_value(Dot d) {
  float s, e;
  two_sum(d.s, d.t, s, e);
  return make(s, e);
}

// 1/x by one Newton-Raphson step of cubic order from the correctly rounded
// FP32 reciprocal r0: with e = 1 - x r0 (formed exactly up to the last
// product), 1/x = r0 (1 + e + e^2 + ...); |e| <= 2^-24, so the truncation
// after e^2 is below 2^-72 and the rounding of the correction term bounds the
// error near 2^-47.
__device__ __forceinline__ dfloat rcp(dfloat x) {
  const float r0 = __frcp_rn(x.hi);
  const float p = __fmul_rn(x.hi, r0);
  const float pe = __fmaf_rn(x.hi, r0, -p);
  // 1 - p is exact (Sterbenz: p is within a few ulps of 1)
  const float e = __fmaf_rn(-x.lo, r0, __fsub_rn(__fsub_rn(1.0f, p), pe));
  const float c = __fmul_rn(r0, __fmaf_rn(e, e, e));
  return fast_two_sum(r0, c);
}

// x^(-1/3) for x > 0 from the FP32 estimate y0 = rcbrtf(x.hi): with
// e = 1 - x y0^3 (double-float), x^(-1/3) = y0 (1 - e)^(-1/3)
// = y0 (1 + e/3 + 2 e^2 / 9 + 14 e^3 / 81 + ...); |e| is a few 2^-24, so two
// terms leave a truncation near 2^-66.
__device__ __forceinline__ dfloat rcbrt(dfloat x) {
  const float y0 = rcbrtf(x.hi);
  const float q = __fmul_rn(y0, y0);
  const dfloat y2 = make(q, __fmaf_rn(y0, y0, -q));  // y0^2 exactly
  const dfloat y3 = mul(y2, y0);
  const dfloat t = mul(x, y3);
  const float e = __fsub_rn(__fsub_rn(1.0f, t.hi), t.lo);
  const float c = __fmul_rn(y0, __fmul_rn(e, __fmaf_rn(e, 2.0f / 9.0f, 1.0f / 3.0f)));
  return fast_two_sum(y0, c);
}

}  // namespace ff
}  // namespace tg
