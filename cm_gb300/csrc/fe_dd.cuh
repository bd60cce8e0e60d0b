// Double-float arithmetic ("dd": an unevaluated sum hi + lo of two FP32
// numbers, about 48 significant bits) for the high-precision phases of the
// mixed-precision assembly.  GB300 executes FP64 at a small fraction of its
// FP32 rate; these routines run on the FP32 pipes instead.
//
// Built from the classical error-free transformations: Knuth's TwoSum,
// Dekker's FastTwoSum, and the FMA-based exact product (TwoProduct).  The
// addition is the "sloppy" double-word sum (TwoSum of the high parts plus the
// low parts, renormalised), whose error is bounded by a small multiple of
// 2^-48 (|a| + |b|) — the same error model as a long FP64 sum, with a
// larger unit.  All primitives use the _rn intrinsics so the compiler cannot
// contract or reassociate them.
#pragma once
#include <cuda_runtime.h>

namespace {

struct dd {
  float hi, lo;
};

__device__ __forceinline__ dd dd_quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ void dd_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ dd operator+(dd a, dd b) {
  float s, e;
  dd_two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return dd_quick_two_sum(s, e);
}

__device__ __forceinline__ dd operator-(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }

__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd_quick_two_sum(p, e);
}

__device__ __forceinline__ dd operator/(dd a, dd b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  // r = a - q1 * b, exactly enough for the second quotient digit
  const float p = __fmul_rn(q1, b.hi);
  const float pe = __fmaf_rn(q1, b.hi, -p);
  float s, e;
  dd_two_sum(a.hi, -p, s, e);
  e = __fsub_rn(__fadd_rn(e, a.lo), __fmaf_rn(q1, b.lo, pe));
  const float r = __fadd_rn(s, e);
  const float q2 = __fdiv_rn(r, b.hi);
  return dd_quick_two_sum(q1, q2);
}

__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }

__device__ __forceinline__ dd to_dd(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ dd to_dd(float x) { return {x, 0.0f}; }
__device__ __forceinline__ double to_double(dd a) { return (double)a.hi + (double)a.lo; }

// Generic helpers used by code templated on the high-precision type H
// (double or dd).
__device__ __forceinline__ double hfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ dd hfma(dd a, dd b, dd c) { return a * b + c; }
__device__ __forceinline__ double habs(double a) { return fabs(a); }
__device__ __forceinline__ dd habs(dd a) { return a.hi < 0.0f ? -a : a; }
__device__ __forceinline__ bool hpos(double a) { return a > 0.0; }
__device__ __forceinline__ bool hpos(dd a) { return a.hi > 0.0f; }
__device__ __forceinline__ bool hfinite(double a) { return isfinite(a); }
__device__ __forceinline__ bool hfinite(dd a) { return isfinite(a.hi) && isfinite(a.lo); }
__device__ __forceinline__ float hf(double a) { return (float)a; }
__device__ __forceinline__ float hf(dd a) { return a.hi + a.lo; }
__device__ __forceinline__ double hd(double a) { return a; }
__device__ __forceinline__ double hd(dd a) { return to_double(a); }
template <class H>
__device__ __forceinline__ H hval(double x);
template <>
__device__ __forceinline__ double hval<double>(double x) { return x; }
template <>
__device__ __forceinline__ dd hval<dd>(double x) { return to_dd(x); }
// x^(-1/3) and exp: evaluated in FP64 (one call per Gauss point) and rounded
// to H.
__device__ __forceinline__ double hrcbrt(double x) { return rcbrt(x); }
__device__ __forceinline__ dd hrcbrt(dd x) { return to_dd(rcbrt(to_double(x))); }
__device__ __forceinline__ double hexp(double x) { return exp(x); }
__device__ __forceinline__ dd hexp(dd x) { return to_dd(exp(to_double(x))); }

}  // namespace
