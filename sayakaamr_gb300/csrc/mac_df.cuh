// Double-float arithmetic on the FP32 pipe.
//
// GB300 issues FP64 at 2 operations per SM and clock against 128 FP32 lanes,
// so the FP64 operator of the outer BiCGSTAB is bound by the FP64 pipe long
// before DRAM.  Where the operator's input is an FP32 vector (the FP32
// V-cycle's output read in place), its products and sums are evaluated in
// double-float instead: a value is the unevaluated sum hi + lo of two floats
// with |lo| <= ulp(hi) / 2, about 48 significand bits in the FP32 exponent
// range (the FP32 V-cycle already confines the vectors to that range).
//
// The building blocks are the classical error-free transformations:
//   * TwoSum (Knuth): s = fl(a + b) and the exact error e, a + b = s + e;
//   * Fast2Sum (Dekker): the same when |a| >= |b|, in three operations;
//   * TwoProd with a fused multiply-add: p = fl(a * b), e = fma(a, b, -p).
// The double-float sum and product are the double-double algorithms of
// Dekker (1971) and of Hida, Li and Bailey (2001, "accurate" sum), with
// floats for doubles.  Every operation is an explicitly rounded intrinsic, so
// the compiler cannot contract or reorder any of them.
#pragma once

#include <cuda_runtime.h>

#include "mac_fp.cuh"

namespace sayaka_gb300 {
namespace dfl {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float ap = __fsub_rn(s, b);
  const float bp = __fsub_rn(s, ap);
  const float e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
  return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df add(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df neg(df x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df mul(df x, df y) {
  df p = two_prod(x.hi, y.hi);
  p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
  p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// x * f for a float f (exact input)
__device__ __forceinline__ df mul_f(df x, float f) {
  df p = two_prod(x.hi, f);
  p.lo = __fmaf_rn(x.lo, f, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// nearest double-float of a double: hi = d rounded to float (integer pipe),
// lo = the rest (exact in FP64: one FP64 subtraction) rounded to float
__device__ __forceinline__ df from_double(double d) {
  const float h = fpint::narrow(d);
  return {h, fpint::narrow(d - fpint::widen(h))};
}

// hi + lo rounded to double: one FP64 addition
__device__ __forceinline__ double to_double(df x) { return fpint::widen(x.hi) + fpint::widen(x.lo); }

__device__ __forceinline__ df load(const float2 *p) {
  const float2 v = *p;
  return {v.x, v.y};
}

}  // namespace dfl
}  // namespace sayaka_gb300
