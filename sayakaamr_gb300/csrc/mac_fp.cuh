// FP64 bookkeeping on the integer pipe.
//
// GB300 issues FP64 at 2 operations per SM and clock, and its FP64 pipe
// also carries FP64 compares, min/max and the FP32 <-> FP64 conversions.
// The BiCGSTAB vector kernels of the device solve are bound by that pipe, so
// every operation here that only moves or orders bits is done on 32/64-bit
// integers instead, with results identical to the FP64 instructions:
//   * non-negative doubles order like their bit patterns read as integers,
//     and a NaN (all-ones exponent, non-zero mantissa) orders above +inf, so
//     the max of |v| over bit patterns is the NaN-propagating max of |v|;
//   * float -> double is exact: rebias the exponent, widen the mantissa
//     (denormals normalised);
//   * double -> float rounds to nearest with ties to even (IEEE 754
//     roundTiesToEven), float denormals, overflow to inf and NaN included.
#pragma once

#include <cuda_runtime.h>

namespace sayaka_gb300 {
namespace fpint {

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// running max of |v| as bit patterns (start from 0 = +0.0)
__device__ __forceinline__ unsigned long long max_abs(unsigned long long m, double v) {
  const unsigned long long u = abs_bits(v);
  return u > m ? u : m;
}

__device__ __forceinline__ double from_bits(unsigned long long u) { return __longlong_as_double((long long)u); }

// v > 0 for v that is never a NaN (volume fractions, operator factors):
// positive doubles, and only they, have positive bit patterns as int64
__device__ __forceinline__ bool positive(double v) { return __double_as_longlong(v) > 0; }

// exact float -> double, every case on the integer pipe (no conversion
// instruction at all, so that none is issued even where the compiler
// evaluates both sides of a branch): normal floats rebias the exponent and
// widen the mantissa; denormals are normalised (the leading one moved to bit
// 23, the exponent lowered by the shift); inf and NaN keep their mantissa
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e != 0u && e != 0xffu)
    return from_bits(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29));
  if (e == 0xffu) return from_bits(sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29));
  if (m == 0u) return from_bits(sign);
  const int s = __clz((int)m) - 8;  // m * 2^-149 = (m << s) * 2^(-149 - s), bit 23 set
  return from_bits(sign | ((unsigned long long)(897 - s) << 52) | ((unsigned long long)((m << s) & 0x7fffffu) << 29));
}

// 0.0 + (double)f: as widen, with -0 turned into +0
__device__ __forceinline__ double widen_plus0(float f) {
  return (__float_as_uint(f) & 0x7fffffffu) == 0u ? 0.0 : widen(f);
}

// double -> float, round to nearest, ties to even, every case on the
// integer pipe: normal float results round the 52-bit mantissa to 23 bits;
// results below the normal range become float denormals (the 53-bit
// significand shifted into place, rounded the same way); |d| at or above
// 2^128 becomes inf; inf stays inf, NaN becomes a quiet NaN
__device__ __forceinline__ float narrow(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7ffu);
  const unsigned long long m = u & 0xfffffffffffffull;
  // normal float results: biased float exponent e - 896 in [1, 254]
  if (e >= 897 && e <= 1150) {
    const unsigned long long rem = m & 0x1fffffffull;  // the 29 bits dropped
    unsigned r = ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29);
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (r & 1u))) r += 1u;  // carry may reach the exponent
    return __uint_as_float(sign | r);  // a carry into exponent 255 is +-inf, as IEEE rounding gives
  }
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u | (unsigned)(m >> 29) : 0u));
  if (e > 1150) return __uint_as_float(sign | 0x7f800000u);
  // |d| < 2^-126: d * 2^149 = M * 2^(e - 926) with M = 2^52 + m, rounded to
  // an integer (a carry into bit 23 gives the smallest normal float); double
  // denormals and everything below 2^-150 round to zero
  const int sh = 926 - e;  // >= 30
  if (e == 0 || sh >= 54) return __uint_as_float(sign);
  const unsigned long long M = (1ull << 52) | m;
  unsigned long long f = M >> sh;
  const unsigned long long rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (f & 1ull))) f += 1ull;
  return __uint_as_float(sign | (unsigned)f);
}

// exact conversion To <- From between float and double on the integer pipe
// (narrowing rounds to nearest even), identity otherwise
template <typename To, typename From>
__device__ __forceinline__ To cvt(From v) {
  if constexpr (sizeof(To) == 8 && sizeof(From) == 4)
    return widen(v);
  else if constexpr (sizeof(To) == 4 && sizeof(From) == 8)
    return narrow(v);
  else
    return (To)v;
}

}  // namespace fpint
}  // namespace sayaka_gb300
