// dfloat.cuh - double-float arithmetic: a value is an unevaluated sum hi + lo
// of two FP32 numbers (|lo| <= ulp(hi)/2), giving a 48-bit significand on the
// FP32 pipes.  On GB300 FP64 runs at 1/62 of the FP32 rate, so double-float
// (about 15 FP32 instructions per fused multiply-add) is the fast route to
// near-FP64 accuracy.
//
// Built from the error-free transformations of Knuth (TwoSum), Dekker
// (FastTwoSum) and the FMA-based TwoProduct; the add and multiply follow the
// "sloppy" double-word algorithms analysed by Joldes, Muller and Popescu
// (ACM TOMS 44(2), 2017), relative error below 2^-44 except under
// cancellation, where the absolute error stays below 2^-44 of the operands.
#pragma once

#include <cuda_runtime.h>

// The type lives in its own namespace: its fma/sqrt/fabs overloads are found
// by argument-dependent lookup only, so they never hide CUDA's float and
// double overloads inside namespace lri.
namespace lri_df {

struct __align__(8) dfloat {
  float hi, lo;

  dfloat() = default;
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit dfloat(int x) : hi((float)x), lo(0.0f) {}
  __device__ __forceinline__ explicit dfloat(float x) : hi(x), lo(0.0f) {}
  __device__ __forceinline__ explicit dfloat(double x) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
  }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfloat fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfloat(s, b - (s - a));
}

__device__ __forceinline__ dfloat two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfloat(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  dfloat s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// a * b + c with one renormalisation
__device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  dfloat s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, s.lo + (e + c.lo));
}

// Accumulation without renormalisation, for long sums of products (tile
// products and Gram reductions): acc.hi carries the TwoSum of the leading
// products, acc.lo collects their errors; renorm() restores |lo| <= ulp(hi)/2.
// 12 FP32 instructions instead of 15 for fma().
__device__ __forceinline__ dfloat fma_acc(dfloat a, dfloat b, dfloat acc) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const dfloat s = two_sum(acc.hi, p);
  return dfloat(s.hi, acc.lo + (s.lo + e));
}
__device__ __forceinline__ dfloat renorm(dfloat a) { return fast_two_sum(a.hi, a.lo); }

__device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) {
  const float q1 = a.hi / b.hi;
  const dfloat r = fma(-dfloat(q1), b, a);  // a - q1 * b
  const float q2 = r.hi / b.hi;
  return fast_two_sum(q1, q2);
}

__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }

__device__ __forceinline__ bool operator==(dfloat a, dfloat b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dfloat a, dfloat b) { return !(a == b); }
__device__ __forceinline__ bool operator<(dfloat a, dfloat b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfloat a, dfloat b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfloat a, dfloat b) { return !(a < b); }

__device__ __forceinline__ dfloat fabs(dfloat a) { return (a.hi < 0.0f) ? -a : a; }
__device__ __forceinline__ dfloat copysign(dfloat a, dfloat s) {
  const dfloat m = fabs(a);
  return (s.hi < 0.0f || (s.hi == 0.0f && signbit(s.hi))) ? -m : m;
}

// sqrt by one Newton correction of the FP32 root: s + (a - s^2) / (2 s)
__device__ __forceinline__ dfloat sqrt(dfloat a) {
  if (a.hi <= 0.0f) return dfloat(0.0f, 0.0f);
  const float s = sqrtf(a.hi);
  const float p = s * s;
  const float e = fmaf(s, s, -p);
  const float resid = ((a.hi - p) - e) + a.lo;
  return fast_two_sum(s, resid / (2.0f * s));
}

__device__ __forceinline__ bool isfinite(dfloat a) { return ::isfinite(a.hi) && ::isfinite(a.lo); }

}  // namespace lri_df

namespace lri {
using lri_df::dfloat;
}  // namespace lri
