// Double-float ("float-float") arithmetic: a value is hi + lo with two FP32 numbers,
// |lo| <= ulp(hi) / 2, about 48 significant bits.  Built from the error-free
// transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the FMA-based TwoProduct,
// in the "sloppy" add / Dekker-style multiply combination of Hida, Li and Bailey's
// double-double library, here on FP32 pairs.  Relative error of one operation is a few
// units of 2^-44; FP32 throughput on GB300 is 64x its FP64 rate, so a double-float
// expression costs a fraction of the FP64 one.
//
// Requires IEEE FP32 with round-to-nearest and an exact fused multiply-add (CUDA without
// fast-math; the host compiler's fmaf).  Exponent range is FP32's: callers scale their
// inputs to moderate magnitudes.
#pragma once
#include <cmath>

#ifndef IBEM_HD
#ifdef __CUDACC__
#define IBEM_HD __host__ __device__
#else
#define IBEM_HD
#endif
#endif

#ifdef __CUDACC__
#define IBEM_DF_INLINE __forceinline__
#else
#define IBEM_DF_INLINE inline
#endif

namespace ibem {

struct dfloat {
  float hi, lo;
};

IBEM_HD inline float df_fmaf(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

IBEM_HD inline dfloat df_make(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
IBEM_HD inline double df_double(dfloat a) { return (double)a.hi + (double)a.lo; }

// |a| >= |b| (or a == 0): s + e == a + b exactly
IBEM_HD inline dfloat df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
IBEM_HD inline dfloat df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}

IBEM_HD inline dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
IBEM_HD inline dfloat operator-(dfloat a) { return {-a.hi, -a.lo}; }
IBEM_HD inline dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
IBEM_HD inline dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = df_fmaf(a.hi, b.hi, -p);
  e = df_fmaf(a.hi, b.lo, df_fmaf(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}
// times an FP32 number (exact constants such as small integers)
IBEM_HD inline dfloat operator*(dfloat a, float b) {
  const float p = a.hi * b;
  const float e = df_fmaf(a.lo, b, df_fmaf(a.hi, b, -p));
  return df_fast_two_sum(p, e);
}
IBEM_HD inline dfloat operator*(float b, dfloat a) { return a * b; }
IBEM_HD inline dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
IBEM_HD inline dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }

// Compensated sums (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005, algorithm Dot2) over double-float operands: s is the FP32 running sum of
// the leading products, c the FP32 sum of every rounding error (TwoSum of each addition,
// FMA residual and cross terms of each product).  The value s + c carries about twice
// FP32's precision like a double-float sum, at 12 instead of 18 FP32 instructions per
// multiply-add (no renormalisation after each term).
struct dacc {
  float s, c;
};
IBEM_HD IBEM_DF_INLINE dacc dacc_of(dfloat x) { return {x.hi, x.lo}; }
IBEM_HD IBEM_DF_INLINE dacc dacc_prod(dfloat x, dfloat y) {
  const float p = x.hi * y.hi;
  return {p, df_fmaf(x.hi, y.lo, df_fmaf(x.lo, y.hi, df_fmaf(x.hi, y.hi, -p)))};
}
// a += x * y
IBEM_HD IBEM_DF_INLINE void dacc_fma(dacc& a, dfloat x, dfloat y) {
  const float p = x.hi * y.hi;
  const float e = df_fmaf(x.hi, y.lo, df_fmaf(x.lo, y.hi, df_fmaf(x.hi, y.hi, -p)));
  const float s = a.s + p;
  const float bb = s - a.s;
  a.c += ((a.s - (s - bb)) + (p - bb)) + e;
  a.s = s;
}
// a += x
IBEM_HD IBEM_DF_INLINE void dacc_add(dacc& a, dfloat x) {
  const float s = a.s + x.hi;
  const float bb = s - a.s;
  a.c += ((a.s - (s - bb)) + (x.hi - bb)) + x.lo;
  a.s = s;
}
IBEM_HD IBEM_DF_INLINE dfloat dacc_val(dacc a) { return df_fast_two_sum(a.s, a.c); }
IBEM_HD IBEM_DF_INLINE dfloat dot3(const dfloat* u, const dfloat* x) {
  dacc a = dacc_prod(u[0], x[0]);
  dacc_fma(a, u[1], x[1]);
  dacc_fma(a, u[2], x[2]);
  return dacc_val(a);
}

}  // namespace ibem
