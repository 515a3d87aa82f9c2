/*
 * Double-float arithmetic: a value is an unevaluated sum hi + lo of two
 * floats with |lo| <= ulp(hi)/2, about 48 significant bits.  GB300 runs FP32
 * at 63 times its FP64 rate, so the assembly stage of the FP64 form (STV
 * components, the 384 x 200 map, the contraction) evaluates in this
 * arithmetic on the FP32 pipe: 7-11 FP32 operations per operation, with
 * relative error ~2^-47 of the operands -- far inside the FP64 form's
 * 1e-12 parity bound, and checked against the FP64 oracle by the tests.
 *
 * The algorithms are the classical error-free transformations: TwoSum
 * (Knuth), Fast2Sum (Dekker), TwoProduct by fused multiply-add; the sum and
 * product follow the double-single arithmetic of Dekker (1971) and Bailey's
 * later double-double / double-single libraries ("sloppy" addition:
 * one TwoSum of the high parts, low parts added in float).
 *
 * Range: that of float (|hi| up to 3.4e38; values below ~1e-38 lose their
 * low part, below 1.4e-45 vanish).
 */
#ifndef KQED_DF_H
#define KQED_DF_H

#include <cmath>

#if defined(__CUDACC__)
#define KQED_HD __host__ __device__ __forceinline__
#else
#define KQED_HD inline
#endif

namespace kqed {

struct df {
  float hi, lo;
  df() = default;
  KQED_HD constexpr df(float h, float l) : hi(h), lo(l) {}
  /* small exact constants (0, +-1/2, 1, 2, 3, 1/4 ...) */
  KQED_HD explicit constexpr df(int v) : hi((float)v), lo(0.0f) {}
  KQED_HD explicit df(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

KQED_HD float df_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

/* s + e = a + b exactly (any a, b) */
KQED_HD void two_sum(float a, float b, float &s, float &e)
{
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

/* s + e = a + b exactly, |a| >= |b| (or a == 0) */
KQED_HD void fast_two_sum(float a, float b, float &s, float &e)
{
  s = a + b;
  e = b - (s - a);
}

KQED_HD df operator+(df a, df b)
{
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  float h, l;
  fast_two_sum(s, e, h, l);
  return df(h, l);
}

KQED_HD df operator-(df a) { return df(-a.hi, -a.lo); }
KQED_HD df operator-(df a, df b) { return a + (-b); }

KQED_HD df operator*(df a, df b)
{
  const float p = a.hi * b.hi;
  float e = df_fma(a.hi, b.hi, -p);
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  float h, l;
  fast_two_sum(p, e, h, l);
  return df(h, l);
}

/* a * b + c with one renormalisation: the product's high part and c.hi
   added by TwoSum, the low terms (product error, cross terms, c.lo) in
   float.  Generic code calls fma(a, b, c) for double, float and df alike. */
using ::fma;
KQED_HD df fma(df a, df b, df c)
{
  const float p = a.hi * b.hi;
  float e = df_fma(a.hi, b.hi, -p);
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  float s, t;
  two_sum(p, c.hi, s, t);
  t += e + c.lo;
  float h, l;
  fast_two_sum(s, t, h, l);
  return df(h, l);
}

/* multiplication by a power of two or its negative (exact) */
KQED_HD df scale_exact(df a, float c) { return df(a.hi * c, a.lo * c); }

KQED_HD df &operator+=(df &a, df b) { return a = a + b; }

KQED_HD double to_double(df a) { return (double)a.hi + (double)a.lo; }

} // namespace kqed

#endif
