// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32 numbers
// (|lo| <= ulp(hi)/2), giving a 48-bit significand with FP32 exponent range.  On GB300 the
// FP64 pipe delivers 1/58 of the FP32 rate, so the refinement residual, right-hand side and
// state of the batched transient use this representation on the FP32 pipes instead.
//
// Algorithms (error-free transformations): TwoSum (Knuth), FastTwoSum (Dekker),
// TwoProduct with a fused multiply-add, as in Dekker 1971 and Hida, Li & Bailey's
// "double-double" library; the sloppy addition below bounds its error by a few ulps of the
// operands (not of the result), which is the property a residual b - A x needs.
#pragma once

#include <cuda_runtime.h>
#include <string.h>

namespace krets {

// 8-byte aligned, so that a pair moves with one 64-bit load or store (every df array of
// the engines starts on a 16-byte boundary of its layout).
struct __align__(8) df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) { return df{hi, lo}; }

// split an FP64 value into hi + lo (FP64 ops; used only at set-up and for source values)
__device__ __forceinline__ df df_from_double(double v) {
  const float hi = (float)v;
  return df{hi, (float)(v - (double)hi)};
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// The same value with one FP64 instruction instead of three: a normal FP32 number widens to
// FP64 exactly by moving its fields (exponent rebased from 127 to 1023, significand shifted
// up 29 bits), so both parts are widened with integer instructions and only their sum runs
// on the FP64 pipe (a small fraction of the FP32 rate on this GPU).  Zero, subnormal and
// non-finite parts take the FP64 conversions; the result is bit-identical to df_to_double.
__device__ __forceinline__ double f32_widened(unsigned u) {
  const unsigned long long e = (u >> 23) & 0xff;
  return __longlong_as_double(((unsigned long long)(u >> 31) << 63) | ((e + 896ull) << 52) |
                              ((unsigned long long)(u & 0x7fffff) << 29));
}

__device__ __forceinline__ double df_to_double_fast(df a) {
  const unsigned hb = __float_as_uint(a.hi), lb = __float_as_uint(a.lo);
  const unsigned he = (hb >> 23) & 0xff, le = (lb >> 23) & 0xff;
  const bool lo_zero = (lb & 0x7fffffff) == 0;
  if (he != 0 && he != 0xff && (lo_zero || (le != 0 && le != 0xff)))
    return f32_widened(hb) + (lo_zero ? 0.0 : f32_widened(lb));
  return df_to_double(a);
}

// hi + lo correctly rounded to FP64 with integer instructions only (no FP64 pipe).
// Both parts are exact binary fractions.  The sum is formed as a signed integer in units of
// 2^-32 ulp(hi): 24 + 32 bits hold hi and every bit of lo that can reach the 53-bit result,
// lo's bits below that unit are folded into a sticky bit, and the total is normalised and
// rounded to nearest-even (guard, round and sticky bits below the kept 53).  Zero,
// subnormal or non-finite parts, and a lo that is not below ulp(hi), take the FP64 sum.
__device__ __host__ __forceinline__ double df_to_double_bits(unsigned hb, unsigned lb, bool &ok) {
  const int he = (int)((hb >> 23) & 0xff), le = (int)((lb >> 23) & 0xff);
  ok = false;
  if (he == 0 || he == 0xff || le == 0xff || (le == 0 && (lb & 0x7fffff))) return 0.0;
  long long acc = (long long)((hb & 0x7fffff) | 0x800000) << 32;  // < 2^56
  if (hb >> 31) acc = -acc;
  if (le != 0) {
    const long long ml = (long long)((lb & 0x7fffff) | 0x800000);
    const int shift = le - he + 32;  // lo in units of 2^(he-182)
    if (shift > 8) return 0.0;       // lo not below ulp(hi): not a normalised pair
    long long lv;
    if (shift >= 0) lv = ml << shift;
    else if (shift > -40) lv = (ml >> (-shift)) | ((ml & ((1ll << (-shift)) - 1)) != 0 ? 1 : 0);
    else lv = 1;
    acc += (lb >> 31) ? -lv : lv;
  }
  if (acc == 0) {
    ok = true;
    return 0.0;
  }
  unsigned long long sign = 0, m = (unsigned long long)acc;
  if (acc < 0) {
    sign = 1ull << 63;
    m = (unsigned long long)(-acc);
  }
  int top = 63;
  while (!((m >> top) & 1)) --top;  // leading bit (loop is at most a few steps: top in 54..56)
  int e2 = he - 182 + top;          // unbiased exponent of the leading bit
  const int drop = top - 52;
  unsigned long long q;
  if (drop > 0) {
    q = m >> drop;
    const unsigned long long rem = m & ((1ull << drop) - 1), half = 1ull << (drop - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
    if (q >> 53) {
      q >>= 1;
      ++e2;
    }
  } else {
    q = m << (-drop);
  }
  if (e2 < -1022 || e2 > 1023) return 0.0;
  ok = true;
  const unsigned long long bits = sign | ((unsigned long long)(e2 + 1023) << 52) | (q & ((1ull << 52) - 1));
  double r;
  memcpy(&r, &bits, sizeof r);
  return r;
}

__device__ __forceinline__ double df_to_double_int(df a) {
  bool ok;
  const double r = df_to_double_bits(__float_as_uint(a.hi), __float_as_uint(a.lo), ok);
  return ok ? r : df_to_double(a);
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df{p, __fmaf_rn(a, b, -p)};
}

// a + b, error O(eps^2 (|a| + |b|))
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

// a + f (f a plain FP32 number)
__device__ __forceinline__ df df_add_f(df a, float f) {
  df s = two_sum(a.hi, f);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}

// a * b
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}

// acc + a * b (the product is not renormalised before the addition)
__device__ __forceinline__ df df_fma(df a, df b, df acc) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  df s = two_sum(acc.hi, p.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(acc.lo, p.lo));
  return fast_two_sum(s.hi, s.lo);
}

// acc + a * b with the result left unnormalised: hi is the rounded running sum (TwoSum
// keeps every step exact), lo collects the error terms.  For dot products over a row;
// df_norm() renormalises once at the end (TwoSum, so |lo| > |hi| is also handled).
__device__ __forceinline__ df df_fma_acc(df a, df b, df acc) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  df s = two_sum(acc.hi, p.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(acc.lo, p.lo));
  return s;
}

__device__ __forceinline__ df df_norm(df a) { return two_sum(a.hi, a.lo); }

// acc - x (x exact +-1 multiple: incidence entries of the MNA matrix)
__device__ __forceinline__ float df_approx(df a) { return __fadd_rn(a.hi, a.lo); }

}  // namespace krets
