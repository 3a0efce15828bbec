// dfloat.cuh -- double-float (FP32 pair) arithmetic for GB300, whose FP64
// pipe runs at 1/58 of the FP32 rate and also executes every float<->double
// conversion.  A value is held as hi + lo with |lo| <= ulp(hi): ~48
// significant bits (relative error <= 2^-47).  Splitting and merging use
// integer bit operations only, never the FP64 pipe.
//
// Products are exact through the FMA two-product (p = a*b, e = fma(a,b,-p));
// sums use Knuth's TwoSum (6 FP32 operations, no branch).  Published
// algorithms: T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18 (1971); D. E. Knuth, TAOCP vol. 2,
// section 4.2.2 (TwoSum).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vdr {

// Biased FP64 exponent field of d (0 for zero/subnormal, 2047 inf/NaN).
__device__ __forceinline__ int df_exp(double d) {
  return (int)(((unsigned long long)__double_as_longlong(d) >> 52) & 0x7ffu);
}

// d * 2^-shift -> (hi, lo): hi = the scaled value truncated to 24
// significant bits, lo = the remainder truncated to 24 bits (scaling by a
// power of two is exact).  Scaled magnitudes below 2^-126 map to 0; at or
// above 2^128 (and inf/NaN) set *bad and map to 0.
__device__ __forceinline__ void df_split(double d, float &hi, float &lo,
                                         bool &bad, int shift = 0) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e == 2047) {
    bad = true;
    hi = lo = 0.0f;
    return;
  }
  if (e == 0) {  // zero or subnormal: 0 (never rescaled into range)
    hi = lo = 0.0f;
    return;
  }
  const int ef = e - 896 - shift;  // float biased exponent after scaling
  if (ef <= 0) {
    hi = 0.0f;
    lo = 0.0f;
    return;
  }
  if (ef >= 255) {
    bad = true;
    hi = 0.0f;
    lo = 0.0f;
    return;
  }
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)(mant >> 29));
  const unsigned tail = (unsigned)(mant & 0x1FFFFFFFull);  // 29 bits
  const int msb = 31 - __clz(tail | 1u);
  const int elo = msb + e - 948 - shift;  // biased exponent, leading tail bit
  if (tail == 0u || elo <= 0) {
    lo = 0.0f;
    return;
  }
  const unsigned m = (msb >= 23) ? (tail >> (msb - 23)) : (tail << (23 - msb));
  lo = __uint_as_float(sign | ((unsigned)elo << 23) | (m & 0x7fffffu));
}

// Exact float -> double by bits (zero and subnormal floats -> signed zero,
// inf/NaN kept).
__device__ __forceinline__ double df_f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned m = u & 0x7fffffu;
  const unsigned ed = (e == 0u) ? 0u : ((e == 255u) ? 2047u : e + 896u);
  const unsigned mm = (e == 0u) ? 0u : m;
  return __hiloint2double((int)(sign | (ed << 20) | (mm >> 3)), (int)(mm << 29));
}

// d * 2^shift by exponent arithmetic; false if the result would leave the
// normal FP64 range (the caller then uses ldexp).
__device__ __forceinline__ bool df_scale(double &d, int shift) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return (b & 0x7fffffffffffffffLL) == 0;  // zero: done; subnormal: ldexp
  const int en = e + shift;
  if (en < 1 || en > 2046) return false;
  d = __longlong_as_double((b & ~(0x7ffLL << 52)) | ((long long)en << 52));
  return true;
}

// hi + lo as one double: two exact conversions and one FP64 add.
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  return df_f2d(hi) + df_f2d(lo);
}

// Accumulator s + c += (ah + al) * (xh + xl), dropping al*xl (2^-48).
// Every operation is an explicit round-to-nearest intrinsic so that the
// compiler cannot contract them into FMAs (that would break TwoSum).
struct DfAcc {
  float s, c;
};
__device__ __forceinline__ void df_fma_acc(DfAcc &acc, float ah, float al,
                                           float xh, float xl) {
  const float p = __fmul_rn(ah, xh);
  float e = __fmaf_rn(ah, xh, -p);  // exact: ah*xh = p + e
  e = __fmaf_rn(ah, xl, e);
  e = __fmaf_rn(al, xh, e);
  const float t = __fadd_rn(acc.s, p);
  const float bp = __fsub_rn(t, acc.s);
  const float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)),
                              __fsub_rn(p, bp));
  acc.s = t;
  acc.c = __fadd_rn(acc.c, __fadd_rn(err, e));
}

// A normalized double-float value (h + l, |l| <= ulp(h)/2).
struct Df2 {
  float h, l;
};

// d -> Df2 (truncated split, no scaling; |d| must lie in the FP32 range).
__device__ __forceinline__ Df2 df_from_double(double d) {
  Df2 r;
  bool bad = false;
  df_split(d, r.h, r.l, bad);
  return r;
}

// d -> Df2 with a range guard: sets *bad unless d is zero or its magnitude
// lies in [2^-60, 2^60] (so that products and sums of such values stay far
// inside the FP32 exponent range), and for inf/NaN.
__device__ __forceinline__ Df2 df_from_double_chk(double d, bool &bad) {
  const int e = df_exp(d);
  if (e != 0 && (e < 1023 - 60 || e > 1023 + 60)) bad = true;
  return df_from_double(d);
}

// Exact product hi part plus first-order cross terms, renormalized.
__device__ __forceinline__ Df2 df_mul(Df2 a, Df2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float s = __fadd_rn(p, e);
  return Df2{s, __fsub_rn(e, __fsub_rn(s, p))};
}

// acc += a * b (the accumulator stays unnormalized until read).
__device__ __forceinline__ void df_acc(DfAcc &acc, Df2 a, Df2 b) {
  df_fma_acc(acc, a.h, a.l, b.h, b.l);
}

// The accumulator as a normalized pair (TwoSum of its two parts).
__device__ __forceinline__ Df2 df_norm(const DfAcc &a) {
  const float s = __fadd_rn(a.s, a.c);
  const float bp = __fsub_rn(s, a.s);
  const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(a.c, bp));
  return Df2{s, e};
}

// a + b and a - b, normalized.
__device__ __forceinline__ Df2 df_add(Df2 a, Df2 b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bp = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bp)), __fsub_rn(b.h, bp));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  const float bq = __fsub_rn(h, s);
  return Df2{h, __fadd_rn(__fsub_rn(s, __fsub_rn(h, bq)), __fsub_rn(e, bq))};
}
__device__ __forceinline__ Df2 df_neg(Df2 a) { return Df2{-a.h, -a.l}; }
__device__ __forceinline__ Df2 df_sub(Df2 a, Df2 b) { return df_add(a, df_neg(b)); }

// 1/a for a normal nonzero pair: the FP32 reciprocal r0 of a.h refined by
// one Newton step r0 (1 + e + e^2) with e = 1 - a r0 formed from the exact
// product a.h r0 (1 - p is exact, p lying within an ulp of 1) and a.l r0;
// relative error ~2^-46.
__device__ __forceinline__ Df2 df_rcp(Df2 a) {
  const float r0 = __frcp_rn(a.h);
  const float p = __fmul_rn(a.h, r0);
  const float pl = __fmaf_rn(a.h, r0, -p);
  float e = __fsub_rn(1.0f, p);
  e = __fsub_rn(e, pl);
  e = __fmaf_rn(-a.l, r0, e);
  const float c = __fmul_rn(r0, __fmaf_rn(e, e, e));
  const float h = __fadd_rn(r0, c);
  return Df2{h, __fsub_rn(c, __fsub_rn(h, r0))};
}

// acc += a.
__device__ __forceinline__ void df_acc_add(DfAcc &acc, Df2 a) {
  const float t = __fadd_rn(acc.s, a.h);
  const float bp = __fsub_rn(t, acc.s);
  const float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)),
                              __fsub_rn(a.h, bp));
  acc.s = t;
  acc.c = __fadd_rn(acc.c, __fadd_rn(err, a.l));
}

}  // namespace vdr
