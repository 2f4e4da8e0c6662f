// Double-float arithmetic: values held as an unevaluated sum h + l of two FP32 numbers
// (|l| <= ulp(h) / 2 after normalisation), about 48 significant bits, computed on the FP32 pipe.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so an f64 evaluation that keeps its arithmetic in
// FP64 is bound by the FP64 pipe an order of magnitude before it is bound by memory. The
// double-float kernels compute the same factors from the same f64 inputs with error-free
// transformations on FP32 operations instead:
//  - TwoSum (Knuth): s = fl(a + b), e = (a - (s - bb)) + (b - bb), bb = s - a, gives a + b = s + e
//    exactly; Fast2Sum (Dekker) does the same in three operations when |a| >= |b|;
//  - TwoProd by FMA: p = fl(a b), e = fma(a, b, -p) gives a b = p + e exactly;
//  - products of double-floats add the cross terms a.h b.l + a.l b.h into the error term;
//  - the reciprocal and the square root take one Newton step in double-float from the FP32
//    result.
// (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2; Joldes, Muller, Popescu 2017.) Every operation is
// an explicitly rounded intrinsic, so the compiler contracts nothing.
//
// Ar<DF<V>> gives the operations of Ar<V> (eval.cuh) on double-floats of V = float or f32 pairs
// (two quadrature points per instruction, FFMA2 / FADD2 / FMUL2), so Factors<DF<V>, TD, GD>
// evaluates det J, K, normals and facet normals in double-float with the formulas of the other
// kernels.
//
// f64 <-> double-float conversions: df_split rounds an f64 to its nearest f32 (integer
// operations) and the remainder with one FP64 subtraction; df_to_f64 assembles the f64 bit
// pattern of h + l with integer operations and one FFMA (the f64 value of h, plus l in units of
// 64 ulp of that f64: about 47 significant bits). Both are branch-free.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "convert.cuh"
#include "eval.cuh"

namespace tlg {

template <typename V>
struct DF {
  V h, l;
};

template <typename V>
struct Ar<DF<V>> {
  using B = Ar<V>;
  using S = typename B::S;
  using D = DF<V>;
  __device__ __forceinline__ static D make(V h, V l) {
    D r;
    r.h = h;
    r.l = l;
    return r;
  }
  __device__ __forceinline__ static D splat(S s) { return make(B::splat(s), B::splat(S(0))); }
  // a + b = s + e exactly (any magnitudes).
  __device__ __forceinline__ static D two_sum(V a, V b) {
    const V s = B::add(a, b);
    const V bb = B::sub(s, a);
    const V e = B::add(B::sub(a, B::sub(s, bb)), B::sub(b, bb));
    return make(s, e);
  }
  // a + b = s + e exactly when |a| >= |b| (or a = 0).
  __device__ __forceinline__ static D fast_two_sum(V a, V b) {
    const V s = B::add(a, b);
    return make(s, B::sub(b, B::sub(s, a)));
  }
  __device__ __forceinline__ static D add(D a, D b) {
    const D s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, B::add(s.l, B::add(a.l, b.l)));
  }
  __device__ __forceinline__ static D neg(D a) { return make(B::neg(a.h), B::neg(a.l)); }
  __device__ __forceinline__ static D sub(D a, D b) { return add(a, neg(b)); }
  // The exact product of the heads plus the cross terms, unnormalised.
  __device__ __forceinline__ static D mul_raw(D a, D b) {
    const V p = B::mul(a.h, b.h);
    V e = B::fma(a.h, b.h, B::neg(p));
    e = B::fma(a.h, b.l, e);
    e = B::fma(a.l, b.h, e);
    return make(p, e);
  }
  __device__ __forceinline__ static D mul(D a, D b) {
    const D r = mul_raw(a, b);
    return fast_two_sum(r.h, r.l);
  }
  // a b + c.
  __device__ __forceinline__ static D fma(D a, D b, D c) {
    const D p = mul_raw(a, b);
    const D s = two_sum(p.h, c.h);
    return fast_two_sum(s.h, B::add(s.l, B::add(p.l, c.l)));
  }
  // 1 / a: r = fl(1 / a.h), then r + r (1 - a r) with 1 - a r formed by FMAs.
  __device__ __forceinline__ static D rcp(D a) {
    const V r = B::rcp(a.h);
    V e = B::fma(B::neg(a.h), r, B::splat(S(1)));
    e = B::fma(B::neg(a.l), r, e);
    return fast_two_sum(r, B::mul(r, e));
  }
  // a / b: q = a.h r, then q + r (a - b q) with the residual in double-float.
  __device__ __forceinline__ static D div(D a, D b) {
    const V r = B::rcp(b.h);
    const V q = B::mul(a.h, r);
    const D bq = mul_raw(b, make(q, B::splat(S(0))));
    // a - b q: the heads nearly cancel (Sterbenz), the rest is small.
    V res = B::sub(a.h, bq.h);
    res = B::add(res, B::sub(a.l, bq.l));
    return fast_two_sum(q, B::mul(r, res));
  }
  // sqrt(a) for a >= 0: s = fl(sqrt(a.h)), then s + (a - s^2) / (2 s).
  __device__ __forceinline__ static D sqrt(D a) {
    const V s = B::sqrt(a.h);
    const V p = B::mul(s, s);
    const V pe = B::fma(s, s, B::neg(p));
    V res = B::sub(B::sub(a.h, p), pe);
    res = B::add(res, a.l);
    // s = 0 (a = 0): no correction.
    const V half_inv = B::mul(B::splat(S(0.5)), B::rcp(s));
    V corr = B::mul(res, half_inv);
    corr = zero_if_zero(s, corr);
    return fast_two_sum(s, corr);
  }
  __device__ __forceinline__ static float zero_if_zero(float s, float c) { return s == 0.0f ? 0.0f : c; }
  __device__ __forceinline__ static float2 zero_if_zero(float2 s, float2 c) {
    return make_float2(s.x == 0.0f ? 0.0f : c.x, s.y == 0.0f ? 0.0f : c.y);
  }
};

// A double-float sum of products accumulated term by term: s the running FP32 sum of the
// products' heads (TwoSum keeps each rounding error), c the FP32 sum of those errors, of the
// products' own errors and of the cross terms. Error about 2^-48 of the largest partial sum per
// term (no renormalisation between terms).
template <typename V>
struct DfAcc {
  using B = Ar<V>;
  V s, c;
  __device__ __forceinline__ void zero() { s = c = B::splat(0.0f); }
  // += (yh + yl) (th + tl), y a node coordinate, t a table value.
  __device__ __forceinline__ void add(V yh, V yl, V th, V tl) {
    const V p = B::mul(yh, th);
    c = B::add(c, B::fma(yh, th, B::neg(p)));
    c = B::fma(yh, tl, c);
    c = B::fma(yl, th, c);
    const V t = B::add(s, p);
    const V bb = B::sub(t, s);
    c = B::add(c, B::add(B::sub(s, B::sub(t, bb)), B::sub(p, bb)));
    s = t;
  }
  __device__ __forceinline__ DF<V> value() const { return Ar<DF<V>>::fast_two_sum(s, c); }
};

// f64 -> f32 rounded to nearest even and f32 -> f64, in integer operations without branches (a
// branch per conversion costs more than the conversion): as convert.cuh's d2f_rn / f2d_exact for
// normal values, with magnitudes below the f32 normal range flushed to a signed zero (below
// 1.2e-38: far below any geometric value these kernels produce), overflow to infinity and NaN to
// NaN.
__device__ __forceinline__ float d2f_nb(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  unsigned r = sign | ((e - 896u) << 23) | (unsigned)(m >> 29);
  const unsigned rest = (unsigned)(m & 0x1FFFFFFFull);
  r += (unsigned)(rest > 0x10000000u) | ((unsigned)(rest == 0x10000000u) & r & 1u);
  // Below 2^-126: zero; from 2^128 on: infinity, NaN stays NaN.
  const unsigned special = e == 0x7FFu && m != 0 ? 0x7FC00000u : 0x7F800000u;
  r = e < 897u ? sign : (e > 1150u ? sign | special : r);
  return __uint_as_float(r);
}

__device__ __forceinline__ double f2d_nb(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  const uint32_t sign = b & 0x80000000u;
  uint32_t hi = sign | (((b & 0x7FFFFFFFu) >> 3) + (e == 0xFFu ? (1792u << 20) : (896u << 20)));
  uint32_t lo = b << 29;
  hi = e == 0u ? sign : hi;  // zero (and f32 subnormals) to a signed zero
  lo = e == 0u ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}

// An f64 as the nearest f32 and the f32 nearest to the remainder (about 48 bits).
__device__ __forceinline__ void df_split(double v, float& h, float& l) {
  h = d2f_nb(v);
  l = d2f_nb(__dsub_rn(v, f2d_nb(h)));
}

// h + l as an f64 (h, l normalised: |l| <= ulp(h) / 2), in integer operations and one FFMA,
// without branches. For |h| in [2^-81, 2^128): the f64 of h plus l in units of 64 ulp of that
// f64 (about 47 significant bits). Below 2^-81 l is dropped (the f64 of h, relative error 2^-24 of
// a value under 4e-25), f32 subnormals and zero give a signed zero, infinity and NaN stay so.
__device__ __forceinline__ double df_to_f64(float h, float l) {
  const uint32_t hb = __float_as_uint(h);
  const uint32_t eh = (hb >> 23) & 0xFFu;
  const bool scaled = eh - 46u <= 208u;
  // n = l / (64 ulp64(h)), rounded to nearest: |l| <= ulp32(h) / 2 = 2^28 ulp64(h), so |n| <= 2^22
  // and 1.5 * 2^23 + n is exact in [2^23, 2^24], its low mantissa bits n. The scale carries h's
  // sign, so that n is the change of h's magnitude.
  const float scale = __uint_as_float(((300u << 23) - (hb & 0x7F800000u)) | (hb & 0x80000000u));
  const float t = __fmaf_rn(l, scaled ? scale : 0.0f, 12582912.0f);
  const int n = (int)(__float_as_uint(t) - 0x4B400000u);
  // A power of two h whose magnitude l lowers lands in the binade below, whose ulp is half: the
  // same change of value is twice as many units of the mantissa field there.
  const int shift = 6 + (int)(((hb << 9) == 0u) & (n < 0));
  const uint32_t sign = hb & 0x80000000u;
  uint32_t hi = sign | (((hb & 0x7FFFFFFFu) >> 3) + (eh == 0xFFu ? (1792u << 20) : (896u << 20)));
  uint32_t lo = hb << 29;
  hi = eh == 0u ? sign : hi;
  lo = eh == 0u ? 0u : lo;
  const uint64_t bits = (((uint64_t)hi << 32) | lo) + (uint64_t)((int64_t)n << shift);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double df_to_f64(DF<float> v) { return df_to_f64(v.h, v.l); }

}  // namespace tlg
