// Double-float arithmetic on the FP32 pipe: a value is hi + lo, two FP32,
// about 48 significant bits.  This GPU issues FP32 64 times faster than FP64
// (its FP64 pipe, conversions included, does 2 operations per clock per SM),
// so the precision forms run their transforms and their xc functional in
// double-float and keep FP64 for the sums that must stay FP64.
//
// Products use Dekker's exact product (with an FMA), sums Knuth's two-sum.
// Sums that only feed other sums may skip the renormalisation (add_lazy);
// the FMA-based products accept such unnormalised pairs as they are.
#pragma once
#include <cuda_runtime.h>

namespace lcp {
namespace {

struct Dfl {
  float hi, lo;
};

// a literal as double-float, folded at compile time
__host__ __device__ constexpr Dfl dflc(double c) { return Dfl{(float)c, (float)(c - (double)(float)c)}; }

__device__ __forceinline__ Dfl quick_two_sum(float s, float e) {
  const float r = s + e;
  return {r, e - (r - s)};
}

// hi parts summed with their exact rounding error, low parts added, not renormalised
__device__ __forceinline__ Dfl add_lazy(Dfl a, Dfl b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  return {s, ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo)};
}
__device__ __forceinline__ Dfl operator-(Dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ Dfl operator+(Dfl a, Dfl b) {
  const Dfl t = add_lazy(a, b);
  return quick_two_sum(t.hi, t.lo);
}
__device__ __forceinline__ Dfl operator-(Dfl a, Dfl b) { return a + (-b); }
__device__ __forceinline__ Dfl operator*(Dfl a, Dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ Dfl operator*(Dfl a, float b) {
  const float p = a.hi * b;
  return quick_two_sum(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}
// a b + c d with one renormalisation: both high products exact (FMA), their
// sum by two-sum, the cross terms accumulated in FP32.
__device__ __forceinline__ Dfl dot2(Dfl a, Dfl b, Dfl c, Dfl d) {
  const float p1 = a.hi * b.hi, p2 = c.hi * d.hi;
  float t = fmaf(a.hi, b.hi, -p1) + fmaf(c.hi, d.hi, -p2);
  const float s = p1 + p2;
  const float bb = s - p1;
  const float e = (p1 - (s - bb)) + (p2 - bb);
  t = fmaf(a.hi, b.lo, t);
  t = fmaf(a.lo, b.hi, t);
  t = fmaf(c.hi, d.lo, t);
  t = fmaf(c.lo, d.hi, t);
  return quick_two_sum(s, e + t);
}
__device__ __forceinline__ bool operator<(Dfl a, float b) { return a.hi < b || (a.hi == b && a.lo < 0.0f); }

// 1 - p as FP32, for p within a few FP32 ulps of 1 (1 - p.hi is exact)
__device__ __forceinline__ float one_minus(Dfl p) { return (1.0f - p.hi) - p.lo; }

// Reciprocal, reciprocal square root and reciprocal cube root of x > 0: an
// FP32 estimate y0 and one Newton step on the residual r = 1 - x y0^k,
// computed in double-float (y = y0 (1 + r / k) up to O(r^2)).  FP32
// estimates within a few ulps leave errors near 2^-45.
__device__ __forceinline__ Dfl dfl_rcp(Dfl x) {
  const float y0 = __frcp_rn(x.hi);
  const float r = one_minus(x * y0);
  return quick_two_sum(y0, y0 * r);
}
__device__ __forceinline__ Dfl dfl_rsqrt(Dfl x) {
  const float y0 = rsqrtf(x.hi);
  const float s = y0 * y0;
  const Dfl y2 = {s, fmaf(y0, y0, -s)};  // y0^2 exactly
  const float r = one_minus(x * y2);
  return quick_two_sum(y0, y0 * (0.5f * r));
}
__device__ __forceinline__ Dfl dfl_rcbrt(Dfl x) {
  const float y0 = rcbrtf(x.hi);
  const float s = y0 * y0;
  const Dfl y3 = Dfl{s, fmaf(y0, y0, -s)} * y0;
  const float r = one_minus(x * y3);
  return quick_two_sum(y0, y0 * (r * (1.0f / 3.0f)));
}

// cube root of x >= 0 as x rcbrt(x)^2, and 0 for 0
__device__ __forceinline__ Dfl dfl_cbrt(Dfl x) {
  if (x.hi == 0.0f) return {0.0f, 0.0f};
  const Dfl y = dfl_rcbrt(x);
  return x * (y * y);
}

// expm1(x): x = k ln2 + r with k = round(x / ln2) and r in double-float
// (|r| <= 0.35), expm1(r / 16) by its Taylor series (the terms from y^4 on in
// FP32, where they stay below 1e-8 of y), four doublings expm1(2y) =
// expm1(y) (expm1(y) + 2), which keep the relative error, then
// 2^k (expm1(r) + 1) - 1.  Relative error about (1 + |x|) 2^-47, the
// conditioning of x's own double-float rounding.  |x| > 80 goes to FP64.
__device__ __forceinline__ Dfl dfl_expm1(Dfl x) {
  if (fabsf(x.hi) > 80.0f) {
    const double v = expm1((double)x.hi + (double)x.lo);
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
  }
  const Dfl ln2 = dflc(0.6931471805599453);
  const float k = rintf(x.hi * 1.4426950408889634f);
  const float p = k * ln2.hi;
  const Dfl r = x - quick_two_sum(p, fmaf(k, ln2.lo, fmaf(k, ln2.hi, -p)));
  const Dfl y = {r.hi * 0.0625f, r.lo * 0.0625f};
  const float yh = y.hi;
  const float T = fmaf(yh, fmaf(yh, fmaf(yh, fmaf(yh, fmaf(yh, 1.0f / 362880.0f, 1.0f / 40320.0f), 1.0f / 5040.0f),
                                        1.0f / 720.0f), 1.0f / 120.0f), 1.0f / 24.0f);
  const Dfl q = dflc(1.0 / 6.0) + y * T;
  const Dfl r2 = dflc(0.5) + y * q;
  Dfl e = y + (y * y) * r2;
#pragma unroll
  for (int i = 0; i < 4; ++i) e = e * (e + dflc(2.0));
  if (k == 0.0f) return e;
  const float sc = __uint_as_float((unsigned)(127 + (int)k) << 23);  // 2^k, |k| <= 116
  const Dfl s1 = e + dflc(1.0);
  return Dfl{s1.hi * sc, s1.lo * sc} - dflc(1.0);
}
// log(u) from an FP32 estimate y0 by one Newton step on exp(y) = u in
// double-float: y = y0 + ((u - 1) + u expm1(-y0)), with u and u - 1 both
// given accurately (so log1p keeps its precision near 0 and log near 1).
__device__ __forceinline__ Dfl log_newton(float y0, Dfl u, Dfl um1) {
  return Dfl{y0, 0.0f} + (um1 + u * dfl_expm1(Dfl{-y0, 0.0f}));
}
// log1p(x) for x > -1 and log(x) for x > 0; relative error about 2^-45 for
// the arguments of this library (|log| < 10)
__device__ __forceinline__ Dfl dfl_log1p(Dfl x) { return log_newton(log1pf(x.hi), x + dflc(1.0), x); }
__device__ __forceinline__ Dfl dfl_log(Dfl x) { return log_newton(logf(x.hi), x, x - dflc(1.0)); }

// FP64 <-> double-float on the integer and FP32 pipes.
// dfl_of: hi is x cut to 24 significant bits, lo the other 29 bits rounded
// to nearest FP32 (|lo| < ulp(hi), about 48 bits in all).  |x| below 2^-60
// keeps hi alone, and below 2^-126 gives 0: the values that go through it
// (densities, potentials, spectra) lie far above.
__device__ __forceinline__ Dfl dfl_of(double x) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const int e = (int)((hw >> 20) & 0x7ff);
  const unsigned sign = hw & 0x80000000u;
  if (e < 897) return {0.f, 0.f};
  if (e > 1150) return {__uint_as_float(sign | 0x7f800000u), 0.f};  // |x| >= 2^128: infinite
  const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  if (e < 963) return {hi, 0.f};
  // lo = r 2^(e - 1075), r the low 29 bits: r = r1 64 + r0 exactly in two
  // FP32 (the 2^23 magic add), one rounding in the FMA, then two exact scalings
  const unsigned r = lw & 0x1fffffffu;
  const float r1 = __uint_as_float(0x4B000000u | (r >> 6)) - 8388608.0f;
  const float r0 = __uint_as_float(0x4B000000u | (r & 63u)) - 8388608.0f;
  const float sc = __uint_as_float((unsigned)(e - 1023 + 127) << 23);  // 2^(e - 1023), normal for e >= 897
  const float lo = fmaf(r1, 64.0f, r0) * 2.220446049250313e-16f * sc;  // * 2^-52 * 2^(e - 1023)
  return {hi, sign ? -lo : lo};
}
// an FP32 as FP64 from its bits (subnormal FP32 give +-0; inf and NaN stay so)
__device__ __forceinline__ double dbl_of_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned sign = u & 0x80000000u;
  if (ex == 0) return __hiloint2double((int)sign, 0);
  const unsigned e64 = ex == 0xffu ? 0x7ffu : ex + 896u;
  return __hiloint2double((int)(sign | (e64 << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
}
// hi + lo as FP64: one FP64 add
__device__ __forceinline__ double dbl_of(Dfl x) { return dbl_of_bits(x.hi) + dbl_of_bits(x.lo); }

}  // namespace
}  // namespace lcp
