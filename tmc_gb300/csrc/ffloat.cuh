// Float-float ("double-float") arithmetic on the FP32 pipes and certified rounding.
//
// GB300 runs float64 at about 1/57 of the float32 rate (1.19 vs 68 TFLOP/s measured).  The
// reference computes some values as a float64 expression rounded once to float32.  Such a value
// can be reproduced bit-exactly with float32 arithmetic: evaluate the expression as an unevaluated
// sum hi + lo of two floats (~46 significant bits), bound the error against the reference's
// float64 result, and round to float32 only when no float32 rounding midpoint lies within the
// bound.  Otherwise the caller falls back to float64 (probability ~2^-20 per value).
//
// Error-free transformations (Knuth TwoSum, Dekker/FMA TwoProduct) need every + and * rounded on its
// own: the library is compiled with -fmad=false and products that must fuse use fma explicitly.
// The header also compiles as plain host C++ (for the CPU checks in tests/cpp).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define TMC_HD __host__ __device__ __forceinline__
// rare paths stay out of line so that the hot loop fits the instruction cache
#define TMC_HD_COLD inline __host__ __device__ __noinline__
#else
#define TMC_HD inline
#define TMC_HD_COLD inline
#endif

namespace tmc {
namespace ffx {

TMC_HD float fma_rn(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

TMC_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

TMC_HD float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

struct ff {
  float hi, lo;
};

// s + e == a + b exactly
TMC_HD ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
TMC_HD ff quick_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return {s, e};
}
// p + e == a * b exactly
TMC_HD ff two_prod(float a, float b) {
  const float p = a * b;
  const float e = fma_rn(a, b, -p);
  return {p, e};
}

TMC_HD ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  ff t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
TMC_HD ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
TMC_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
TMC_HD ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  p.lo = fma_rn(a.hi, b.lo, p.lo);
  p.lo = fma_rn(a.lo, b.hi, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
TMC_HD ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.hi, b);
  p.lo = fma_rn(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
TMC_HD ff ff_div(ff a, ff b) {
  const float q1 = a.hi / b.hi;
  const ff r = ff_sub(a, ff_mul_f(b, q1));
  const float q2 = r.hi / b.hi;
  const ff r2 = ff_sub(r, ff_mul_f(b, q2));
  const float q3 = r2.hi / b.hi;
  ff q = quick_two_sum(q1, q2);
  return ff_add(q, ff{q3, 0.0f});
}
TMC_HD ff ff_from(float a) { return {a, 0.0f}; }
TMC_HD double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
TMC_HD float ff_abs_hi(ff a) { return a.hi < 0 ? -a.hi : a.hi; }

// A float64 value as a float pair (exact when it has at most ~48 significant bits, else the
// pair is within 2^-48 relative).
TMC_HD ff ff_from_double(double x) {
  const float h = (float)x;
  const float l = (float)(x - (double)h);
  return {h, l};
}

// ulp of |x| for a finite float
TMC_HD float ulpf(float x) {
  const uint32_t e = (fbits(x) >> 23) & 0xFF;
  if (e <= 23) return bitsf(1u);  // subnormal range and tiny normals: the smallest step
  return bitsf((e - 23) << 23);
}

// Round x (within `err` of the reference's float64 value X) to float32 as fl32(X) does.  Returns
// false when a rounding midpoint lies within err (the caller must then compute X in float64).
// x must be normalised (hi = fl(hi + lo)), which every ff_* result is.
TMC_HD bool ff_round(ff x, float err, float& out) {
  const float h = x.hi, l = x.lo;
  if (!(std::isfinite(h))) return false;
  if (h == 0.0f) {
    // |X| <= err: the rounding is only known when nothing but 0 is in reach
    if (err == 0.0f && l == 0.0f) {
      out = 0.0f;
      return true;
    }
    return false;
  }
  const float u = ulpf(h);
  const bool pos = h > 0;
  const float lm = pos ? l : -l;  // lo measured away from zero
  float room;
  if (lm >= 0) {
    room = 0.5f * u - lm;
  } else {
    // below a power of two the next float down is half an ulp away
    const bool pow2 = (fbits(h) & 0x7FFFFF) == 0;
    room = (pow2 ? 0.25f * u : 0.5f * u) + lm;
  }
  if (!(room > err)) return false;
  out = h;
  return true;
}

// smallest float >= x / largest float <= x, for a finite double x
TMC_HD float f_ceil(double x) {
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}
TMC_HD float f_floor(double x) {
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}

}  // namespace ffx
}  // namespace tmc
