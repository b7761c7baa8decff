// The float arc cosine of the host C library the reference is built against, restated so that the
// GPU reproduces it bit for bit.
//
// The reference's quad -> triangle split (cpp_dmc/DualMarchingCubes.cpp:1387-1460, minAngle in
// cpp_dmc/DualMarchingCubes.h:746-756) compares minimum angles obtained with std::acos on floats,
// i.e. the C library's acosf.  That function is not correctly rounded in GNU libc up to 2.40 (2.39
// on x86-64 differs from the correctly rounded arc cosine on 5.4 M of the 2.13 G floats in [-1, 1],
// at most 0.9 ulp away), so a split whose two candidate angles are within an ulp of each other is
// decided by its exact rounding, and that rounding differs between machines.
//
// GNU libc up to 2.40 computes acosf with fdlibm's method (Sun Microsystems, 1993):
//   |x| < 1/2:  acos x = pi/2 - (x - (pi/2_lo - x R(x^2)))
//   x < -1/2:   acos x = pi - 2 (s + (R(z) s - pi/2_lo)),  z = (1 + x) / 2, s = sqrt(z)
//   x > 1/2:    acos x = 2 (d + (R(z) s + c)),             z = (1 - x) / 2, s = sqrt(z), d = s with
//                                                          its low 12 bits cleared, c = (z - d^2)/(s + d)
// with R(z) = z P(z) / Q(z), P of degree 5 and Q of degree 4 in Horner form (the fdlibm asin/acos
// rational approximation; the float coefficients are its float64 coefficients rounded to float), and
// pi/2 split into a float head and tail.  The same source gives two different functions:
//   kAcosfSeparate  every product and sum rounded on its own (x86-64 builds: no fused multiply-add)
//   kAcosfFused     every product that feeds a sum fused with it (aarch64 builds: the compiler
//                   contracts them), i.e. the Horner steps, x R, R s and d^2 against their addends
// A correctly rounded acosf (GNU libc 2.41 and later) is the third kind, kAcosfCorrect, computed here
// by rounding the float64 arc cosine once.  host_acosf_kind() (runtime) tells which one the host
// library is; tests/cpp/acos_check.cpp checks the restatements against it over all of [-1, 1].
//
// Every operation is a single IEEE float operation (the library is built with -fmad=false for device
// code and -ffp-contract=off for host code; fused steps are explicit fmaf), and sqrt and the
// divisions are correctly rounded on both sides, so host and device results are the same floats.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

#if defined(__CUDACC__)
#define TMC_LIBM_HD __host__ __device__ __forceinline__
#else
#define TMC_LIBM_HD inline
#endif

namespace tmc {
namespace libm {

enum { kAcosfSeparate = 0, kAcosfFused = 1, kAcosfCorrect = 2 };

TMC_LIBM_HD float bits_to_float(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
TMC_LIBM_HD uint32_t float_to_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

// a * b + c, fused or with two roundings
template <bool kFused>
TMC_LIBM_HD float mul_add(float a, float b, float c) {
  if (kFused) return fmaf(a, b, c);
  const float p = a * b;
  return p + c;
}

// z P(z) / Q(z): the rational part of fdlibm's asin/acos approximation, by Horner's rule
template <bool kFused>
TMC_LIBM_HD float acos_rational(float z) {
  const float p0 = (float)1.66666666666666657415e-01, p1 = (float)-3.25565818622400915405e-01,
              p2 = (float)2.01212532134862925881e-01, p3 = (float)-4.00555345006794114027e-02,
              p4 = (float)7.91534994289814532176e-04, p5 = (float)3.47933107596021167570e-05;
  const float q1 = (float)-2.40339491173441421878e+00, q2 = (float)2.02094576023350569471e+00,
              q3 = (float)-6.88283971605453293030e-01, q4 = (float)7.70381505559019352791e-02;
  float t = mul_add<kFused>(z, p5, p4);
  t = mul_add<kFused>(z, t, p3);
  t = mul_add<kFused>(z, t, p2);
  t = mul_add<kFused>(z, t, p1);
  t = mul_add<kFused>(z, t, p0);
  const float num = z * t;
  float u = mul_add<kFused>(z, q4, q3);
  u = mul_add<kFused>(z, u, q2);
  u = mul_add<kFused>(z, u, q1);
  const float den = mul_add<kFused>(z, u, 1.0f);
  return num / den;
}

template <bool kFused>
TMC_LIBM_HD float acosf_fdlibm(float x) {
  const float pi = bits_to_float(0x40490fdau);         // pi rounded down to float
  const float half_pi_hi = bits_to_float(0x3fc90fdau);  // pi/2 rounded down to float
  const float half_pi_lo = bits_to_float(0x33a22168u);  // pi/2 - half_pi_hi, to float
  const uint32_t bits = float_to_bits(x), mag = bits & 0x7fffffffu;
  const bool neg = (bits >> 31) != 0;
  if (mag == 0x3f800000u) return neg ? pi + 2.0f * half_pi_lo : 0.0f;  // |x| = 1
  if (mag > 0x3f800000u) return (x - x) / (x - x);                    // |x| > 1 or NaN: NaN
  if (mag < 0x3f000000u) {                                             // |x| < 1/2
    if (mag <= 0x23000000u) return half_pi_hi + half_pi_lo;            // |x| <= 2^-57
    const float r = acos_rational<kFused>(x * x);
    return half_pi_hi - (x - mul_add<kFused>(-x, r, half_pi_lo));
  }
  if (neg) {  // x <= -1/2
    const float z = (1.0f + x) * 0.5f;
    const float r = acos_rational<kFused>(z);
    const float s = sqrtf(z);
    const float w = mul_add<kFused>(r, s, -half_pi_lo);
    return pi - 2.0f * (s + w);  // 2 (s + w) is exact: fused or not, one rounding
  }
  // x >= 1/2
  const float z = (1.0f - x) * 0.5f;
  const float s = sqrtf(z);
  const float d = bits_to_float(float_to_bits(s) & 0xfffff000u);
  const float c = mul_add<kFused>(-d, d, z) / (s + d);
  const float r = acos_rational<kFused>(z);
  const float w = mul_add<kFused>(r, s, c);
  return 2.0f * (d + w);
}

// The host library's acosf of the given kind
TMC_LIBM_HD float acosf_kind(float x, int kind) {
  if (kind == kAcosfFused) return acosf_fdlibm<true>(x);
  if (kind == kAcosfSeparate) return acosf_fdlibm<false>(x);
  return (float)acos((double)x);
}

// Which kind the host C library's acosf is: its results on a fixed sample of [-1, 1] compared with
// each restatement.  The sample is uniform in value (the two fdlibm kinds differ on about 1 % of the
// floats above 1/2 in magnitude, 0.01 % overall) plus inputs known to separate them; the first kind
// that matches every sample is taken, the correctly rounded one when neither fdlibm kind does.
// Evaluated once per process (host code).
inline int host_acosf_kind() {
  static const int kind = [] {
    bool sep = true, fused = true;
    auto check = [&](float x) {
      const uint32_t want = float_to_bits(std::acos(x));
      sep = sep && float_to_bits(acosf_fdlibm<false>(x)) == want;
      fused = fused && float_to_bits(acosf_fdlibm<true>(x)) == want;
    };
    const uint32_t known[] = {0x3c6caf76u, 0x3ca42679u, 0xbc5e5dafu, 0x3d40791du, 0xbd3aa98du};
    for (uint32_t b : known) check(bits_to_float(b));
    uint64_t state = 0x9e3779b97f4a7c15ull;
    for (int q = 0; q < 65536 && (sep || fused); q++) {
      state ^= state << 13;
      state ^= state >> 7;
      state ^= state << 17;
      const double u = (double)(state >> 11) * 0x1p-53;  // [0, 1)
      check((float)(2.0 * u - 1.0));
    }
    return sep ? kAcosfSeparate : fused ? kAcosfFused : kAcosfCorrect;
  }();
  return kind;
}

}  // namespace libm
}  // namespace tmc
