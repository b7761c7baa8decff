// The float arc cosine of the host C library the reference is built against, restated so that the
// GPU reproduces it bit for bit.
//
// The reference's quad -> triangle split (cpp_dmc/DualMarchingCubes.cpp:1387-1460, minAngle in
// cpp_dmc/DualMarchingCubes.h:746-756) compares minimum angles obtained with std::acos on floats,
// i.e. the C library's acosf.  That function is not correctly rounded (GNU libc 2.39 differs from
// the correctly rounded arc cosine on 5.4 M of the 2.13 G floats in [-1, 1], at most 0.9 ulp away),
// so a split whose two candidate angles are within an ulp of each other is decided by its exact
// rounding.  GNU libc up to 2.40 computes acosf with fdlibm's method (Sun Microsystems, 1993):
//   |x| < 1/2:  acos x = pi/2 - (x + x R(x^2))
//   x < -1/2:   acos x = pi - 2 (s + s R(z)),     z = (1 + x) / 2, s = sqrt(z)
//   x > 1/2:    acos x = 2 (d + (c + s R(z))),    z = (1 - x) / 2, s = sqrt(z), d = s with its low
//                                                12 bits cleared, c = (z - d^2) / (s + d)
// with R(z) = z P(z) / Q(z), P of degree 5 and Q of degree 4 (the fdlibm asin/acos rational
// approximation; the float coefficients are its float64 coefficients rounded to float), and pi/2
// split into a float head and tail.  Every operation is a single IEEE float operation (no
// contraction: the library is built with -fmad=false, host code with -ffp-contract=off), and sqrt
// and the divisions are correctly rounded on both sides, so host and device results are the same
// floats.  tests/cpp/acos_check.cpp compares this function with the platform's acosf over [-1, 1].
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

// z P(z) / Q(z): the rational part of fdlibm's asin/acos approximation, evaluated by Horner's rule
TMC_LIBM_HD float acos_rational(float z) {
  const float p0 = (float)1.66666666666666657415e-01, p1 = (float)-3.25565818622400915405e-01,
              p2 = (float)2.01212532134862925881e-01, p3 = (float)-4.00555345006794114027e-02,
              p4 = (float)7.91534994289814532176e-04, p5 = (float)3.47933107596021167570e-05;
  const float q1 = (float)-2.40339491173441421878e+00, q2 = (float)2.02094576023350569471e+00,
              q3 = (float)-6.88283971605453293030e-01, q4 = (float)7.70381505559019352791e-02;
  const float num = z * (p0 + z * (p1 + z * (p2 + z * (p3 + z * (p4 + z * p5)))));
  const float den = 1.0f + z * (q1 + z * (q2 + z * (q3 + z * q4)));
  return num / den;
}

TMC_LIBM_HD float acosf(float x) {
  const float pi = bits_to_float(0x40490fdau);         // pi rounded down to float
  const float half_pi_hi = bits_to_float(0x3fc90fdau);  // pi/2 rounded down to float
  const float half_pi_lo = bits_to_float(0x33a22168u);  // pi/2 - half_pi_hi, to float
  const uint32_t bits = float_to_bits(x), mag = bits & 0x7fffffffu;
  const bool neg = (bits >> 31) != 0;
  if (mag == 0x3f800000u) return neg ? pi + 2.0f * half_pi_lo : 0.0f;  // |x| = 1
  if (mag > 0x3f800000u) return (x - x) / (x - x);                    // |x| > 1 or NaN: NaN
  if (mag < 0x3f000000u) {                                             // |x| < 1/2
    if (mag <= 0x23000000u) return half_pi_hi + half_pi_lo;            // |x| <= 2^-57
    const float r = acos_rational(x * x);
    return half_pi_hi - (x - (half_pi_lo - x * r));
  }
  if (neg) {  // x <= -1/2
    const float z = (1.0f + x) * 0.5f;
    const float r = acos_rational(z);
    const float s = sqrtf(z);
    const float w = r * s - half_pi_lo;
    return pi - 2.0f * (s + w);
  }
  // x >= 1/2
  const float z = (1.0f - x) * 0.5f;
  const float s = sqrtf(z);
  const float d = bits_to_float(float_to_bits(s) & 0xfffff000u);
  const float c = (z - d * d) / (s + d);
  const float r = acos_rational(z);
  const float w = r * s + c;
  return 2.0f * (d + w);
}

}  // namespace libm
}  // namespace tmc
