// Portable single-precision transcendental functions for the render path.
//
// The reference evaluates std::sin / std::cos / std::asin / std::acos /
// std::pow (include/bsdf/diffuse.h:30-45, include/bsdf/glossy.h:26-49,
// include/lib/projection.h:9-32, include/bsdf/dielectric_refractive.h:24-33,
// include/integrate/term_prob/multiplier_func/multiplier_func.h:19-30).  The
// C library and CUDA implement those functions differently in the last bit,
// and a path tracer turns a one-ulp change in a bounce direction into a
// different path now and then.  These functions are therefore evaluated by
// our own polynomials (coefficients fitted by gen_pmath.py) using only IEEE
// single-precision +, -, *, / and sqrt, which CPU and GPU round identically.
// Translation units that include this header must not contract a*b+c into a
// fused multiply-add (host: -ffp-contract=off, device: --fmad=false).
//
// Accuracy (float32 ulps against the exact function): the polynomial
// kernels are within 1.5 ulps on their reduced ranges (gen_pmath.py); after
// argument reduction sin / cos are within 4e-7 absolute on [-2 pi, 2 pi],
// asin / acos within 3 ulps on [-1, 1]; pow is evaluated in double precision
// and is within 1 ulp (tests/test_oracle_pins.py::test_pmath_accuracy).
#pragma once

#include <stdint.h>

#include "pmath_coeffs.h"

#if defined(__CUDACC__)
#define PM_HD __host__ __device__ __forceinline__
#define PM_HDM __host__ __device__ __forceinline__
#else
#define PM_HD static inline
#define PM_HDM inline
#include <math.h>
#include <string.h>
#endif

namespace pm {

PM_HD uint32_t as_uint(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

PM_HD float as_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

PM_HD float sqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return sqrtf(x);
#endif
}

PM_HD float fabs(float x) { return as_float(as_uint(x) & 0x7fffffffu); }

// round to nearest integer, ties to even (the IEEE default rounding mode)
PM_HD float rint(float x) {
#if defined(__CUDA_ARCH__)
  return rintf(x);
#else
  return nearbyintf(x);
#endif
}

PM_HD float copysign(float mag, float sgn) {
  return as_float((as_uint(mag) & 0x7fffffffu) | (as_uint(sgn) & 0x80000000u));
}

PM_HD bool isfinite(float x) {
  return (as_uint(x) & 0x7f800000u) != 0x7f800000u;
}

// Horner evaluation, constant term first in the coefficient list.
template <int N>
PM_HD float horner(const float (&c)[N], float x) {
  float acc = c[N - 1];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = N - 2; i >= 0; --i) {
    acc = acc * x;
    acc = acc + c[i];
  }
  return acc;
}

// pi/2 split in three parts; the first two have trailing zero bits so that
// k * part is exact for the quadrant counts that occur here (Cody-Waite).
#define PM_PIO2_1 0x1.92p+0f
#define PM_PIO2_2 0x1.fb4p-12f
#define PM_PIO2_3 0x1.4442d2p-24f
#define PM_TWO_OVER_PI 0x1.45f306p-1f
#define PM_PIO2_HI 0x1.921fb6p+0f
#define PM_PIO2_LO -0x1.777a5cp-25f
#define PM_PI_HI 0x1.921fb6p+1f
#define PM_PI_LO -0x1.777a5cp-24f
#define PM_SQRT2 0x1.6a09e6p+0f

// sin and cos on |r| <= pi/4
PM_HD float sin_kernel(float r) {
  const float c[] = PM_SIN_COEFFS;
  float r2 = r * r;
  float r3 = r * r2;
  return r + r3 * horner(c, r2);
}

PM_HD float cos_kernel(float r) {
  const float c[] = PM_COS_COEFFS;
  float r2 = r * r;
  float half = 0.5f * r2;
  float r4 = r2 * r2;
  return (1.0f - half) + r4 * horner(c, r2);
}

PM_HD void sincos(float x, float *s_out, float *c_out) {
  if (!isfinite(x)) {
    float nan = x - x;
    *s_out = nan;
    *c_out = nan;
    return;
  }
  float kf = rint(x * PM_TWO_OVER_PI);
  float r = x - kf * PM_PIO2_1;
  r = r - kf * PM_PIO2_2;
  r = r - kf * PM_PIO2_3;
  int q = ((int)kf) & 3;
  float s = sin_kernel(r);
  float c = cos_kernel(r);
  switch (q) {
  case 0:
    *s_out = s;
    *c_out = c;
    break;
  case 1:
    *s_out = c;
    *c_out = -s;
    break;
  case 2:
    *s_out = -s;
    *c_out = -c;
    break;
  default:
    *s_out = -c;
    *c_out = s;
    break;
  }
}

PM_HD float sin(float x) {
  float s, c;
  sincos(x, &s, &c);
  return s;
}

PM_HD float cos(float x) {
  float s, c;
  sincos(x, &s, &c);
  return c;
}

// asin(x) for 0 <= x <= 0.5 (also used on sqrt((1 - |x|) / 2) <= 0.5)
PM_HD float asin_kernel(float x) {
  const float c[] = PM_ASIN_COEFFS;
  float x2 = x * x;
  float x3 = x * x2;
  return x + x3 * horner(c, x2);
}

// asin(x) = pi/2 - 2 asin(sqrt((1 - x) / 2)) for x > 0.5
PM_HD float asin(float x) {
  float ax = fabs(x);
  float r;
  if (ax <= 0.5f) {
    r = asin_kernel(ax);
  } else {
    float z = (1.0f - ax) * 0.5f;
    float s = sqrt(z);
    float a = asin_kernel(s);
    r = PM_PIO2_HI - (2.0f * a - PM_PIO2_LO);
  }
  return copysign(r, x);
}

PM_HD float acos(float x) {
  if (fabs(x) <= 0.5f) {
    float a = copysign(asin_kernel(fabs(x)), x);
    return PM_PIO2_HI - (a - PM_PIO2_LO);
  }
  if (x > 0.5f) {
    float z = (1.0f - x) * 0.5f;
    float s = sqrt(z);
    return 2.0f * asin_kernel(s);
  }
  float z = (1.0f + x) * 0.5f;
  float s = sqrt(z);
  float a = asin_kernel(s);
  return PM_PI_HI - (2.0f * a - PM_PI_LO);
}

// ---- pow, evaluated in double precision --------------------------------
// pow(x, y) = 2^(y log2 x) with log2 and exp2 evaluated in IEEE double (+, -,
// *, / only, which host and device round identically; no contraction) and
// the result rounded once to float, so it is within one float ulp of the
// exact power (tests/test_oracle_pins.py::test_pmath_accuracy).  log2 of the
// mantissa m in [sqrt(1/2), sqrt(2)) is 2 atanh(s) / ln 2 with s = (m - 1) /
// (m + 1), |s| <= 0.1716, by its Taylor series to s^25 (truncation below
// 1e-19); 2^f for |f| <= 1/2 is exp(f ln 2) by its Taylor series to degree
// 14 (truncation below 1e-18).

PM_HD uint64_t as_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

PM_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

// round to nearest, ties to even, for |t| < 2^51
PM_HD double rint_d(double t) {
  const double shift = 6755399441055744.0; // 1.5 * 2^52
  double r = t + shift;
  return r - shift;
}

// log2 of a positive normal double
PM_HD double log2_d(double x) {
  uint64_t b = as_bits(x);
  int e = (int)((b >> 52) & 0x7ffu) - 1023;
  double m = from_bits((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  double s = (m - 1.0) / (m + 1.0);
  double s2 = s * s;
  double p = 1.0 / 25.0;
  p = p * s2 + 1.0 / 23.0;
  p = p * s2 + 1.0 / 21.0;
  p = p * s2 + 1.0 / 19.0;
  p = p * s2 + 1.0 / 17.0;
  p = p * s2 + 1.0 / 15.0;
  p = p * s2 + 1.0 / 13.0;
  p = p * s2 + 1.0 / 11.0;
  p = p * s2 + 1.0 / 9.0;
  p = p * s2 + 1.0 / 7.0;
  p = p * s2 + 1.0 / 5.0;
  p = p * s2 + 1.0 / 3.0;
  p = p * s2 + 1.0;
  // 2 / ln 2
  return (double)e + (2.8853900817779268 * s) * p;
}

// 2^t for -1100 < t < 1100
PM_HD double exp2_d(double t) {
  double n = rint_d(t);
  double g = (t - n) * 0.69314718055994531; // ln 2
  double p = 1.0 / 87178291200.0;           // 1/14!
  p = p * g + 1.0 / 6227020800.0;
  p = p * g + 1.0 / 479001600.0;
  p = p * g + 1.0 / 39916800.0;
  p = p * g + 1.0 / 3628800.0;
  p = p * g + 1.0 / 362880.0;
  p = p * g + 1.0 / 40320.0;
  p = p * g + 1.0 / 5040.0;
  p = p * g + 1.0 / 720.0;
  p = p * g + 1.0 / 120.0;
  p = p * g + 1.0 / 24.0;
  p = p * g + 1.0 / 6.0;
  p = p * g + 0.5;
  p = p * g + 1.0;
  p = p * g + 1.0;
  // scale by 2^n in two steps so both factors are normal doubles
  int k = (int)n;
  int k1 = k / 2;
  int k2 = k - k1;
  double s1 = from_bits((uint64_t)(k1 + 1023) << 52);
  double s2 = from_bits((uint64_t)(k2 + 1023) << 52);
  return (p * s1) * s2;
}

// pow for x >= 0 (every use in the renderer has a non-negative base)
PM_HD float pow(float x, float y) {
  if (y == 0.0f || x == 1.0f) {
    return 1.0f;
  }
  if (x == 0.0f) {
    return y > 0.0f ? 0.0f : as_float(0x7f800000u);
  }
  if (!(x > 0.0f) || !(y == y)) {
    return as_float(0x7fc00000u);
  }
  if (!isfinite(x) || !isfinite(y)) {
    // the limits of 2^(y log2 x): infinite or zero by the sign of y log2 x
    // (x == 1 was handled above, so that product is not zero)
    double lx = isfinite(x) ? log2_d((double)x) : 1.0;
    return (double)y * lx > 0.0 ? as_float(0x7f800000u) : 0.0f;
  }
  double t = (double)y * log2_d((double)x);
  if (t > 129.0) {
    return as_float(0x7f800000u);
  }
  if (t < -151.0) {
    return 0.0f;
  }
  return (float)exp2_d(t);
}

} // namespace pm
