// Deterministic single-precision transcendental functions for host and device.
//
// The projection stage derives integer results (tile counts, tile ids, depth
// keys) from float arithmetic that includes exp, log, sin, cos and atan2
// (reference: src/renderer/kernels/compactGaussians.ts:2-19,
// src/renderer/kernels/projectionHelpers.ts:38-70,
// src/renderer/pipeline/ProjectionStage.ts:536-547). Platform math libraries
// differ in their last bits between CPU and GPU, so these functions are written
// from the mathematics using only IEEE-754 add, sub, mul, div and fused
// multiply-add (all correctly rounded on both sides) plus exact bit
// manipulation; the series are evaluated by Horner steps, each one fused
// multiply-add:
//
//   exp   : Cody-Waite reduction x = n ln2 + r, |r| <= ln2/2, Taylor series of
//           e^r to degree 8, scaling by 2^n through exact exponent arithmetic.
//   log   : x = 2^e m with m in (sqrt(1/2), sqrt(2)], log m = 2 atanh(s),
//           s = (m-1)/(m+1), odd series to s^11.
//   sin/cos: reduction by k pi/2 with a three-part split of pi/2, Taylor series
//           on |r| <= pi/4 (sin to r^11, cos to r^12), quadrant selection.
//   atan2 : C99 special-case semantics; reduction to a = min/max in (0,1],
//           atan a = pi/4 + atan((a-1)/(a+1)) for a > tan(pi/8), odd Taylor
//           series to t^21 on |t| <= tan(pi/8).
//
// Every constant below is a Taylor coefficient 1/k!, 1/(2k+1), or a split of
// pi/2, ln 2 computed for this file. Accuracy is a few ULP (tests compare with
// float64 numpy), well inside the WGSL accuracy bounds the reference runs under.
//
// Bit-identical results on host and device need the two compilers to evaluate
// the same operation sequence: device translation units that include this file
// for exact stages are built with --fmad=false, host code with
// -ffp-contract=off, and neither side uses fast-math or flush-to-zero; the
// fused steps are explicit (GS_FMA: __fmaf_rn on the device, C99 fmaf on the
// host, both the correctly rounded a * b + c).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDA_ARCH__)
#define GS_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define GS_FMA(a, b, c) fmaf((a), (b), (c))
#endif

#if defined(__CUDACC__)
#define GS_HD __host__ __device__ __forceinline__
#else
#define GS_HD static inline
#endif

namespace gsdm {

GS_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

GS_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

GS_HD float inf() { return u2f(0x7f800000u); }
GS_HD float qnan() { return u2f(0x7fc00000u); }
GS_HD bool isnan_(float x) { return x != x; }
GS_HD float fabs_(float x) { return u2f(f2u(x) & 0x7fffffffu); }
GS_HD float copysign_(float mag, float sgn) {
  return u2f((f2u(mag) & 0x7fffffffu) | (f2u(sgn) & 0x80000000u));
}

// 2^n for n in [-149, 127], exact (subnormal for n < -126).
GS_HD float pow2i(int n) {
  if (n >= -126) return u2f((uint32_t)(n + 127) << 23);
  return u2f(1u << (n + 149));
}

// p * 2^n with a single final rounding (p in [0.5, 2], n in [-152, 130]).
GS_HD float scale2(float p, int n) {
  if (n > 127) return (p * pow2i(127)) * pow2i(n - 127);
  if (n < -126) return (p * pow2i(n + 126)) * pow2i(-126);
  return p * pow2i(n);
}

// Half-to-even rounding of a float holding a value below 2^22 in magnitude.
GS_HD float round_even_small(float x) {
  // Adding and subtracting 1.5 * 2^23 rounds to an integer under the default
  // round-to-nearest-even mode on both host and device.
  const float magic = 12582912.0f;
  return (x + magic) - magic;
}

GS_HD float expf_(float x) {
  if (isnan_(x)) return x;
  if (x > 88.72283935546875f) return inf();
  if (x < -103.972084045410156f) return 0.0f;
  const float LOG2E = 1.44269502162933349609375f;
  const float LN2_HI = 0.693145751953125f;           // 0x3f317200
  const float LN2_LO = 1.428606765330187045037746e-06f;
  float n = round_even_small(x * LOG2E);
  float r = (x - n * LN2_HI) - n * LN2_LO;
  // Taylor coefficients 1/k!
  float p = 2.4801587301587302e-05f;                 // 1/8!
  p = GS_FMA(r, p, 1.9841269841269841e-04f);               // 1/7!
  p = GS_FMA(r, p, 1.3888888888888889e-03f);               // 1/6!
  p = GS_FMA(r, p, 8.3333333333333333e-03f);               // 1/5!
  p = GS_FMA(r, p, 4.1666666666666667e-02f);               // 1/4!
  p = GS_FMA(r, p, 1.6666666666666667e-01f);               // 1/3!
  p = GS_FMA(r, p, 0.5f);
  p = GS_FMA(r, p, 1.0f);
  p = GS_FMA(r, p, 1.0f);
  return scale2(p, (int)n);
}

GS_HD float logf_(float x) {
  if (isnan_(x) || x < 0.0f) return qnan();
  if (x == 0.0f) return -inf();
  if (x == inf()) return x;
  uint32_t b = f2u(x);
  int eadj = 0;
  if ((b >> 23) == 0u) {  // subnormal: scale into the normal range exactly
    x = x * 8388608.0f;
    b = f2u(x);
    eadj = -23;
  }
  int e = (int)((b >> 23) & 0xffu) - 127 + eadj;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421353816986083984375f) {
    m = m * 0.5f;
    e += 1;
  }
  // With f = m - 1 (exact) and s = f / (2 + f): log m = 2 atanh(s)
  // = 2s (1 + z/3 + z^2/5 + ... + z^5/11), z = s^2, and 2s = f - f s,
  // so log m = f - (f s - 2s q) keeps the dominant term f exact.
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float q = 9.0909090909090909e-02f;                 // 1/11
  q = GS_FMA(z, q, 1.1111111111111111e-01f);               // 1/9
  q = GS_FMA(z, q, 1.4285714285714286e-01f);               // 1/7
  q = GS_FMA(z, q, 2.0000000000000000e-01f);               // 1/5
  q = GS_FMA(z, q, 3.3333333333333333e-01f);               // 1/3
  q = z * q;
  float lm = f - (f * s - (2.0f * s) * q);
  const float LN2_HI = 0.693145751953125f;
  const float LN2_LO = 1.428606765330187045037746e-06f;
  float fe = (float)e;
  return fe * LN2_HI + (fe * LN2_LO + lm);
}

// sin and cos of r with |r| <= pi/4 (Taylor series).
GS_HD float sin_poly(float r) {
  float z = r * r;
  float p = -2.5052108385441720e-08f;                // -1/11!
  p = GS_FMA(z, p, 2.7557319223985891e-06f);               // 1/9!
  p = GS_FMA(z, p, -1.9841269841269841e-04f);              // -1/7!
  p = GS_FMA(z, p, 8.3333333333333333e-03f);               // 1/5!
  p = GS_FMA(z, p, -1.6666666666666667e-01f);              // -1/3!
  return GS_FMA(r * z, p, r);
}

GS_HD float cos_poly(float r) {
  float z = r * r;
  float p = 2.0876756987868099e-09f;                 // 1/12!
  p = GS_FMA(z, p, -2.7557319223985891e-07f);              // -1/10!
  p = GS_FMA(z, p, 2.4801587301587302e-05f);               // 1/8!
  p = GS_FMA(z, p, -1.3888888888888889e-03f);              // -1/6!
  p = GS_FMA(z, p, 4.1666666666666667e-02f);               // 1/4!
  p = GS_FMA(z, p, -0.5f);
  return GS_FMA(z, p, 1.0f);
}

// Reduce x to r in [-pi/4, pi/4] (approximately) and quadrant q = k mod 4.
GS_HD float reduce_pio2(float x, int* q) {
  const float TWO_OVER_PI = 0.636619746685028076171875f;
  const float PIO2_1 = 1.5703125f;                        // 0x3fc90000
  const float PIO2_2 = 4.838705062866210938e-04f;         // 0x39fdb000
  const float PIO2_3 = -4.371138828673792933e-08f;        // 0xb33bbd2e
  float k = round_even_small(x * TWO_OVER_PI);
  float r = ((x - k * PIO2_1) - k * PIO2_2) - k * PIO2_3;
  *q = ((int)k) & 3;
  return r;
}

// Valid for |x| <= 4096 (the pass only needs |x| <= pi/2).
GS_HD float sinf_(float x) {
  if (isnan_(x) || fabs_(x) == inf()) return qnan();
  int q;
  float r = reduce_pio2(x, &q);
  float s = sin_poly(r), c = cos_poly(r);
  switch (q) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
  }
}

GS_HD float cosf_(float x) {
  if (isnan_(x) || fabs_(x) == inf()) return qnan();
  int q;
  float r = reduce_pio2(x, &q);
  float s = sin_poly(r), c = cos_poly(r);
  switch (q) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
  }
}

// atan(t) for |t| <= tan(pi/8): odd Taylor series to t^21.
GS_HD float atan_poly(float t) {
  float z = t * t;
  float p = 4.7619047619047619e-02f;                 // 1/21
  p = GS_FMA(z, p, -5.2631578947368421e-02f);              // -1/19
  p = GS_FMA(z, p, 5.8823529411764706e-02f);               // 1/17
  p = GS_FMA(z, p, -6.6666666666666667e-02f);              // -1/15
  p = GS_FMA(z, p, 7.6923076923076923e-02f);               // 1/13
  p = GS_FMA(z, p, -9.0909090909090909e-02f);              // -1/11
  p = GS_FMA(z, p, 1.1111111111111111e-01f);               // 1/9
  p = GS_FMA(z, p, -1.4285714285714286e-01f);              // -1/7
  p = GS_FMA(z, p, 2.0000000000000000e-01f);               // 1/5
  p = GS_FMA(z, p, -3.3333333333333333e-01f);              // -1/3
  return GS_FMA(t * z, p, t);
}

GS_HD float atan2f_(float y, float x) {
  const float PI = 3.1415927410125732421875f;
  const float PI_LO = -8.742277657347585773e-08f;
  const float PIO2 = 1.57079637050628662109375f;
  const float PIO2_LO = -4.371138828673792933e-08f;
  const float PIO4 = 0.785398185253143310546875f;
  const float PIO4_LO = -2.185569414336896467e-08f;
  const float TAN_PI8 = 0.4142135679721832275390625f;
  if (isnan_(x) || isnan_(y)) return x + y;
  float ax = fabs_(x), ay = fabs_(y);
  bool xneg = (f2u(x) >> 31) != 0u;
  if (ay == inf()) {
    if (ax == inf()) return copysign_(xneg ? 3.0f * PIO4 : PIO4, y);
    return copysign_(PIO2, y);
  }
  if (ax == inf()) return copysign_(xneg ? PI : 0.0f, y);
  if (ay == 0.0f) return copysign_(xneg ? PI : 0.0f, y);
  if (ax == 0.0f) return copysign_(PIO2, y);
  bool swap = ay > ax;
  float a = swap ? ax / ay : ay / ax;  // (0, 1]
  float res;
  if (a > TAN_PI8) {
    float t = (a - 1.0f) / (a + 1.0f);
    res = PIO4 + (PIO4_LO + atan_poly(t));
  } else {
    res = atan_poly(a);
  }
  if (swap) res = PIO2 + (PIO2_LO - res);
  if (xneg) res = PI + (PI_LO - res);
  return copysign_(res, y);
}

// IEEE binary16 bits -> float (exact, subnormals included).
GS_HD float half_bits_to_float(uint32_t h) {
  uint32_t sign = (h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu;
  uint32_t m = h & 0x3ffu;
  if (e == 0u) {
    // value = m * 2^-24, exact in float
    float v = (float)m * 5.9604644775390625e-08f;
    return u2f(f2u(v) | sign);
  }
  if (e == 31u) return u2f(sign | 0x7f800000u | (m << 13));
  return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

GS_HD float clampf_(float x, float lo, float hi) {
  float y = x < lo ? lo : x;
  return y > hi ? hi : y;
}

}  // namespace gsdm
