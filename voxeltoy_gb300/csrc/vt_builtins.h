// vt_builtins.h — single-precision definitions of the GLSL builtins whose
// precision the GLSL specification leaves to the implementation (sin, cos,
// pow, acos, atan2) plus the exactly-specified helpers (min, max, sign, step,
// mod) with their GLSL definitions, and IEEE half <-> float conversion.
//
// The reference shaders (src/shaders/shared/sampling.h:2-43,
// src/shaders/shared/coordinates.h:84-116, src/shaders/bsdf/microfacet.h:24-68,
// src/shaders/integrator/pathTracer.fs:191,294) call these builtins; GL drivers
// evaluate them with unspecified error.  This header fixes one definition so
// that the CUDA kernels and the FP32 CPU restatement evaluate the exact same
// sequence of IEEE-754 single-precision operations and therefore agree bit for
// bit.  Each function names the published method it implements:
//
//   sin/cos   Cody & Waite argument reduction by pi/2 with a three-part
//             constant ("Software Manual for the Elementary Functions", 1980),
//             then the Taylor series of sin and cos on [-pi/4, pi/4].
//   log2      exponent/mantissa split, mantissa in [sqrt(1/2), sqrt(2)),
//             ln(m) = 2 atanh((m-1)/(m+1)) by its odd power series.
//   exp2      2^y = 2^k * e^(f ln 2), k = rint(y), Taylor series of e^x.
//   pow       exp2(y * log2(x)); y == 5 (Schlick) as (x*x)^2 * x.
//   atan      reduction to [0, tan(pi/12)] by the identities
//             atan(t) = pi/2 - atan(1/t) and
//             atan(t) = pi/6 + atan((sqrt(3) t - 1) / (sqrt(3) + t))
//             (Hart et al., "Computer Approximations", 1968), then the
//             Taylor series of atan.
//   acos      acos(x) = atan2(sqrt((1-x)(1+x)), x).
//
// Polynomials are evaluated in Horner form with fused multiply-add, which is
// correctly rounded on both the GPU and the host C library, so host and device
// agree exactly.  Accuracy against float64 libm is checked by the CPU test
// suite (a few ulp over the argument ranges the renderer uses).
//
// Domain conventions where GLSL says "undefined": pow(x<=0, y) returns 0 for
// y != 0 and 1 for y == 0; acos clamps its argument to [-1, 1]; atan2(0, 0) = 0.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define VT_HD __host__ __device__ __forceinline__
#else
#define VT_HD static inline
#endif

namespace vtb {

// ---- bit casts -------------------------------------------------------------
VT_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
VT_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f; memcpy(&f, &u, 4); return f;
#endif
}

// ---- exactly specified GLSL helpers -----------------------------------------
// GLSL 4.30 section 8.3: min(x, y) = y < x ? y : x; max(x, y) = x < y ? y : x.
VT_HD float gmin(float x, float y) { return y < x ? y : x; }
VT_HD float gmax(float x, float y) { return x < y ? y : x; }
VT_HD double gmin(double x, double y) { return y < x ? y : x; }
VT_HD double gmax(double x, double y) { return x < y ? y : x; }
// sign(x): 1.0 if x > 0, 0.0 if x == 0, -1.0 if x < 0.
VT_HD float gsign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
VT_HD double gsign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
// step(edge, x): 0.0 if x < edge, else 1.0.
VT_HD bool gstep(float edge, float x) { return !(x < edge); }
VT_HD bool gstep(double edge, double x) { return !(x < edge); }

VT_HD float vfma(float a, float b, float c) { return fmaf(a, b, c); }
VT_HD float vrint(float x) { return rintf(x); }
VT_HD float vfloor(float x) { return floorf(x); }
VT_HD float vsqrt(float x) { return sqrtf(x); }
VT_HD float vabs(float x) { return fabsf(x); }

// ---- sin / cos ---------------------------------------------------------------
// pi/2 = C1 + C2 + C3 with C1 (8 significant bits) and C2 (10 significant
// bits) chosen so that k*C1 and k*C2 are exact for |k| < 2^13.
#define VTB_PIO2_C1 1.5703125f
#define VTB_PIO2_C2 4.8351287841796875e-4f
#define VTB_PIO2_C3 3.139164786e-7f
#define VTB_TWO_OVER_PI 0.636619772367581343f

// Taylor series of sin(r) and cos(r) for |r| <= pi/4; truncation error below
// 1e-11, far under one float ulp.
VT_HD float sin_poly(float r) {
  const float r2 = r * r;
  float p = -2.50521083854417188e-8f;          // -1/11!
  p = vfma(p, r2, 2.75573192239858907e-6f);    //  1/9!
  p = vfma(p, r2, -1.98412698412698413e-4f);   // -1/7!
  p = vfma(p, r2, 8.33333333333333333e-3f);    //  1/5!
  p = vfma(p, r2, -1.66666666666666667e-1f);   // -1/3!
  return vfma(p * r2, r, r);
}
VT_HD float cos_poly(float r) {
  const float r2 = r * r;
  float p = 2.08767569878680990e-9f;           //  1/12!
  p = vfma(p, r2, -2.75573192239858907e-7f);   // -1/10!
  p = vfma(p, r2, 2.48015873015873016e-5f);    //  1/8!
  p = vfma(p, r2, -1.38888888888888889e-3f);   // -1/6!
  p = vfma(p, r2, 4.16666666666666667e-2f);    //  1/4!
  p = vfma(p, r2, -0.5f);                      // -1/2!
  return vfma(p, r2, 1.0f);
}
// Reduce x to r in [-pi/4, pi/4] and quadrant q = k mod 4.
VT_HD float reduce_pio2(float x, int* q) {
  const float k = vrint(x * VTB_TWO_OVER_PI);
  float r = x - k * VTB_PIO2_C1;
  r = r - k * VTB_PIO2_C2;
  r = r - k * VTB_PIO2_C3;
  *q = ((int)k) & 3;
  return r;
}
VT_HD float vsin(float x) {
  int q; const float r = reduce_pio2(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  switch (q) { case 0: return s; case 1: return c; case 2: return -s; default: return -c; }
}
VT_HD float vcos(float x) {
  int q; const float r = reduce_pio2(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  switch (q) { case 0: return c; case 1: return -s; case 2: return -c; default: return s; }
}

// ---- log2 / exp2 / pow --------------------------------------------------------
VT_HD float vlog2(float x) {
  // x > 0 and finite is the caller's contract (pow handles the rest).
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }   // subnormal
  uint32_t u = f2u(x);
  e += (int)((u >> 23) & 0xff) - 127;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u);             // [1, 2)
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }               // [0.707, 1.414]
  const float s = (m - 1.0f) / (m + 1.0f);                      // |s| <= 0.1716
  const float s2 = s * s;
  float p = 1.0f / 11.0f;
  p = vfma(p, s2, 1.0f / 9.0f);
  p = vfma(p, s2, 1.0f / 7.0f);
  p = vfma(p, s2, 1.0f / 5.0f);
  p = vfma(p, s2, 1.0f / 3.0f);
  const float ln_m = 2.0f * vfma(p * s2, s, s);                // 2 atanh(s)
  return vfma(ln_m, 1.44269504088896341f, (float)e);            // e + ln(m)/ln 2
}
VT_HD float vexp2(float y) {
  if (y != y) return y;
  if (y >= 128.0f) return u2f(0x7f800000u);
  if (y < -150.0f) return 0.0f;
  const float k = vrint(y);
  const float g = (y - k) * 0.693147180559945309f;              // |g| <= 0.3466
  float p = 2.48015873015873016e-5f;                             // 1/8!
  p = vfma(p, g, 1.98412698412698413e-4f);                       // 1/7!
  p = vfma(p, g, 1.38888888888888889e-3f);                       // 1/6!
  p = vfma(p, g, 8.33333333333333333e-3f);                       // 1/5!
  p = vfma(p, g, 4.16666666666666667e-2f);                       // 1/4!
  p = vfma(p, g, 1.66666666666666667e-1f);                       // 1/3!
  p = vfma(p, g, 0.5f);                                          // 1/2!
  p = vfma(p, g, 1.0f);
  p = vfma(p, g, 1.0f);
  int ki = (int)k;
  // scale by 2^k in two steps so that subnormal results are produced correctly
  if (ki < -126) { p = p * 5.9604644775390625e-8f; ki += 24; }   // 2^-24
  return p * u2f((uint32_t)(ki + 127) << 23);
}
VT_HD float vpow(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (!(x > 0.0f)) return 0.0f;
  if (x == 1.0f) return 1.0f;
  if (y == 5.0f) {                 // Schlick's fifth power: three correctly rounded products
    const float x2 = x * x;
    return (x2 * x2) * x;
  }
  return vexp2(y * vlog2(x));
}

// ---- atan / atan2 / acos ---------------------------------------------------
// atan(t) for t in [0, 1].
VT_HD float atan01(float t) {
  float base = 0.0f;
  if (t > 0.267949192431122706f) {                              // tan(pi/12)
    t = (t * 1.73205080756887729f - 1.0f) / (1.73205080756887729f + t);
    base = 0.523598775598298873f;                               // pi/6
  }
  const float t2 = t * t;
  float p = -1.0f / 15.0f;
  p = vfma(p, t2, 1.0f / 13.0f);
  p = vfma(p, t2, -1.0f / 11.0f);
  p = vfma(p, t2, 1.0f / 9.0f);
  p = vfma(p, t2, -1.0f / 7.0f);
  p = vfma(p, t2, 1.0f / 5.0f);
  p = vfma(p, t2, -1.0f / 3.0f);
  return base + vfma(p * t2, t, t);
}
VT_HD float vatan2(float y, float x) {
  const float ax = vabs(x), ay = vabs(y);
  const float mx = ax < ay ? ay : ax;
  const float mn = ax < ay ? ax : ay;
  if (mx == 0.0f) return 0.0f;
  float a = atan01(mn / mx);
  if (ay > ax) a = 1.57079632679489662f - a;
  if (x < 0.0f) a = 3.14159265358979324f - a;
  if (y < 0.0f) a = -a;
  return a;
}
VT_HD float vacos(float x) {
  x = x < -1.0f ? -1.0f : (x > 1.0f ? 1.0f : x);
  return vatan2(vsqrt((1.0f - x) * (1.0f + x)), x);
}

// ---- IEEE binary16 <-> binary32 ------------------------------------------------
// Round-to-nearest-even conversion, exact on both host and device.
VT_HD uint16_t f2h(float f) {
  const uint32_t u = f2u(f);
  const uint32_t sign = (u >> 16) & 0x8000u;
  const uint32_t au = u & 0x7fffffffu;
  if (au >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (au > 0x7f800000u ? 0x200u : 0u));
  if (au >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);          // overflow -> inf
  if (au < 0x38800000u) {                                            // subnormal half
    if (au < 0x33000000u) return (uint16_t)sign;                     // < 2^-25 -> 0
    const uint32_t mant = (au & 0x007fffffu) | 0x00800000u;
    const int shift = 126 - (int)(au >> 23);                          // 14..24
    const uint32_t keep = mant >> shift;
    const uint32_t rem = mant & ((1u << shift) - 1u);
    const uint32_t half = 1u << (shift - 1);
    uint32_t r = keep;
    if (rem > half || (rem == half && (keep & 1u))) r += 1u;
    return (uint16_t)(sign | r);
  }
  uint32_t r = ((au >> 13) - (112u << 10));
  const uint32_t rem = au & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r += 1u;
  return (uint16_t)(sign | r);
}
// Clamp to the finite half range before conversion (environment texels).
VT_HD float clamp_half(float x) { return x > 65504.0f ? 65504.0f : (x < -65504.0f ? -65504.0f : x); }
VT_HD float h2f(uint16_t h) {
  const uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  const uint32_t e = ((uint32_t)h >> 10) & 0x1fu;
  const uint32_t m = (uint32_t)h & 0x3ffu;
  if (e == 0) {
    if (m == 0) return u2f(sign);
    // subnormal: m * 2^-24
    const float v = (float)m * 5.9604644775390625e-8f;
    return sign ? -v : v;
  }
  if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
  return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

}  // namespace vtb
