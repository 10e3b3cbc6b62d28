// Project-written single-precision sin, cos, atan, atan2, exp, exp2, log2 and
// pow for host and device code.
//
// The wind-tunnel shaders call sin/cos/atan inside the signed-distance field
// (src/engine/f1.ts:37-46 rake transform, src/engine/wgsl.ts:65-74 wing
// elements).  WGSL leaves the accuracy of these builtins to the
// implementation, and solid flags flip on a one-ulp change for cells that sit
// on the 0.3*h inside threshold (src/engine/wgsl.ts:314).  So the device
// voxelizer and every CPU model of it must evaluate the very same function,
// bit for bit.  These definitions are that function.
//
// Method (textbook, no library code):
//   sin/cos: Cody-Waite reduction of x by pi/2 with a three-part split of
//            pi/2 (C1 has 8 significant bits, C2 10 bits, so k*C1 and k*C2 are
//            exact for |k| < 2^14), then the Taylor series of sin (to r^11)
//            and cos (to r^12) on |r| <= pi/4, evaluated by Horner's rule.
//            Truncation error is below 1e-11, far under float rounding.
//   atan:    atan(x) = pi/2 - atan(1/x) for |x| > 1, then
//            atan(t) = pi/4 + atan((t-1)/(t+1)) for t > tan(pi/8), then the
//            Gregory series t - t^3/3 + t^5/5 - ... to t^23 on |t| <= 0.4143.
// Coefficients are 1/n! and 1/n rounded to float.  Every operation is a
// single IEEE float add, multiply or divide; callers must compile without
// floating-point contraction (-ffp-contract=off for g++, -fmad=false for nvcc)
// so that host and device results agree bit for bit.
// Valid for |x| < 2^14 * pi/2 (sin/cos); accuracy measured against double
// libm is a few ulp over the angles the scene uses.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define WT_HD __host__ __device__ __forceinline__
#else
#define WT_HD static inline
#endif

namespace wtm {

// pi/2 = C1 + C2 + C3
#define WTM_C1 0x1.92p+0f
#define WTM_C2 0x1.fb4p-12f
#define WTM_C3 0x1.4442d2p-24f
#define WTM_2_OVER_PI 0x1.45f306p-1f

WT_HD float rint_even(float x) {
#if defined(__CUDA_ARCH__)
  return rintf(x);
#else
  return __builtin_rintf(x);  // default rounding mode: nearest, ties to even
#endif
}

// Reduced argument r in [-pi/4, pi/4] and quadrant q (0..3).
WT_HD float reduce_pio2(float x, int* q) {
  float k = rint_even(x * WTM_2_OVER_PI);
  float r = x - k * WTM_C1;
  r = r - k * WTM_C2;
  r = r - k * WTM_C3;
  int ki = (k == k && k < 1e9f && k > -1e9f) ? (int)k : 0;
  *q = ki & 3;
  return r;
}

WT_HD float sin_poly(float r) {
  float z = r * r;
  float p = -0x1.ae6456p-26f;         // -1/11!
  p = p * z + 0x1.71de3ap-19f;        //  1/9!
  p = p * z + -0x1.a01a02p-13f;       // -1/7!
  p = p * z + 0x1.111112p-7f;         //  1/5!
  p = p * z + -0x1.555556p-3f;        // -1/3!
  return r + (r * z) * p;
}

WT_HD float cos_poly(float r) {
  float z = r * r;
  float p = 0x1.1eed8ep-29f;          //  1/12!
  p = p * z + -0x1.27e4fcp-22f;       // -1/10!
  p = p * z + 0x1.a01a02p-16f;        //  1/8!
  p = p * z + -0x1.6c16c2p-10f;       // -1/6!
  p = p * z + 0x1.555556p-5f;         //  1/4!
  return (1.0f - 0.5f * z) + (z * z) * p;
}

WT_HD float sinf(float x) {
  int q;
  float r = reduce_pio2(x, &q);
  float v = (q & 1) ? cos_poly(r) : sin_poly(r);
  return (q & 2) ? -v : v;
}

WT_HD float cosf(float x) {
  int q;
  float r = reduce_pio2(x, &q);
  float v = (q & 1) ? sin_poly(r) : cos_poly(r);
  return ((q + 1) & 2) ? -v : v;
}

WT_HD float atan_poly(float t) {
  float z = t * t;
  float p = -0x1.642c86p-5f;          // -1/23
  p = p * z + 0x1.861862p-5f;         //  1/21
  p = p * z + -0x1.af286cp-5f;        // -1/19
  p = p * z + 0x1.e1e1e2p-5f;         //  1/17
  p = p * z + -0x1.111112p-4f;        // -1/15
  p = p * z + 0x1.3b13b2p-4f;         //  1/13
  p = p * z + -0x1.745d18p-4f;        // -1/11
  p = p * z + 0x1.c71c72p-4f;         //  1/9
  p = p * z + -0x1.24924ap-3f;        // -1/7
  p = p * z + 0x1.99999ap-3f;         //  1/5
  p = p * z + -0x1.555556p-2f;        // -1/3
  return t + (t * z) * p;
}

WT_HD float atanf(float x) {
  float ax = x < 0.0f ? -x : x;
  bool inv = ax > 1.0f;
  float t = inv ? 1.0f / ax : ax;
  bool hi = t > 0x1.a8279ap-2f;       // tan(pi/8)
  float u = hi ? (t - 1.0f) / (t + 1.0f) : t;
  float r = atan_poly(u);
  if (hi) r = 0x1.921fb6p-1f + r;     // pi/4
  if (inv) r = 0x1.921fb6p+0f - r;    // pi/2
  return x < 0.0f ? -r : r;
}

// atan2 by quadrant: atan(y/x) for x > 0, shifted by +-pi for x < 0, +-pi/2 on
// the y axis; 0 at the origin (WGSL leaves atan2(0, 0) undefined).
WT_HD float atan2f(float y, float x) {
  if (x != x || y != y) return x + y;
  if (x == 0.0f) return y > 0.0f ? 0x1.921fb6p+0f : (y < 0.0f ? -0x1.921fb6p+0f : 0.0f);
  const float t = atanf(y / x);
  if (x > 0.0f) return t;
  return y < 0.0f ? t - 0x1.921fb6p+1f : t + 0x1.921fb6p+1f;
}

// ---- exponentials and logarithms (used by the renderer's shading) ---------
// Method (textbook, no library code):
//   exp2:  x = n + f with n = rint(x), |f| <= 1/2 (exact), 2^f = e^(f ln 2)
//          by its Taylor series in f to degree 7 (coefficients ln2^k/k!;
//          truncation below 6e-9 relative), scaled by 2^n in two exact steps.
//   exp:   Cody-Waite: n = rint(x log2 e), r = x - n*L1 - n*L2 with
//          L1 = ln 2 to 15 bits (n*L1 exact for |n| < 2^9), |r| <= 0.347;
//          e^r by Taylor to degree 7, scaled by 2^n.
//   log2:  x = m 2^e with m in [sqrt(1/2), sqrt(2)]; ln m = 2 atanh(s),
//          s = (m-1)/(m+1), |s| <= 0.172, series s + s^3/3 + ... + s^11/11;
//          log2 x = e + ln(m) log2(e).
//   pow:   exp2(y log2 x), the definition WGSL gives for pow.
// Accuracy against double libm is a few ulp; inputs outside the float range
// saturate to 0 / inf, NaN propagates.  As above, every operation is a single
// IEEE add, multiply or divide, so host and device agree bit for bit.
WT_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  __builtin_memcpy(&u, &x, 4);
  return u;
#endif
}
WT_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  __builtin_memcpy(&x, &u, 4);
  return x;
#endif
}
// r * 2^n for |n| <= 170: two exact power-of-two factors, one final rounding.
WT_HD float scale2(float r, int n) {
  const int n1 = n / 2, n2 = n - n1;
  return (r * u2f((uint32_t)(n1 + 127) << 23)) * u2f((uint32_t)(n2 + 127) << 23);
}

WT_HD float exp2f(float x) {
  if (x != x) return x;
  if (x >= 129.0f) return u2f(0x7f800000u);
  if (x <= -151.0f) return 0.0f;
  const float n = rint_even(x);
  const float f = x - n;
  float p = 0x1.ffcbfcp-17f;
  p = p * f + 0x1.430912p-13f;
  p = p * f + 0x1.5d87fep-10f;
  p = p * f + 0x1.3b2ab6p-7f;
  p = p * f + 0x1.c6b08ep-5f;
  p = p * f + 0x1.ebfbe0p-3f;
  p = p * f + 0x1.62e430p-1f;
  return scale2(1.0f + f * p, (int)n);
}

WT_HD float expf(float x) {
  if (x != x) return x;
  if (x >= 89.0f) return u2f(0x7f800000u);
  if (x <= -104.0f) return 0.0f;
  const float n = rint_even(x * 0x1.715476p+0f);
  float r = x - n * 0x1.62e4p-1f;
  r = r - n * 0x1.7f7d1cp-20f;
  float p = 0x1.a01a02p-13f;          // 1/7!
  p = p * r + 0x1.6c16c2p-10f;        // 1/6!
  p = p * r + 0x1.111112p-7f;         // 1/5!
  p = p * r + 0x1.555556p-5f;         // 1/4!
  p = p * r + 0x1.555556p-3f;         // 1/3!
  p = p * r + 0.5f;                   // 1/2!
  p = p * r + 1.0f;
  return scale2(1.0f + r * p, (int)n);
}

WT_HD float log2f(float x) {
  if (x != x || x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return u2f(0xff800000u);
  uint32_t u = f2u(x);
  if (u == 0x7f800000u) return x;
  int e = 0;
  if (u < 0x00800000u) {              // subnormal: scale into the normal range
    u = f2u(x * 8388608.0f);
    e = -23;
  }
  e += (int)((u >> 23) & 0xffu) - 127;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u);
  if (m > 0x1.6a09e6p+0f) {           // sqrt(2)
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float p = 0x1.745d18p-4f;           // 1/11
  p = p * z + 0x1.c71c72p-4f;         // 1/9
  p = p * z + 0x1.24924ap-3f;         // 1/7
  p = p * z + 0x1.99999ap-3f;         // 1/5
  p = p * z + 0x1.555556p-2f;         // 1/3
  const float lnm = (s + s * (z * p)) * 2.0f;
  return (float)e + lnm * 0x1.715476p+0f;
}

WT_HD float powf(float x, float y) { return exp2f(y * log2f(x)); }

}  // namespace wtm
