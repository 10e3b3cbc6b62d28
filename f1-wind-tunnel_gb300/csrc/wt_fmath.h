// Project-written single-precision sin, cos and atan for host and device code.
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

}  // namespace wtm
