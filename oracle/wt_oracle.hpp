// TEST INFRASTRUCTURE ONLY - the oracle.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load it, and only as the checker or the
// timed CPU baseline; the product library never links it.
//
// A plain C++ restatement of the reference's simulation shaders:
//   lattice tables + feq        src/engine/wgsl.ts:123-139
//   LBM_INIT                    src/engine/wgsl.ts:141-155
//   LBM_STEP (stepCell, force)  src/engine/wgsl.ts:176-291
//   VOXELIZE                    src/engine/wgsl.ts:305-321
//   scene SDFs                  src/engine/wgsl.ts:20-76,101-116; src/engine/f1.ts:20-320,397-407
//   HEAT                        src/engine/wgsl.ts:469-510
//   engine dispatch order       src/engine/engine.ts:371-381,469,708-712,739-761
//
// The lattice is templated on the arithmetic type: float reproduces the
// reference's f32 arithmetic operation for operation (bit-exact against the
// translated reference shaders in oracle/_ref), double is the FP64 model used
// to judge low-precision storage.  Voxelization is always float (it defines the
// geometry).  Build with -ffp-contract=off.
//
// Parity pin: oracle/_ref builds the reference's own WGSL text as C++ and the
// tests compare this restatement against it bit for bit; tests/golden holds
// outputs of that build so the pin travels without the reference checkout.
#pragma once
#include <stdint.h>
#include <string.h>
#include <vector>
#include "../f1-wind-tunnel_gb300/csrc/wt_fmath.h"

namespace wto {

// ------------------------------------------------------------ WGSL builtins
// Definitions from the WGSL specification (min/max/clamp/mix/smoothstep/length).
static inline float fmin_w(float a, float b) { return b < a ? b : a; }
static inline float fmax_w(float a, float b) { return a < b ? b : a; }
static inline float fabs_w(float x) { return x < 0.0f ? -x : (x == 0.0f ? 0.0f : x); }
static inline float fclamp_w(float e, float lo, float hi) { return fmin_w(fmax_w(e, lo), hi); }
static inline float fmix_w(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline float fsmooth_w(float lo, float hi, float x) {
  float t = fclamp_w((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
static inline float fsqrt_w(float x) { return __builtin_sqrtf(x); }
static inline int32_t f2i_w(float x) {  // truncate toward zero, saturate, NaN -> 0
  if (!(x == x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)x;
}
static inline uint32_t f2u_w(float x) {
  if (!(x == x) || x <= 0.0f) return 0u;
  if (x >= 4294967296.0f) return 4294967295u;
  return (uint32_t)x;
}

struct F2 { float x, y; };
struct F3 { float x, y, z; };
static inline F2 f2(float x, float y) { F2 r = {x, y}; return r; }
static inline F3 f3(float x, float y, float z) { F3 r = {x, y, z}; return r; }
static inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline F2 sub(F2 a, F2 b) { return f2(a.x - b.x, a.y - b.y); }
static inline F2 add(F2 a, F2 b) { return f2(a.x + b.x, a.y + b.y); }
static inline F3 mul(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
static inline F2 mul(F2 a, float s) { return f2(a.x * s, a.y * s); }
static inline float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot2(F2 a, F2 b) { return a.x * b.x + a.y * b.y; }
static inline float len3(F3 a) { return fsqrt_w(dot3(a, a)); }
static inline float len2(F2 a) { return fsqrt_w(dot2(a, a)); }
static inline F3 abs3(F3 a) { return f3(fabs_w(a.x), fabs_w(a.y), fabs_w(a.z)); }
static inline F2 abs2(F2 a) { return f2(fabs_w(a.x), fabs_w(a.y)); }
static inline F3 max3s(F3 a, float s) { return f3(fmax_w(a.x, s), fmax_w(a.y, s), fmax_w(a.z, s)); }
static inline F2 max2s(F2 a, float s) { return f2(fmax_w(a.x, s), fmax_w(a.y, s)); }
static inline F2 mix2(F2 a, F2 b, float t) { return f2(fmix_w(a.x, b.x, t), fmix_w(a.y, b.y, t)); }

// ------------------------------------------------------------ Shape uniform
// Field order and meaning of the Shape uniform, src/engine/wgsl.ts:9-18, plus the
// build's axis-aligned box scene (kind 7), which has no reference counterpart.
struct Shape {
  uint32_t kind, profileMode, pw, ph;
  float frontFlap, rearMain, rearFlap, rideH;
  float aoa, width, axisY, pScale;
  float pOrigin[2], heatBrakes, heatEngine;
  float heatRad, frontWing, rearWing, sidepod;
  float cover, nose, rearRide, duct;
  float boxCenter[3], boxHalf[3];
};

// ------------------------------------------------------------ SDF primitives (wgsl.ts:20-76)
struct Sdf {
  const Shape& sh;
  explicit Sdf(const Shape& s) : sh(s) {}

  static float box(F3 p, F3 b) {
    F3 q = sub(abs3(p), b);
    return len3(max3s(q, 0.0f)) + fmin_w(fmax_w(q.x, fmax_w(q.y, q.z)), 0.0f);
  }
  static float round_box(F3 p, F3 b, float r) { return box(p, sub(b, f3(r, r, r))) - r; }
  static float capsule(F3 p, F3 a, F3 b, float r) {
    F3 pa = sub(p, a), ba = sub(b, a);
    float hh = fclamp_w(dot3(pa, ba) / dot3(ba, ba), 0.0f, 1.0f);
    return len3(sub(pa, mul(ba, hh))) - r;
  }
  static float round_rect(F2 p, F2 b, float r) {
    F2 q = add(sub(abs2(p), b), f2(r, r));
    return len2(max2s(q, 0.0f)) + fmin_w(fmax_w(q.x, q.y), 0.0f) - r;
  }
  static float extrude(float d2, float dz) {
    F2 w = f2(d2, dz);
    return fmin_w(fmax_w(w.x, w.y), 0.0f) + len2(max2s(w, 0.0f));
  }
  static float taper(F3 p, float x0, float x1, F2 c0, F2 c1, F2 s0, F2 s1, float r0, float r1) {
    float t = fclamp_w((p.x - x0) / (x1 - x0), 0.0f, 1.0f);
    F2 c = mix2(c0, c1, t);
    F2 s = mix2(s0, s1, t);
    float r = fmin_w(fmix_w(r0, r1, t), fmin_w(s.x, s.y));
    float d2 = round_rect(sub(f2(p.y, p.z), c), s, r);
    float dx = fabs_w(p.x - 0.5f * (x0 + x1)) - 0.5f * (x1 - x0);
    return extrude(d2, dx) * 0.8f;
  }
  static float uneven_capsule(F2 p0, float r1, float r2, float hh) {
    F2 p = f2(fabs_w(p0.x), p0.y);
    float b = (r1 - r2) / hh;
    float a = fsqrt_w(fmax_w(1.0f - b * b, 0.0f));
    float k = dot2(p, f2(-b, a));
    if (k < 0.0f) return len2(p) - r1;
    if (k > a * hh) return len2(sub(p, f2(0.0f, hh))) - r2;
    return dot2(p, f2(a, b)) - r1;
  }
  static float wing(F3 p, F2 le, float chord, float ang, float thick, float z0, float z1) {
    F2 q = sub(f2(p.x, p.y), le);
    float c = wtm::cosf(ang), s = wtm::sinf(ang);
    float lx = q.x * c + q.y * s;
    float ly = -q.x * s + q.y * c;
    float r1 = thick * 0.5f;
    float r2 = fmax_w(thick * 0.12f, 0.006f);
    float d2 = uneven_capsule(f2(ly, lx - r1), r1, r2, fmax_w(chord - r1 - r2, 0.01f));
    return extrude(d2, fabs_w(p.z - 0.5f * (z0 + z1)) - 0.5f * (z1 - z0));
  }
  static F2 op_u(F2 a, F2 b) { return (b.x < a.x) ? b : a; }

  // ---------------------------------------------------------- generic F1 (f1.ts:20-320)
  static constexpr float DEG = 0.017453292f, FA = 1.0f, RA = 4.6f, WR = 0.36f, FWZ = 0.84f,
                         FHW = 0.152f, RWZ = 0.80f, RHW = 0.20f, RA26 = 4.4f, WR26 = 0.355f,
                         FHW26 = 0.14f, RHW26 = 0.1875f, BODY_X = 0.9444444f, BODY_Z = 0.96f,
                         BODY_LIP = 0.96f;

  float rake() const { return wtm::atanf((sh.rearRide - sh.rideH) / (RA26 - FA)); }
  F3 body_frame(F3 pw) const {
    float th = rake();
    float c = wtm::cosf(th), s = wtm::sinf(th);
    float dx = pw.x - FA, dy = pw.y - sh.rideH;
    F3 p = f3(FA + dx * c + dy * s, sh.rideH - dx * s + dy * c, pw.z);
    float x = p.x;
    if (x > FA) {
      float a = FA + (x - FA) / BODY_X;
      float b = x + (RA - RA26);
      x = (x > RA26) ? b : a;
    }
    return f3(x, p.y, p.z / BODY_Z);
  }
  static float smin(float a, float b, float k) {
    float h = fmax_w(k - fabs_w(a - b), 0.0f) / k;
    return fmin_w(a, b) - h * h * k * 0.25f;
  }
  static float smax(float a, float b, float k) { return -smin(-a, -b, k); }
  static float ellipsoid(F3 p, F3 r) {
    float k0 = len3(f3(p.x / r.x, p.y / r.y, p.z / r.z));
    F3 rr = f3(r.x * r.x, r.y * r.y, r.z * r.z);
    float k1 = len3(f3(p.x / rr.x, p.y / rr.y, p.z / rr.z));
    return k0 * (k0 - 1.0f) / fmax_w(k1, 1e-5f);
  }
  static float cyl_z(F3 p, float r, float hz) {
    F2 d = f2(len2(f2(p.x, p.y)) - r, fabs_w(p.z) - hz);
    return fmin_w(fmax_w(d.x, d.y), 0.0f) + len2(max2s(d, 0.0f));
  }
  static float wing_z(F3 p, F2 le, float chord, float ang, float thick, float z0, float z1, float rise,
                      float taper_, float curl) {
    float s = fsmooth_w(curl, z1, p.z);
    return wing(p, add(le, f2(0.0f, rise * s)), chord * (1.0f - taper_ * s), ang + rise * s * 0.6f, thick,
                z0, z1) * 0.85f;
  }
  static float tunnel_roof(float x, float b) {
    if (x < 2.5f) return fmix_w(b + 0.12f, b + 0.05f, fsmooth_w(1.55f, 2.5f, x));
    if (x < 3.8f) return b + 0.05f;
    return fmix_w(b + 0.05f, b + 0.25f, fsmooth_w(3.8f, 4.98f, x));
  }
  static float floor_(F3 p, float b) {
    float roof = tunnel_roof(p.x, b);
    float zlim = fmix_w(0.80f, 0.58f, fsmooth_w(3.6f, 4.15f, p.x));
    float top = (fabs_w(p.z - 0.40f) < 0.28f) ? roof + 0.03f : b + 0.05f;
    float slab = fmax_w(fmax_w(b - p.y, p.y - top), fmax_w(fabs_w(p.x - 3.265f) - 1.715f, p.z - zlim));
    float tunnel = fmax_w(p.y - roof, fabs_w(p.z - 0.40f) - 0.255f);
    float d = fmax_w(slab, -tunnel) * 0.8f;
    for (int i = 0; i < 2; i++) {
      float fz = 0.26f + (float)i * 0.16f;
      float fence = box(sub(p, f3(1.84f, b + 0.08f, fz)), f3(0.28f, 0.08f, 0.012f));
      d = fmin_w(d, fmax_w(fence, p.y - roof - 0.02f));
    }
    for (int i = 0; i < 2; i++) {
      float sz = 0.30f + (float)i * 0.20f;
      float strake = box(sub(p, f3(4.62f, b + 0.17f, sz)), f3(0.34f, 0.17f, 0.008f));
      d = fmin_w(d, fmax_w(strake, p.y - roof));
    }
    d = fmin_w(d, capsule(p, f3(2.25f, b + 0.065f, 0.79f), f3(3.85f, b + 0.05f, 0.78f), 0.02f));
    return d;
  }
  static float tyre(F3 p, F3 c, float hw) {
    F3 q = sub(p, c);
    return round_rect(f2(len2(f2(q.x, q.y)) - 0.2925f, q.z), f2(0.0625f, hw), 0.06f);
  }
  static float wheel_cover(F3 p, F3 c, float hw) {
    F3 q = sub(p, c);
    float d = cyl_z(q, 0.234f, hw - 0.028f);
    d = fmin_w(d, cyl_z(sub(q, f3(0.0f, 0.0f, hw - 0.02f)), 0.045f, 0.02f));
    return d;
  }
  static F2 wheel_set(F3 p, F2 res, F3 c, float hw, float inboard) {
    if (box(sub(p, c), f3(WR26 + 0.02f, WR26 + 0.02f, hw + 0.2f)) > res.x) return res;
    res = op_u(res, f2(tyre(p, c, hw), 2.0f));
    res = op_u(res, f2(wheel_cover(p, c, hw), 9.0f));
    float duct = cyl_z(sub(p, f3(c.x, c.y, c.z - hw - inboard * 0.5f)), 0.17f, inboard * 0.5f);
    float duct_wing = round_box(sub(p, f3(c.x - 0.04f, c.y + 0.21f, c.z - hw - 0.05f)),
                                f3(0.16f, 0.012f, 0.05f), 0.006f);
    res = op_u(res, f2(fmin_w(duct, duct_wing), 10.0f));
    return res;
  }
  static float suspension(F3 p, float b) {
    const float fz = FWZ - FHW - 0.05f, rz = RWZ - RHW - 0.05f;
    float d = capsule(p, f3(1.10f, b + 0.43f, 0.17f), f3(FA + 0.02f, WR + 0.16f, fz), 0.017f);
    d = fmin_w(d, capsule(p, f3(1.42f, b + 0.40f, 0.17f), f3(FA + 0.02f, WR + 0.16f, fz), 0.017f));
    d = fmin_w(d, capsule(p, f3(0.98f, b + 0.19f, 0.15f), f3(FA, WR - 0.13f, fz), 0.017f));
    d = fmin_w(d, capsule(p, f3(1.38f, b + 0.17f, 0.15f), f3(FA, WR - 0.13f, fz), 0.017f));
    d = fmin_w(d, capsule(p, f3(FA + 0.03f, WR - 0.10f, FWZ - FHW - 0.07f), f3(1.20f, b + 0.47f, 0.16f), 0.014f));
    d = fmin_w(d, capsule(p, f3(0.86f, b + 0.29f, 0.16f), f3(0.88f, WR + 0.02f, fz), 0.013f));
    d = fmin_w(d, capsule(p, f3(4.30f, b + 0.42f, 0.20f), f3(RA, WR + 0.17f, rz), 0.017f));
    d = fmin_w(d, capsule(p, f3(4.78f, b + 0.40f, 0.16f), f3(RA, WR + 0.17f, rz), 0.017f));
    d = fmin_w(d, capsule(p, f3(4.28f, b + 0.16f, 0.24f), f3(RA, WR - 0.14f, rz), 0.017f));
    d = fmin_w(d, capsule(p, f3(4.82f, b + 0.15f, 0.18f), f3(RA, WR - 0.14f, rz), 0.017f));
    d = fmin_w(d, capsule(p, f3(RA - 0.03f, WR + 0.14f, RWZ - RHW - 0.07f), f3(4.40f, b + 0.18f, 0.22f), 0.014f));
    return d;
  }
  uint32_t variant(float v) const { return f2u_w(v + 0.5f); }
  float nose_tip_y(float b) const { return b + ((variant(sh.nose) == 2u) ? 0.25f : 0.17f); }
  float nose_start_x() const { return (variant(sh.nose) == 1u) ? 0.34f : 0.10f; }
  float nose(F3 p, float b) const {
    uint32_t v = variant(sh.nose);
    float x0 = nose_start_x(), y0 = nose_tip_y(b);
    F2 s0 = f2(0.055f, 0.11f);
    if (v == 1u) s0 = f2(0.075f, 0.15f);
    if (v == 2u) s0 = f2(0.045f, 0.075f);
    float d = taper(p, x0, 1.26f, f2(y0, 0.0f), f2(b + 0.36f, 0.0f), s0, f2(0.15f, 0.17f), 0.04f, 0.12f);
    d = smin(d, ellipsoid(sub(p, f3(x0 + 0.02f, y0, 0.0f)), f3(0.09f, s0.x, s0.y)), 0.04f);
    if (v != 0u) {
      float yw = 0.19f + b * 0.45f;
      float pylon = round_box(sub(p, f3(x0 + 0.06f, 0.5f * (yw + y0), 0.09f)),
                              f3(0.09f, 0.5f * (y0 - yw) + 0.02f, 0.006f), 0.004f);
      d = fmin_w(d, pylon);
    }
    return d;
  }
  float engine_cover(F3 p, float b) const {
    uint32_t v = variant(sh.cover);
    if (v == 1u)
      return taper(p, 2.96f, 4.86f, f2(b + 0.60f, 0.0f), f2(b + 0.40f, 0.0f), f2(0.32f, 0.31f), f2(0.12f, 0.13f), 0.15f, 0.08f);
    if (v == 2u)
      return taper(p, 2.96f, 4.70f, f2(b + 0.57f, 0.0f), f2(b + 0.34f, 0.0f), f2(0.29f, 0.19f), f2(0.06f, 0.05f), 0.12f, 0.04f);
    return taper(p, 2.96f, 4.86f, f2(b + 0.58f, 0.0f), f2(b + 0.36f, 0.0f), f2(0.30f, 0.24f), f2(0.08f, 0.07f), 0.14f, 0.06f);
  }
  float sidepods(F3 p, float b) const {
    uint32_t v = variant(sh.sidepod);
    float pod;
    if (v == 1u) {
      pod = taper(p, 2.30f, 4.05f, f2(b + 0.40f, 0.36f), f2(b + 0.24f, 0.24f), f2(0.16f, 0.08f), f2(0.07f, 0.05f), 0.06f, 0.04f);
      pod = smax(pod, -round_box(sub(p, f3(2.27f, b + 0.42f, 0.38f)), f3(0.06f, 0.12f, 0.05f), 0.03f), 0.02f);
      return pod;
    }
    if (v == 2u) {
      pod = taper(p, 2.30f, 4.25f, f2(b + 0.41f, 0.52f), f2(b + 0.24f, 0.30f), f2(0.18f, 0.28f), f2(0.08f, 0.11f), 0.10f, 0.05f);
      pod = smax(pod, -capsule(p, f3(2.30f, b + 0.13f, 0.84f), f3(3.70f, b + 0.08f, 0.58f), 0.15f), 0.05f);
      pod = smax(pod, -capsule(p, f3(2.55f, b + 0.66f, 0.52f), f3(4.00f, b + 0.40f, 0.36f), 0.11f), 0.04f);
      pod = smax(pod, -round_box(sub(p, f3(2.28f, b + 0.47f, 0.57f)), f3(0.06f, 0.10f, 0.17f), 0.05f), 0.02f);
      return pod;
    }
    if (v == 3u) {
      pod = taper(p, 2.30f, 4.25f, f2(b + 0.47f, 0.52f), f2(b + 0.26f, 0.28f), f2(0.15f, 0.25f), f2(0.07f, 0.10f), 0.12f, 0.05f);
      pod = smax(pod, -capsule(p, f3(2.25f, b + 0.17f, 0.86f), f3(3.70f, b + 0.10f, 0.56f), 0.22f), 0.05f);
      pod = smax(pod, -round_box(sub(p, f3(2.28f, b + 0.52f, 0.55f)), f3(0.06f, 0.07f, 0.17f), 0.04f), 0.02f);
      return pod;
    }
    pod = taper(p, 2.30f, 4.25f, f2(b + 0.41f, 0.52f), f2(b + 0.22f, 0.28f), f2(0.18f, 0.25f), f2(0.07f, 0.10f), 0.12f, 0.05f);
    pod = smax(pod, -capsule(p, f3(2.30f, b + 0.13f, 0.82f), f3(3.70f, b + 0.08f, 0.56f), 0.16f), 0.05f);
    pod = smax(pod, -round_box(sub(p, f3(2.28f, b + 0.47f, 0.57f)), f3(0.06f, 0.10f, 0.17f), 0.05f), 0.02f);
    return pod;
  }
  float bodywork(F3 p, float b) const {
    float d = nose(p, b);
    d = smin(d, taper(p, 1.20f, 2.24f, f2(b + 0.36f, 0.0f), f2(b + 0.42f, 0.0f), f2(0.15f, 0.17f), f2(0.25f, 0.29f), 0.12f, 0.16f), 0.08f);
    d = smin(d, taper(p, 2.20f, 3.06f, f2(b + 0.42f, 0.0f), f2(b + 0.42f, 0.0f), f2(0.25f, 0.30f), f2(0.25f, 0.34f), 0.16f, 0.16f), 0.06f);
    d = smin(d, engine_cover(p, b), 0.10f);
    float keel = taper(p, 1.30f, 4.70f, f2(b + 0.22f, 0.0f), f2(b + 0.20f, 0.0f), f2(0.19f, 0.19f), f2(0.17f, 0.14f), 0.06f, 0.05f);
    d = smin(d, keel, 0.08f);
    d = smin(d, sidepods(p, b), 0.12f);
    float airbox = round_box(sub(p, f3(3.02f, b + 0.84f, 0.0f)), f3(0.17f, 0.11f, 0.12f), 0.08f);
    airbox = smax(airbox, -ellipsoid(sub(p, f3(2.85f, b + 0.86f, 0.0f)), f3(0.09f, 0.066f, 0.078f)), 0.015f);
    d = smin(d, airbox, 0.10f);
    d = smax(d, -round_box(sub(p, f3(2.62f, b + 0.72f, 0.0f)), f3(0.42f, 0.13f, 0.215f), 0.10f), 0.03f);
    return d;
  }
  static float halo(F3 p, float b) {
    float d = capsule(p, f3(2.17f, b + 0.62f, 0.0f), f3(2.36f, b + 0.90f, 0.0f), 0.034f);
    d = smin(d, capsule(p, f3(2.36f, b + 0.90f, 0.0f), f3(2.52f, b + 0.92f, 0.20f), 0.031f), 0.03f);
    d = smin(d, capsule(p, f3(2.52f, b + 0.92f, 0.20f), f3(2.82f, b + 0.88f, 0.26f), 0.031f), 0.03f);
    d = smin(d, capsule(p, f3(2.82f, b + 0.88f, 0.26f), f3(3.02f, b + 0.74f, 0.25f), 0.033f), 0.03f);
    return d;
  }
  float front_wing(F3 p, float yw) const {
    const float ff = sh.frontFlap;
    uint32_t v = variant(sh.frontWing);
    float d, ep;
    if (v == 1u) {
      d = wing_z(p, f2(-0.03f, yw), 0.31f, 2.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, 0.03f, 0.2f, 0.5f);
      d = fmin_w(d, wing_z(p, f2(0.21f, yw + 0.036f), 0.17f, 9.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, 0.15f, 0.35f, 0.3f));
      d = fmin_w(d, wing_z(p, f2(0.335f, yw + 0.075f + ff * 0.03f), 0.14f, 17.0f * DEG + ff * 0.75f, 0.020f, 0.10f, 0.94f, 0.19f, 0.35f, 0.25f));
      d = fmin_w(d, wing_z(p, f2(0.425f, yw + 0.118f + ff * 0.07f), 0.12f, 26.0f * DEG + ff, 0.018f, 0.12f, 0.94f, 0.22f, 0.4f, 0.25f));
      ep = round_rect(f2(p.x - 0.25f, p.y - (yw + 0.17f)), f2(0.29f, 0.20f), 0.08f);
    } else if (v == 2u) {
      d = wing_z(p, f2(-0.03f, yw), 0.31f, 3.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, -0.02f, 0.15f, 0.55f);
      d = fmin_w(d, wing_z(p, f2(0.21f, yw + 0.04f), 0.19f, 13.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, -0.04f, 0.35f, 0.35f));
      d = fmin_w(d, wing_z(p, f2(0.35f, yw + 0.085f + ff * 0.03f), 0.16f, 22.0f * DEG + ff * 0.75f, 0.020f, 0.06f, 0.94f, -0.06f, 0.4f, 0.35f));
      d = fmin_w(d, wing_z(p, f2(0.45f, yw + 0.13f + ff * 0.07f), 0.13f, 31.0f * DEG + ff, 0.018f, 0.08f, 0.94f, -0.08f, 0.45f, 0.35f));
      ep = round_rect(f2(p.x - 0.25f, p.y - (yw + 0.06f)), f2(0.29f, 0.10f), 0.06f);
    } else if (v == 3u) {
      d = wing_z(p, f2(-0.03f, yw), 0.30f, 1.0f * DEG + ff * 0.05f, 0.030f, 0.0f, 0.94f, 0.0f, 0.1f, 0.6f);
      d = fmin_w(d, wing_z(p, f2(0.20f, yw + 0.03f), 0.16f, 4.0f * DEG + ff * 0.3f, 0.022f, 0.0f, 0.94f, 0.02f, 0.2f, 0.5f));
      ep = round_rect(f2(p.x - 0.22f, p.y - (yw + 0.05f)), f2(0.26f, 0.085f), 0.05f);
    } else {
      d = wing_z(p, f2(-0.03f, yw), 0.31f, 2.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, 0.06f, 0.2f, 0.5f);
      d = fmin_w(d, wing_z(p, f2(0.21f, yw + 0.036f), 0.17f, 9.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, 0.09f, 0.25f, 0.45f));
      d = fmin_w(d, wing_z(p, f2(0.335f, yw + 0.075f + ff * 0.03f), 0.14f, 17.0f * DEG + ff * 0.75f, 0.020f, 0.10f, 0.94f, 0.11f, 0.25f, 0.4f));
      d = fmin_w(d, wing_z(p, f2(0.425f, yw + 0.118f + ff * 0.07f), 0.12f, 26.0f * DEG + ff, 0.018f, 0.12f, 0.94f, 0.13f, 0.25f, 0.4f));
      ep = round_rect(f2(p.x - 0.25f, p.y - (yw + 0.085f)), f2(0.29f, 0.115f), 0.07f);
    }
    const float span = 0.94f;
    d = fmin_w(d, fmax_w(ep, fabs_w(p.z - (span + 0.012f)) - 0.010f));
    d = fmin_w(d, round_box(sub(p, f3(0.22f, yw - 0.008f, span - 0.04f)), f3(0.30f, 0.006f, 0.06f), 0.004f));
    return d;
  }
  float rear_wing(F3 p, float b, float yr) const {
    uint32_t v = variant(sh.rearWing);
    float chord_m = 0.36f, ang_m = sh.rearMain, rise_m = -0.10f;
    float chord_f = 0.26f, ang_f = sh.rearFlap;
    F2 ep_h = f2(0.33f, 0.29f);
    if (v == 1u) {
      chord_m = 0.42f; ang_m = ang_m + 3.0f * DEG; rise_m = -0.15f;
      chord_f = 0.32f; ang_f = ang_f + 6.0f * DEG;
      ep_h = f2(0.36f, 0.33f);
    } else if (v == 2u) {
      chord_m = 0.27f; ang_m = ang_m - 5.0f * DEG; rise_m = 0.02f;
      chord_f = 0.15f; ang_f = ang_f * 0.55f;
      ep_h = f2(0.30f, 0.25f);
    }
    float d = wing_z(p, f2(4.98f, yr), chord_m, ang_m, 0.05f, 0.0f, 0.50f, rise_m, 0.12f, 0.22f);
    F2 te = add(add(f2(4.98f, yr), mul(f2(wtm::cosf(ang_m), wtm::sinf(ang_m)), chord_m - 0.01f)), f2(-0.03f, 0.035f));
    d = fmin_w(d, wing_z(p, te, chord_f, ang_f, 0.03f, 0.0f, 0.49f, rise_m * 0.8f, 0.10f, 0.28f));
    d = fmin_w(d, capsule(p, f3(5.26f, yr + 0.05f, 0.0f), f3(5.30f, yr + 0.12f, 0.0f), 0.024f));
    float ep = round_rect(f2(p.x - 5.25f, p.y - (yr - 0.03f)), ep_h, 0.13f);
    d = fmin_w(d, fmax_w(ep, fabs_w(p.z - 0.513f) - 0.012f));
    d = fmin_w(d, round_box(sub(p, f3(5.09f, 0.5f * (b + 0.36f + yr + 0.06f), 0.06f)),
                            f3(0.07f, 0.5f * (yr + 0.06f - b - 0.36f), 0.008f), 0.006f));
    return d;
  }
  F2 f1(F3 pw) const {
    F3 pworld = f3(pw.x, pw.y, fabs_w(pw.z));
    F3 p = body_frame(pworld);
    float b = sh.rideH;
    float yw = 0.19f + b * 0.45f;
    float yr = b + 0.80f;
    F2 res = f2(1e3f, 0.0f);
    if (box(sub(p, f3(2.72f, b + 0.52f, 0.0f)), f3(2.74f, 0.62f, 0.95f)) < res.x) {
      res = op_u(res, f2(bodywork(p, b), 0.0f));
      res = op_u(res, f2(ellipsoid(sub(p, f3(2.67f, b + 0.71f, 0.0f)), f3(0.15f, 0.13f, 0.12f)), 3.0f));
      res = op_u(res, f2(halo(p, b), 4.0f));
      float mirror = round_box(sub(p, f3(2.32f, b + 0.67f, 0.60f)), f3(0.035f, 0.035f, 0.085f), 0.02f);
      mirror = fmin_w(mirror, capsule(p, f3(2.36f, b + 0.66f, 0.53f), f3(2.45f, b + 0.50f, 0.46f), 0.011f));
      res = op_u(res, f2(mirror, 0.0f));
      float carbon = suspension(p, b);
      carbon = fmin_w(carbon, taper(p, 4.78f, 5.40f, f2(b + 0.33f, 0.0f), f2(b + 0.33f, 0.0f), f2(0.07f, 0.065f), f2(0.045f, 0.045f), 0.04f, 0.03f));
      carbon = fmin_w(carbon, round_box(sub(p, f3(3.95f, b + 0.74f, 0.0f)), f3(0.55f, 0.10f, 0.008f), 0.006f));
      res = op_u(res, f2(carbon, 1.0f));
      res = op_u(res, f2(round_box(sub(p, f3(5.405f, b + 0.33f, 0.0f)), f3(0.012f, 0.028f, 0.05f), 0.006f), 11.0f));
      float exhaust = capsule(p, f3(4.95f, b + 0.44f, 0.0f), f3(5.13f, b + 0.45f, 0.0f), 0.042f);
      exhaust = fmax_w(exhaust, -capsule(p, f3(5.0f, b + 0.44f, 0.0f), f3(5.2f, b + 0.45f, 0.0f), 0.028f));
      res = op_u(res, f2(exhaust, 10.0f));
    }
    if (box(sub(p, f3(3.26f, b + 0.2f, 0.4f)), f3(1.75f, 0.22f, 0.42f)) < res.x)
      res = op_u(res, f2(floor_(p, b), 1.0f));
    const float lip = BODY_LIP * BODY_X;
    res.x = res.x * lip;
    if (box(sub(p, f3(0.24f, yw + 0.17f, 0.48f)), f3(0.36f, 0.34f, 0.50f)) < res.x / lip)
      res = op_u(res, f2(front_wing(p, yw) * BODY_LIP * BODY_X, 7.0f));  // (d * LIP) * X (f1.ts:309)
    if (box(sub(p, f3(5.20f, b + 0.64f, 0.27f)), f3(0.46f, 0.56f, 0.29f)) < res.x / lip)
      res = op_u(res, f2(rear_wing(p, b, yr) * BODY_LIP * BODY_X, 8.0f));
    res = wheel_set(pworld, res, f3(FA, WR26, FWZ * BODY_Z), FHW26, 0.10f);
    res = wheel_set(pworld, res, f3(RA26, WR26, RWZ * BODY_Z), RHW26, 0.08f);
    return res;
  }
  float f1_emission(F3 pw) const {
    F3 p = body_frame(f3(pw.x, pw.y, fabs_w(pw.z)));
    float b = sh.rideH;
    float e = 0.0f;
    if (len2(sub(f2(p.x, p.y), f2(FA, WR))) < 0.21f && fabs_w(p.z - (FWZ - FHW - 0.03f)) < 0.12f) e = fmax_w(e, sh.heatBrakes);
    if (len2(sub(f2(p.x, p.y), f2(RA, WR))) < 0.21f && fabs_w(p.z - (RWZ - RHW - 0.03f)) < 0.12f) e = fmax_w(e, sh.heatBrakes * 0.8f);
    if (p.x > 5.02f && capsule(p, f3(4.95f, b + 0.44f, 0.0f), f3(5.16f, b + 0.45f, 0.0f), 0.09f) < 0.0f) e = fmax_w(e, sh.heatEngine);
    if (p.x > 3.85f && p.x < 4.5f && p.z > 0.10f && p.y > b + 0.12f && p.y < b + 0.45f) e = fmax_w(e, sh.heatRad);
    if (p.x > 3.55f && p.x < 4.25f && p.z < 0.13f && p.y > b + 0.42f) e = fmax_w(e, sh.heatRad * 1.4f);
    return e;
  }
  // sceneSdf / sceneEmission (wgsl.ts:101-116) for the analytic scenes.
  F2 scene(F3 p) const {
    switch (sh.kind) {
      case 0: return f1(p);
      case 1: return f2(len3(sub(p, f3(2.6f, 1.0f, 0.0f))) - 0.6f, 6.0f);
      case 2: return f2(round_box(sub(p, f3(2.6f, 1.0f, 0.0f)), f3(0.5f, 0.5f, 0.5f), 0.03f), 6.0f);
      case 3: return f2(wing(p, f2(1.6f, 1.2f), 1.8f, -sh.aoa, 0.24f, -1.25f, 1.25f), 6.0f);
      case 6: return f2(1e3f, 0.0f);
      case 7:  // build extension: axis-aligned box
        return f2(box(sub(p, f3(sh.boxCenter[0], sh.boxCenter[1], sh.boxCenter[2])),
                      f3(sh.boxHalf[0], sh.boxHalf[1], sh.boxHalf[2])), 6.0f);
      default: return f2(1e3f, 0.0f);
    }
  }
  float emission(F3 p) const { return sh.kind == 0 ? f1_emission(p) : 0.0f; }
};

// ------------------------------------------------------------ lattice tables (wgsl.ts:123-133)
static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
static const int ZMIR[19] = {0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 13, 14, 11, 12, 17, 18, 15, 16};

template <class R> struct Consts;
template <> struct Consts<float> {
  static float w(int i) { return i == 0 ? 0.33333334f : (i < 7 ? 0.055555556f : 0.027777778f); }
  static float third() { return 0x1.555556p-2f; }
  static float smag_k() { return 0x1.974b24p+4f; }  // 18 * 1.41421356 rounded once to f32
};
template <> struct Consts<double> {
  static double w(int i) { return i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0); }
  static double third() { return 1.0 / 3.0; }
  static double smag_k() { return 18.0 * 1.41421356; }
};

template <class R> static inline R feq(int i, R rho, R ux, R uy, R uz) {
  R cu = (R)CX[i] * ux + (R)CY[i] * uy + (R)CZ[i] * uz;
  R uu = ux * ux + uy * uy + uz * uz;
  return Consts<R>::w(i) * rho * ((R)1 + (R)3 * cu + (R)4.5 * cu * cu - (R)1.5 * uu);
}
template <class R> static inline R rmax(R a, R b) { return a < b ? b : a; }
template <class R> static inline R rmin(R a, R b) { return b < a ? b : a; }
template <class R> static inline R rsmooth(R lo, R hi, R x) {
  R t = rmin(rmax((x - lo) / (hi - lo), (R)0), (R)1);
  return t * t * ((R)3 - (R)2 * t);
}
template <class R> static inline R rsqrt_ieee(R x);
template <> inline float rsqrt_ieee<float>(float x) { return __builtin_sqrtf(x); }
template <> inline double rsqrt_ieee<double>(double x) { return __builtin_sqrt(x); }
static inline bool is_bad(float x) { uint32_t u; memcpy(&u, &x, 4); return (u & 0x7f800000u) == 0x7f800000u; }
static inline bool is_bad(double x) { uint64_t u; memcpy(&u, &x, 8); return (u & 0x7ff0000000000000ull) == 0x7ff0000000000000ull; }
static inline int32_t round_i32(float x) { return f2i_w(__builtin_rintf(x)); }
static inline int32_t round_i32(double x) {
  double r = __builtin_rint(x);
  if (!(r == r)) return 0;
  if (r >= 2147483647.0) return 2147483647;
  if (r <= -2147483648.0) return (int32_t)0x80000000u;
  return (int32_t)r;
}

// Simulation parameters: Sim uniform (wgsl.ts:158) plus the constants the
// reference hard-codes in the collision and heat shaders, exposed so the
// benchmark configurations can set the sponge length they specify.
struct Params {
  float uIn = 0.0925f, tau0 = 0.508f, smag = 0.17f;
  float sponge_cells = 18.0f, sponge_amp = 0.4f;   // wgsl.ts:260 smoothstep(NX-18, NX-1, x) * 0.4
  float inlet_cells = 10.0f, inlet_amp = 0.25f;    // wgsl.ts:260 0.25 * (1 - smoothstep(0, 10, x))
  float cool = 0.004f, diffuse = 0.04f, src_mix = 0.35f;  // engine.ts:263, wgsl.ts:508
};

// ------------------------------------------------------------ the lattice
template <class R>
struct Lattice {
  int nx, ny, nz;
  size_t n;
  float origin[3], h;
  Params prm;
  std::vector<R> fa, fb;            // ping-pong populations, SoA f[i*n + idx]
  std::vector<uint32_t> solid;      // 0 fluid, 1 body, 2 front wing, 3 rear wing
  std::vector<float> emit;
  std::vector<R> fields;            // (ux, uy, uz, rho) per cell
  std::vector<float> ta, tb;        // heat ping-pong
  int32_t forces[12];               // i32 fixed-point accumulator (engine.ts:242)
  double forces64[9];               // same sums in FP64 (x, y, z per group)
  uint64_t guarded = 0;             // cells reset by the divergence guard
  bool cur_a = true;                // which buffer holds the latest populations

  Lattice(int nx_, int ny_, int nz_, const float o[3], float h_) : nx(nx_), ny(ny_), nz(nz_) {
    n = (size_t)nx * ny * nz;
    origin[0] = o[0]; origin[1] = o[1]; origin[2] = o[2]; h = h_;
    fa.assign(n * 19, (R)0); fb.assign(n * 19, (R)0);
    solid.assign(n, 0u); emit.assign(n, 0.0f);
    fields.assign(n * 4, (R)0);
    ta.assign(n, 0.0f); tb.assign(n, 0.0f);
    memset(forces, 0, sizeof(forces));
    memset(forces64, 0, sizeof(forces64));
  }

  // LBM_INIT on both buffers + zeroed temps (engine.ts:371-381, wgsl.ts:147-155).
  void reset() {
    const R u = (R)prm.uIn;
    for (int i = 0; i < 19; i++) {
      R v = feq<R>(i, (R)1, u, (R)0, (R)0);
      for (size_t c = 0; c < n; c++) { fa[i * n + c] = v; fb[i * n + c] = v; }
    }
    for (size_t c = 0; c < n; c++) {
      fields[4 * c] = u; fields[4 * c + 1] = 0; fields[4 * c + 2] = 0; fields[4 * c + 3] = 1;
      ta[c] = 0.0f; tb[c] = 0.0f;
    }
    cur_a = true;
  }

  // VOXELIZE (wgsl.ts:305-321) for the analytic scenes.
  void voxelize(const Shape& sh) {
    Sdf sdf(sh);
#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < nz; z++)
      for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
          size_t idx = (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z);
          F3 p = f3(origin[0] + ((float)x + 0.5f) * h, origin[1] + ((float)y + 0.5f) * h,
                    origin[2] + ((float)z + 0.5f) * h);
          F2 r = sdf.scene(p);
          bool inside = r.x < 0.3f * h && x > 1 && x < nx - 2;
          uint32_t group = 1;
          if (fabs_w(r.y - 7.0f) < 0.5f) group = 2;
          if (fabs_w(r.y - 8.0f) < 0.5f) group = 3;
          solid[idx] = inside ? group : 0u;
          emit[idx] = inside ? sdf.emission(p) : 0.0f;
        }
  }

  // One LBM_STEP dispatch (wgsl.ts:179-291) from `fin` to `fout`.
  void step_once(const std::vector<R>& fin, std::vector<R>& fout) {
    const int NX = nx, NY = ny, NZ = nz;
    const R uin = (R)prm.uIn;
    uint32_t fsum[9] = {0};  // i32 accumulators wrap like the shader's atomicAdd
    std::vector<double> plane64((size_t)NZ * 9, 0.0);
    uint64_t nguard = 0;
#pragma omp parallel for schedule(static) reduction(+ : nguard)
    for (int z = 0; z < NZ; z++) {
      uint32_t local[9] = {0};
      double* p64 = &plane64[(size_t)z * 9];
      for (int y = 0; y < NY; y++)
        for (int x = 0; x < NX; x++) {
          size_t idx = (size_t)x + (size_t)NX * ((size_t)y + (size_t)NY * z);
          R g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
          cell(fin, fout, idx, x, y, z, uin, g, nguard);
          for (int k = 0; k < 3; k++) {
            if (g[k][0] != (R)0) local[3 * k] += (uint32_t)round_i32(g[k][0] * (R)10000);
            if (g[k][1] != (R)0) local[3 * k + 1] += (uint32_t)round_i32(g[k][1] * (R)10000);
            p64[3 * k] += (double)g[k][0];
            p64[3 * k + 1] += (double)g[k][1];
            p64[3 * k + 2] += (double)g[k][2];
          }
        }
#pragma omp critical
      for (int k = 0; k < 9; k++) fsum[k] += local[k];
    }
    for (int k = 0; k < 9; k++) forces[k] = (int32_t)((uint32_t)forces[k] + fsum[k]);
    for (int z = 0; z < NZ; z++)
      for (int k = 0; k < 9; k++) forces64[k] += plane64[(size_t)z * 9 + k];
    guarded += nguard;
  }

  void cell(const std::vector<R>& fin, std::vector<R>& fout, size_t idx, int x, int y, int z, R uin,
            R g[3][3], uint64_t& nguard) {
    const int NX = nx, NY = ny, NZ = nz;
    const size_t N = n;
    if (solid[idx] != 0u) {  // wgsl.ts:182-186
      for (int i = 0; i < 19; i++) fout[i * N + idx] = Consts<R>::w(i);
      for (int k = 0; k < 4; k++) fields[4 * idx + k] = (R)0;
      return;
    }
    // moving belt: no-slip under contact patches (wgsl.ts:191-198)
    R floor_u = uin;
    if (y == 0) {
      size_t row = (size_t)z * NX * NY;
      int xl = x - 2 < 0 ? 0 : x - 2, xr = x + 2 > NX - 1 ? NX - 1 : x + 2;
      int zl = z - 1 < 0 ? 0 : z - 1, zr = z + 1 > NZ - 1 ? NZ - 1 : z + 1;
      if (solid[row + xl] || solid[row + xr] || solid[idx + NX] || solid[(size_t)zl * NX * NY + x] ||
          solid[(size_t)zr * NX * NY + x])
        floor_u = (R)0;
    }
    const R pu[3] = {fields[4 * idx], fields[4 * idx + 1], fields[4 * idx + 2]};
    const bool duct = emit[idx] < 0.0f;
    R f[19];
    for (int i = 0; i < 19; i++) {  // pull streaming with boundary precedence (wgsl.ts:203-229)
      int sx = x - CX[i], sy = y - CY[i], sz = z - CZ[i];
      R v;
      if (sx < 0) v = feq<R>(i, (R)1, uin, (R)0, (R)0);
      else if (sx >= NX) v = feq<R>(i, (R)1, pu[0], pu[1], pu[2]);
      else if (sy < 0) v = fin[OPP[i] * N + idx] + (R)6 * Consts<R>::w(i) * (R)CX[i] * floor_u;
      else if (sy >= NY || sz >= NZ) v = feq<R>(i, (R)1, uin, (R)0, (R)0);
      else {
        int src = i;
        bool mirrored = false;
        if (sz < 0) { sz = 0; src = ZMIR[i]; mirrored = true; }
        size_t sidx = (size_t)sx + (size_t)NX * ((size_t)sy + (size_t)NY * sz);
        uint32_t sg = solid[sidx];
        if (sg != 0u) {
          v = fin[OPP[i] * N + idx];
          if (!mirrored && !duct) {
            R t = (R)2 * (v - Consts<R>::w(i));
            g[sg - 1][0] = g[sg - 1][0] - t * (R)CX[i];
            g[sg - 1][1] = g[sg - 1][1] - t * (R)CY[i];
            g[sg - 1][2] = g[sg - 1][2] - t * (R)CZ[i];
          }
        } else {
          v = fin[src * N + sidx];
        }
      }
      f[i] = v;
    }
    // moments + divergence guard (wgsl.ts:231-243)
    R rho = 0, mx = 0, my = 0, mz = 0;
    for (int i = 0; i < 19; i++) {
      rho = rho + f[i];
      mx = mx + f[i] * (R)CX[i];
      my = my + f[i] * (R)CY[i];
      mz = mz + f[i] * (R)CZ[i];
    }
    R den = rmax(rho, (R)1e-4);
    R ux = mx / den, uy = my / den, uz = mz / den;
    if (is_bad(rho) || is_bad(ux) || is_bad(uy) || is_bad(uz) || rho < (R)0.3 || rho > (R)3 ||
        rsqrt_ieee<R>(ux * ux + uy * uy + uz * uz) > (R)0.35) {
      rho = (R)1;
      ux = uin * (R)0.5; uy = (R)0 * (R)0.5; uz = (R)0 * (R)0.5;
      for (int i = 0; i < 19; i++) f[i] = feq<R>(i, rho, ux, uy, uz);
      for (int k = 0; k < 3; k++) g[k][0] = g[k][1] = g[k][2] = (R)0;
      nguard++;
    }
    if (duct) {  // wgsl.ts:248
      const R t = (R)0.04, tu = (R)1 - t;
      R tx = (R)0.55 * (R)prm.uIn;
      ux = ux * tu + tx * t; uy = uy * tu + uy * t; uz = uz * tu + uz * t;
    }
    // regularized collision + Smagorinsky (wgsl.ts:250-271)
    R pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
    R eq[19];
    for (int i = 0; i < 19; i++) {
      eq[i] = feq<R>(i, rho, ux, uy, uz);
      R ne = f[i] - eq[i];
      R cx = (R)CX[i], cy = (R)CY[i], cz = (R)CZ[i];
      pxx = pxx + ne * cx * cx; pyy = pyy + ne * cy * cy; pzz = pzz + ne * cz * cz;
      pxy = pxy + ne * cx * cy; pxz = pxz + ne * cx * cz; pyz = pyz + ne * cy * cz;
    }
    R q = rsqrt_ieee<R>(pxx * pxx + pyy * pyy + pzz * pzz + (R)2 * (pxy * pxy + pxz * pxz + pyz * pyz));
    const R fx = (R)x, fnx = (R)NX;
    R tau0 = (R)prm.tau0 + (R)prm.sponge_amp * rsmooth<R>(fnx - (R)prm.sponge_cells, fnx - (R)1, fx) +
             (R)prm.inlet_amp * ((R)1 - rsmooth<R>((R)0, (R)prm.inlet_cells, fx));
    R sm = (R)prm.smag;
    R tau = (R)0.5 * (tau0 + rsqrt_ieee<R>(tau0 * tau0 + Consts<R>::smag_k() * sm * sm * q / rho));
    R omega = (R)1 / tau;
    const R third = Consts<R>::third();
    for (int i = 0; i < 19; i++) {
      R cx = (R)CX[i], cy = (R)CY[i], cz = (R)CZ[i];
      R qp = (cx * cx - third) * pxx + (cy * cy - third) * pyy + (cz * cz - third) * pzz +
             (R)2 * (cx * cy * pxy + cx * cz * pxz + cy * cz * pyz);
      fout[i * N + idx] = eq[i] + ((R)1 - omega) * (R)4.5 * Consts<R>::w(i) * qp;
    }
    fields[4 * idx] = ux; fields[4 * idx + 1] = uy; fields[4 * idx + 2] = uz; fields[4 * idx + 3] = rho;
  }

  // The frame's LBM loop (engine.ts:710): n dispatches alternating A->B, B->A.
  void steps(int nsteps) {
    for (int s = 0; s < nsteps; s++) {
      if (cur_a) step_once(fa, fb);
      else step_once(fb, fa);
      cur_a = !cur_a;
    }
  }

  // HEAT (wgsl.ts:480-510): one pass tin -> tout.
  void heat_once(const std::vector<float>& tin, std::vector<float>& tout, float dt) {
    const int NX = nx, NY = ny, NZ = nz;
    auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
    auto idx_of = [&](int x, int y, int z) -> size_t {
      if (z < 0) z = -z - 1;
      x = clampi(x, 0, NX - 1); y = clampi(y, 0, NY - 1); z = clampi(z, 0, NZ - 1);
      return (size_t)x + (size_t)NX * ((size_t)y + (size_t)NY * z);
    };
    auto t_at = [&](int x, int y, int z) -> float { return x < 0 ? 0.0f : tin[idx_of(x, y, z)]; };
#pragma omp parallel for schedule(static)
    for (int z = 0; z < NZ; z++)
      for (int y = 0; y < NY; y++)
        for (int x = 0; x < NX; x++) {
          size_t idx = (size_t)x + (size_t)NX * ((size_t)y + (size_t)NY * z);
          float fw = (float)fields[4 * idx + 3];
          if (fw <= 0.0f) { tout[idx] = emit[idx]; continue; }
          float gx = (float)x - (float)fields[4 * idx] * dt;
          float gy = (float)y - (float)fields[4 * idx + 1] * dt;
          float gz = (float)z - (float)fields[4 * idx + 2] * dt;
          float flx = __builtin_floorf(gx), fly = __builtin_floorf(gy), flz = __builtin_floorf(gz);
          int ix = f2i_w(flx), iy = f2i_w(fly), iz = f2i_w(flz);
          float frx = gx - (float)ix, fry = gy - (float)iy, frz = gz - (float)iz;
          float t = 0.0f;
          for (int k = 0; k < 8; k++) {
            int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
            float w = (ox == 1 ? frx : 1.0f - frx) * (oy == 1 ? fry : 1.0f - fry) * (oz == 1 ? frz : 1.0f - frz);
            t = t + t_at(ix + ox, iy + oy, iz + oz) * w;
          }
          static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
          float nb = 0.0f, src = 0.0f;
          for (int k = 0; k < 6; k++) {
            int cx = x + off[k][0], cy = y + off[k][1], cz = z + off[k][2];
            nb = nb + t_at(cx, cy, cz);
            if (cx >= 0 && cy >= 0 && cx < NX && cy < NY && cz < NZ) src = fmax_w(src, emit[idx_of(cx, cy, cz)]);
          }
          t = fmix_w(t, nb / 6.0f, prm.diffuse);
          if (src > 0.0f) t = fmix_w(t, src, prm.src_mix);
          tout[idx] = fmax_w(t * (1.0f - prm.cool), 0.0f);
        }
  }
  // heat[0] then heat[1] (engine.ts:711-712): tA -> tB -> tA.
  void heat(float dt) {
    heat_once(ta, tb, dt);
    heat_once(tb, ta, dt);
  }

  // Bounce-back link mask as the reference derives it on the fly (wgsl.ts:203-229):
  // bit i (1..18) set when direction i takes the `solid[sidx] != 0` branch for a fluid cell.
  uint32_t link_mask(int x, int y, int z) const {
    const int NX = nx, NY = ny, NZ = nz;
    size_t idx = (size_t)x + (size_t)NX * ((size_t)y + (size_t)NY * z);
    if (solid[idx]) return 0u;
    uint32_t m = 0;
    for (int i = 1; i < 19; i++) {
      int sx = x - CX[i], sy = y - CY[i], sz = z - CZ[i];
      if (sx < 0 || sx >= NX || sy < 0 || sy >= NY || sz >= NZ) continue;
      if (sz < 0) sz = 0;
      size_t sidx = (size_t)sx + (size_t)NX * ((size_t)sy + (size_t)NY * sz);
      if (solid[sidx]) m |= 1u << i;
    }
    return m;
  }
  // Belt contact flag (wgsl.ts:192-197): floorU = 0 for this y=0 cell.
  bool belt_contact(int x, int y, int z) const {
    if (y != 0) return false;
    const int NX = nx, NY = ny, NZ = nz;
    size_t idx = (size_t)x + (size_t)NX * (size_t)NY * z;
    size_t row = (size_t)z * NX * NY;
    int xl = x - 2 < 0 ? 0 : x - 2, xr = x + 2 > NX - 1 ? NX - 1 : x + 2;
    int zl = z - 1 < 0 ? 0 : z - 1, zr = z + 1 > NZ - 1 ? NZ - 1 : z + 1;
    return solid[row + xl] || solid[row + xr] || solid[idx + NX] || solid[(size_t)zl * NX * NY + x] ||
           solid[(size_t)zr * NX * NY + x];
  }
  const std::vector<R>& cur() const { return cur_a ? fa : fb; }
};

}  // namespace wto
