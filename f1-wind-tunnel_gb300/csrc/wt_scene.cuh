// The reference's analytic signed-distance scenes on the device
// (src/engine/wgsl.ts:20-76,101-116 primitives and scene switch;
// src/engine/f1.ts:20-320 generic F1, :397-407 heat emission), shared by the
// voxelizer and the renderer.  Every float operation keeps the reference's
// order (units built with -fmad=false); sin, cos and atan are the project's
// functions (wt_fmath.h).  Shape-wide values (rake rotation, rear main-plane
// direction) are computed once on the host by make_scene with the same
// functions, which gives the same bits as evaluating them per point.
#pragma once
#include <cuda_fp16.h>

#include "wt_fmath.h"
#include "wt_internal.h"
#include "wt_vec.cuh"

namespace wt {
namespace {

// Shape plus host-computed shape-wide constants.
struct Scene {
  wt_shape s;
  CarView car;                // the W17 model (kind 5)
  float rake_c, rake_s;       // cos/sin of the rake angle (f1.ts:37-40)
  float rear_c, rear_s;       // cos/sin of the rear main-plane angle after variant offsets (f1.ts:274)
  float ang_m, ang_f, chord_m, chord_f, rise_m, ep_hx, ep_hy;  // rear-wing variant (f1.ts:260-272)
};

constexpr float DEG = 0.017453292f, FA = 1.0f, RA = 4.6f, WR = 0.36f, FWZ = 0.84f, FHW = 0.152f, RWZ = 0.80f,
                RHW = 0.20f, RA26 = 4.4f, WR26 = 0.355f, FHW26 = 0.14f, RHW26 = 0.1875f, BODY_X = 0.9444444f,
                BODY_Z = 0.96f, BODY_LIP = 0.96f;

// ---------------------------------------------------------------- primitives
__device__ float sd_box(V3 p, V3 b) {
  const V3 q = v3(ab(p.x) - b.x, ab(p.y) - b.y, ab(p.z) - b.z);
  return len3(v3(mx(q.x, 0.0f), mx(q.y, 0.0f), mx(q.z, 0.0f))) + mn(mx(q.x, mx(q.y, q.z)), 0.0f);
}
__device__ float sd_rbox(V3 p, V3 b, float r) { return sd_box(p, v3(b.x - r, b.y - r, b.z - r)) - r; }
__device__ float sd_capsule(V3 p, V3 a, V3 b, float r) {
  const V3 pa = p - a, ba = b - a;
  const float hh = clmp(dv(dot3(pa, ba), dot3(ba, ba)), 0.0f, 1.0f);
  return len3(pa - ba * hh) - r;
}
__device__ float sd_rrect(V2 p, V2 b, float r) {
  const V2 q = v2(ab(p.x) - b.x + r, ab(p.y) - b.y + r);
  return len2(v2(mx(q.x, 0.0f), mx(q.y, 0.0f))) + mn(mx(q.x, q.y), 0.0f) - r;
}
__device__ float op_extrude(float d2, float dz) {
  return mn(mx(d2, dz), 0.0f) + len2(v2(mx(d2, 0.0f), mx(dz, 0.0f)));
}
__device__ float sd_taper(V3 p, float x0, float x1, V2 c0, V2 c1, V2 s0, V2 s1, float r0, float r1) {
  const float t = clmp(dv(p.x - x0, x1 - x0), 0.0f, 1.0f);
  const V2 c = mix2(c0, c1, t);
  const V2 s = mix2(s0, s1, t);
  const float r = mn(mixf(r0, r1, t), mn(s.x, s.y));
  const float d2 = sd_rrect(v2(p.y, p.z) - c, s, r);
  const float dx = ab(p.x - 0.5f * (x0 + x1)) - 0.5f * (x1 - x0);
  return op_extrude(d2, dx) * 0.8f;
}
__device__ float sd_uneven_capsule(V2 p0, float r1, float r2, float hh) {
  const V2 p = v2(ab(p0.x), p0.y);
  const float b = dv(r1 - r2, hh);
  const float a = __fsqrt_rn(mx(1.0f - b * b, 0.0f));
  const float k = dot2(p, v2(-b, a));
  if (k < 0.0f) return len2(p) - r1;
  if (k > a * hh) return len2(p - v2(0.0f, hh)) - r2;
  return dot2(p, v2(a, b)) - r1;
}
__device__ float sd_wing_cs(V3 p, V2 le, float chord, float c, float s, float thick, float z0, float z1) {
  const V2 q = v2(p.x, p.y) - le;
  const float lx = q.x * c + q.y * s;
  const float ly = -q.x * s + q.y * c;
  const float r1 = thick * 0.5f;
  const float r2 = mx(thick * 0.12f, 0.006f);
  const float d2 = sd_uneven_capsule(v2(ly, lx - r1), r1, r2, mx(chord - r1 - r2, 0.01f));
  return op_extrude(d2, ab(p.z - 0.5f * (z0 + z1)) - 0.5f * (z1 - z0));
}
__device__ float sd_wing(V3 p, V2 le, float chord, float ang, float thick, float z0, float z1) {
  return sd_wing_cs(p, le, chord, wtm::cosf(ang), wtm::sinf(ang), thick, z0, z1);
}
__device__ __forceinline__ V2 op_u(V2 a, V2 b) { return (b.x < a.x) ? b : a; }

// ---------------------------------------------------------------- generic F1
__device__ V3 body_frame(const Scene& S, V3 pw) {
  const float c = S.rake_c, s = S.rake_s;
  const float dx = pw.x - FA, dy = pw.y - S.s.ride_h;
  const V3 p = v3(FA + dx * c + dy * s, S.s.ride_h - dx * s + dy * c, pw.z);
  float x = p.x;
  if (x > FA) {
    const float a = FA + dv(x - FA, BODY_X);
    const float b = x + (RA - RA26);
    x = (x > RA26) ? b : a;
  }
  return v3(x, p.y, dv(p.z, BODY_Z));
}
__device__ float smin(float a, float b, float k) {
  const float h = dv(mx(k - ab(a - b), 0.0f), k);
  return mn(a, b) - h * h * k * 0.25f;
}
__device__ float smax(float a, float b, float k) { return -smin(-a, -b, k); }
__device__ float sd_ellipsoid(V3 p, V3 r) {
  const float k0 = len3(v3(dv(p.x, r.x), dv(p.y, r.y), dv(p.z, r.z)));
  const V3 rr = v3(r.x * r.x, r.y * r.y, r.z * r.z);
  const float k1 = len3(v3(dv(p.x, rr.x), dv(p.y, rr.y), dv(p.z, rr.z)));
  return dv(k0 * (k0 - 1.0f), mx(k1, 1e-5f));
}
__device__ float sd_cyl_z(V3 p, float r, float hz) {
  const float dx = len2(v2(p.x, p.y)) - r, dz = ab(p.z) - hz;
  return mn(mx(dx, dz), 0.0f) + len2(v2(mx(dx, 0.0f), mx(dz, 0.0f)));
}
// Out of line (as is wheel_set): sixteen call sites would otherwise each carry a
// copy, with its sin/cos, and the SDF's code would outgrow the instruction cache.
__device__ __noinline__ float sd_wing_z(V3 p, V2 le, float chord, float ang, float thick, float z0, float z1, float rise,
                           float taper, float curl) {
  const float s = sstep(curl, z1, p.z);
  return sd_wing(p, le + v2(0.0f, rise * s), chord * (1.0f - taper * s), ang + rise * s * 0.6f, thick, z0, z1) *
         0.85f;
}
__device__ float tunnel_roof(float x, float b) {
  if (x < 2.5f) return mixf(b + 0.12f, b + 0.05f, sstep(1.55f, 2.5f, x));
  if (x < 3.8f) return b + 0.05f;
  return mixf(b + 0.05f, b + 0.25f, sstep(3.8f, 4.98f, x));
}
__device__ float sd_floor(V3 p, float b) {
  const float roof = tunnel_roof(p.x, b);
  const float zlim = mixf(0.80f, 0.58f, sstep(3.6f, 4.15f, p.x));
  const float top = (ab(p.z - 0.40f) < 0.28f) ? roof + 0.03f : b + 0.05f;
  const float slab = mx(mx(b - p.y, p.y - top), mx(ab(p.x - 3.265f) - 1.715f, p.z - zlim));
  const float tunnel = mx(p.y - roof, ab(p.z - 0.40f) - 0.255f);
  float d = mx(slab, -tunnel) * 0.8f;
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float fz = 0.26f + (float)i * 0.16f;
    const float fence = sd_box(p - v3(1.84f, b + 0.08f, fz), v3(0.28f, 0.08f, 0.012f));
    d = mn(d, mx(fence, p.y - roof - 0.02f));
  }
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float sz = 0.30f + (float)i * 0.20f;
    const float strake = sd_box(p - v3(4.62f, b + 0.17f, sz), v3(0.34f, 0.17f, 0.008f));
    d = mn(d, mx(strake, p.y - roof));
  }
  d = mn(d, sd_capsule(p, v3(2.25f, b + 0.065f, 0.79f), v3(3.85f, b + 0.05f, 0.78f), 0.02f));
  return d;
}
__device__ float sd_tyre(V3 p, V3 c, float hw) {
  const V3 q = p - c;
  return sd_rrect(v2(len2(v2(q.x, q.y)) - 0.2925f, q.z), v2(0.0625f, hw), 0.06f);
}
__device__ float sd_wheel_cover(V3 p, V3 c, float hw) {
  const V3 q = p - c;
  float d = sd_cyl_z(q, 0.234f, hw - 0.028f);
  d = mn(d, sd_cyl_z(q - v3(0.0f, 0.0f, hw - 0.02f), 0.045f, 0.02f));
  return d;
}
__device__ __noinline__ V2 wheel_set(V3 p, V2 res, V3 c, float hw, float inboard) {
  if (sd_box(p - c, v3(WR26 + 0.02f, WR26 + 0.02f, hw + 0.2f)) > res.x) return res;
  res = op_u(res, v2(sd_tyre(p, c, hw), 2.0f));
  res = op_u(res, v2(sd_wheel_cover(p, c, hw), 9.0f));
  const float duct = sd_cyl_z(p - v3(c.x, c.y, c.z - hw - inboard * 0.5f), 0.17f, inboard * 0.5f);
  const float duct_wing = sd_rbox(p - v3(c.x - 0.04f, c.y + 0.21f, c.z - hw - 0.05f), v3(0.16f, 0.012f, 0.05f), 0.006f);
  return op_u(res, v2(mn(duct, duct_wing), 10.0f));
}
__device__ float sd_suspension(V3 p, float b) {
  const float fz = FWZ - FHW - 0.05f, rz = RWZ - RHW - 0.05f;
  float d = sd_capsule(p, v3(1.10f, b + 0.43f, 0.17f), v3(FA + 0.02f, WR + 0.16f, fz), 0.017f);
  d = mn(d, sd_capsule(p, v3(1.42f, b + 0.40f, 0.17f), v3(FA + 0.02f, WR + 0.16f, fz), 0.017f));
  d = mn(d, sd_capsule(p, v3(0.98f, b + 0.19f, 0.15f), v3(FA, WR - 0.13f, fz), 0.017f));
  d = mn(d, sd_capsule(p, v3(1.38f, b + 0.17f, 0.15f), v3(FA, WR - 0.13f, fz), 0.017f));
  d = mn(d, sd_capsule(p, v3(FA + 0.03f, WR - 0.10f, FWZ - FHW - 0.07f), v3(1.20f, b + 0.47f, 0.16f), 0.014f));
  d = mn(d, sd_capsule(p, v3(0.86f, b + 0.29f, 0.16f), v3(0.88f, WR + 0.02f, fz), 0.013f));
  d = mn(d, sd_capsule(p, v3(4.30f, b + 0.42f, 0.20f), v3(RA, WR + 0.17f, rz), 0.017f));
  d = mn(d, sd_capsule(p, v3(4.78f, b + 0.40f, 0.16f), v3(RA, WR + 0.17f, rz), 0.017f));
  d = mn(d, sd_capsule(p, v3(4.28f, b + 0.16f, 0.24f), v3(RA, WR - 0.14f, rz), 0.017f));
  d = mn(d, sd_capsule(p, v3(4.82f, b + 0.15f, 0.18f), v3(RA, WR - 0.14f, rz), 0.017f));
  d = mn(d, sd_capsule(p, v3(RA - 0.03f, WR + 0.14f, RWZ - RHW - 0.07f), v3(4.40f, b + 0.18f, 0.22f), 0.014f));
  return d;
}
__device__ float sd_nose(const Scene& S, V3 p, float b) {
  const uint32_t v = variant(S.s.nose);
  const float x0 = (v == 1u) ? 0.34f : 0.10f;
  const float y0 = b + ((v == 2u) ? 0.25f : 0.17f);
  V2 s0 = v2(0.055f, 0.11f);
  if (v == 1u) s0 = v2(0.075f, 0.15f);
  if (v == 2u) s0 = v2(0.045f, 0.075f);
  float d = sd_taper(p, x0, 1.26f, v2(y0, 0.0f), v2(b + 0.36f, 0.0f), s0, v2(0.15f, 0.17f), 0.04f, 0.12f);
  d = smin(d, sd_ellipsoid(p - v3(x0 + 0.02f, y0, 0.0f), v3(0.09f, s0.x, s0.y)), 0.04f);
  if (v != 0u) {
    const float yw = 0.19f + b * 0.45f;
    const float pylon = sd_rbox(p - v3(x0 + 0.06f, 0.5f * (yw + y0), 0.09f), v3(0.09f, 0.5f * (y0 - yw) + 0.02f, 0.006f), 0.004f);
    d = mn(d, pylon);
  }
  return d;
}
__device__ float sd_engine_cover(const Scene& S, V3 p, float b) {
  const uint32_t v = variant(S.s.cover);
  if (v == 1u) return sd_taper(p, 2.96f, 4.86f, v2(b + 0.60f, 0.0f), v2(b + 0.40f, 0.0f), v2(0.32f, 0.31f), v2(0.12f, 0.13f), 0.15f, 0.08f);
  if (v == 2u) return sd_taper(p, 2.96f, 4.70f, v2(b + 0.57f, 0.0f), v2(b + 0.34f, 0.0f), v2(0.29f, 0.19f), v2(0.06f, 0.05f), 0.12f, 0.04f);
  return sd_taper(p, 2.96f, 4.86f, v2(b + 0.58f, 0.0f), v2(b + 0.36f, 0.0f), v2(0.30f, 0.24f), v2(0.08f, 0.07f), 0.14f, 0.06f);
}
__device__ float sd_sidepods(const Scene& S, V3 p, float b) {
  const uint32_t v = variant(S.s.sidepod);
  float pod;
  if (v == 1u) {
    pod = sd_taper(p, 2.30f, 4.05f, v2(b + 0.40f, 0.36f), v2(b + 0.24f, 0.24f), v2(0.16f, 0.08f), v2(0.07f, 0.05f), 0.06f, 0.04f);
    return smax(pod, -sd_rbox(p - v3(2.27f, b + 0.42f, 0.38f), v3(0.06f, 0.12f, 0.05f), 0.03f), 0.02f);
  }
  if (v == 2u) {
    pod = sd_taper(p, 2.30f, 4.25f, v2(b + 0.41f, 0.52f), v2(b + 0.24f, 0.30f), v2(0.18f, 0.28f), v2(0.08f, 0.11f), 0.10f, 0.05f);
    pod = smax(pod, -sd_capsule(p, v3(2.30f, b + 0.13f, 0.84f), v3(3.70f, b + 0.08f, 0.58f), 0.15f), 0.05f);
    pod = smax(pod, -sd_capsule(p, v3(2.55f, b + 0.66f, 0.52f), v3(4.00f, b + 0.40f, 0.36f), 0.11f), 0.04f);
    return smax(pod, -sd_rbox(p - v3(2.28f, b + 0.47f, 0.57f), v3(0.06f, 0.10f, 0.17f), 0.05f), 0.02f);
  }
  if (v == 3u) {
    pod = sd_taper(p, 2.30f, 4.25f, v2(b + 0.47f, 0.52f), v2(b + 0.26f, 0.28f), v2(0.15f, 0.25f), v2(0.07f, 0.10f), 0.12f, 0.05f);
    pod = smax(pod, -sd_capsule(p, v3(2.25f, b + 0.17f, 0.86f), v3(3.70f, b + 0.10f, 0.56f), 0.22f), 0.05f);
    return smax(pod, -sd_rbox(p - v3(2.28f, b + 0.52f, 0.55f), v3(0.06f, 0.07f, 0.17f), 0.04f), 0.02f);
  }
  pod = sd_taper(p, 2.30f, 4.25f, v2(b + 0.41f, 0.52f), v2(b + 0.22f, 0.28f), v2(0.18f, 0.25f), v2(0.07f, 0.10f), 0.12f, 0.05f);
  pod = smax(pod, -sd_capsule(p, v3(2.30f, b + 0.13f, 0.82f), v3(3.70f, b + 0.08f, 0.56f), 0.16f), 0.05f);
  return smax(pod, -sd_rbox(p - v3(2.28f, b + 0.47f, 0.57f), v3(0.06f, 0.10f, 0.17f), 0.05f), 0.02f);
}
__device__ float sd_bodywork(const Scene& S, V3 p, float b) {
  float d = sd_nose(S, p, b);
  d = smin(d, sd_taper(p, 1.20f, 2.24f, v2(b + 0.36f, 0.0f), v2(b + 0.42f, 0.0f), v2(0.15f, 0.17f), v2(0.25f, 0.29f), 0.12f, 0.16f), 0.08f);
  d = smin(d, sd_taper(p, 2.20f, 3.06f, v2(b + 0.42f, 0.0f), v2(b + 0.42f, 0.0f), v2(0.25f, 0.30f), v2(0.25f, 0.34f), 0.16f, 0.16f), 0.06f);
  d = smin(d, sd_engine_cover(S, p, b), 0.10f);
  const float keel = sd_taper(p, 1.30f, 4.70f, v2(b + 0.22f, 0.0f), v2(b + 0.20f, 0.0f), v2(0.19f, 0.19f), v2(0.17f, 0.14f), 0.06f, 0.05f);
  d = smin(d, keel, 0.08f);
  d = smin(d, sd_sidepods(S, p, b), 0.12f);
  float airbox = sd_rbox(p - v3(3.02f, b + 0.84f, 0.0f), v3(0.17f, 0.11f, 0.12f), 0.08f);
  airbox = smax(airbox, -sd_ellipsoid(p - v3(2.85f, b + 0.86f, 0.0f), v3(0.09f, 0.066f, 0.078f)), 0.015f);
  d = smin(d, airbox, 0.10f);
  return smax(d, -sd_rbox(p - v3(2.62f, b + 0.72f, 0.0f), v3(0.42f, 0.13f, 0.215f), 0.10f), 0.03f);
}
__device__ float sd_halo(V3 p, float b) {
  float d = sd_capsule(p, v3(2.17f, b + 0.62f, 0.0f), v3(2.36f, b + 0.90f, 0.0f), 0.034f);
  d = smin(d, sd_capsule(p, v3(2.36f, b + 0.90f, 0.0f), v3(2.52f, b + 0.92f, 0.20f), 0.031f), 0.03f);
  d = smin(d, sd_capsule(p, v3(2.52f, b + 0.92f, 0.20f), v3(2.82f, b + 0.88f, 0.26f), 0.031f), 0.03f);
  return smin(d, sd_capsule(p, v3(2.82f, b + 0.88f, 0.26f), v3(3.02f, b + 0.74f, 0.25f), 0.033f), 0.03f);
}
__device__ float sd_front_wing(const Scene& S, V3 p, float yw) {
  const float ff = S.s.front_flap;
  const uint32_t v = variant(S.s.front_wing);
  float d, ep;
  if (v == 1u) {
    d = sd_wing_z(p, v2(-0.03f, yw), 0.31f, 2.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, 0.03f, 0.2f, 0.5f);
    d = mn(d, sd_wing_z(p, v2(0.21f, yw + 0.036f), 0.17f, 9.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, 0.15f, 0.35f, 0.3f));
    d = mn(d, sd_wing_z(p, v2(0.335f, yw + 0.075f + ff * 0.03f), 0.14f, 17.0f * DEG + ff * 0.75f, 0.020f, 0.10f, 0.94f, 0.19f, 0.35f, 0.25f));
    d = mn(d, sd_wing_z(p, v2(0.425f, yw + 0.118f + ff * 0.07f), 0.12f, 26.0f * DEG + ff, 0.018f, 0.12f, 0.94f, 0.22f, 0.4f, 0.25f));
    ep = sd_rrect(v2(p.x - 0.25f, p.y - (yw + 0.17f)), v2(0.29f, 0.20f), 0.08f);
  } else if (v == 2u) {
    d = sd_wing_z(p, v2(-0.03f, yw), 0.31f, 3.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, -0.02f, 0.15f, 0.55f);
    d = mn(d, sd_wing_z(p, v2(0.21f, yw + 0.04f), 0.19f, 13.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, -0.04f, 0.35f, 0.35f));
    d = mn(d, sd_wing_z(p, v2(0.35f, yw + 0.085f + ff * 0.03f), 0.16f, 22.0f * DEG + ff * 0.75f, 0.020f, 0.06f, 0.94f, -0.06f, 0.4f, 0.35f));
    d = mn(d, sd_wing_z(p, v2(0.45f, yw + 0.13f + ff * 0.07f), 0.13f, 31.0f * DEG + ff, 0.018f, 0.08f, 0.94f, -0.08f, 0.45f, 0.35f));
    ep = sd_rrect(v2(p.x - 0.25f, p.y - (yw + 0.06f)), v2(0.29f, 0.10f), 0.06f);
  } else if (v == 3u) {
    d = sd_wing_z(p, v2(-0.03f, yw), 0.30f, 1.0f * DEG + ff * 0.05f, 0.030f, 0.0f, 0.94f, 0.0f, 0.1f, 0.6f);
    d = mn(d, sd_wing_z(p, v2(0.20f, yw + 0.03f), 0.16f, 4.0f * DEG + ff * 0.3f, 0.022f, 0.0f, 0.94f, 0.02f, 0.2f, 0.5f));
    ep = sd_rrect(v2(p.x - 0.22f, p.y - (yw + 0.05f)), v2(0.26f, 0.085f), 0.05f);
  } else {
    d = sd_wing_z(p, v2(-0.03f, yw), 0.31f, 2.0f * DEG + ff * 0.1f, 0.034f, 0.0f, 0.94f, 0.06f, 0.2f, 0.5f);
    d = mn(d, sd_wing_z(p, v2(0.21f, yw + 0.036f), 0.17f, 9.0f * DEG + ff * 0.45f, 0.024f, 0.0f, 0.94f, 0.09f, 0.25f, 0.45f));
    d = mn(d, sd_wing_z(p, v2(0.335f, yw + 0.075f + ff * 0.03f), 0.14f, 17.0f * DEG + ff * 0.75f, 0.020f, 0.10f, 0.94f, 0.11f, 0.25f, 0.4f));
    d = mn(d, sd_wing_z(p, v2(0.425f, yw + 0.118f + ff * 0.07f), 0.12f, 26.0f * DEG + ff, 0.018f, 0.12f, 0.94f, 0.13f, 0.25f, 0.4f));
    ep = sd_rrect(v2(p.x - 0.25f, p.y - (yw + 0.085f)), v2(0.29f, 0.115f), 0.07f);
  }
  const float span = 0.94f;
  d = mn(d, mx(ep, ab(p.z - (span + 0.012f)) - 0.010f));
  return mn(d, sd_rbox(p - v3(0.22f, yw - 0.008f, span - 0.04f), v3(0.30f, 0.006f, 0.06f), 0.004f));
}
__device__ float sd_rear_wing(const Scene& S, V3 p, float b, float yr) {
  float d = sd_wing_z(p, v2(4.98f, yr), S.chord_m, S.ang_m, 0.05f, 0.0f, 0.50f, S.rise_m, 0.12f, 0.22f);
  const V2 te = (v2(4.98f, yr) + v2(S.rear_c, S.rear_s) * (S.chord_m - 0.01f)) + v2(-0.03f, 0.035f);
  d = mn(d, sd_wing_z(p, te, S.chord_f, S.ang_f, 0.03f, 0.0f, 0.49f, S.rise_m * 0.8f, 0.10f, 0.28f));
  d = mn(d, sd_capsule(p, v3(5.26f, yr + 0.05f, 0.0f), v3(5.30f, yr + 0.12f, 0.0f), 0.024f));
  const float ep = sd_rrect(v2(p.x - 5.25f, p.y - (yr - 0.03f)), v2(S.ep_hx, S.ep_hy), 0.13f);
  d = mn(d, mx(ep, ab(p.z - 0.513f) - 0.012f));
  return mn(d, sd_rbox(p - v3(5.09f, 0.5f * (b + 0.36f + yr + 0.06f), 0.06f), v3(0.07f, 0.5f * (yr + 0.06f - b - 0.36f), 0.008f), 0.006f));
}
__device__ V2 sd_f1(const Scene& S, V3 pw) {
  const V3 pworld = v3(pw.x, pw.y, ab(pw.z));
  const V3 p = body_frame(S, pworld);
  const float b = S.s.ride_h;
  const float yw = 0.19f + b * 0.45f;
  const float yr = b + 0.80f;
  V2 res = v2(1e3f, 0.0f);
  if (sd_box(p - v3(2.72f, b + 0.52f, 0.0f), v3(2.74f, 0.62f, 0.95f)) < res.x) {
    res = op_u(res, v2(sd_bodywork(S, p, b), 0.0f));
    res = op_u(res, v2(sd_ellipsoid(p - v3(2.67f, b + 0.71f, 0.0f), v3(0.15f, 0.13f, 0.12f)), 3.0f));
    res = op_u(res, v2(sd_halo(p, b), 4.0f));
    float mirror = sd_rbox(p - v3(2.32f, b + 0.67f, 0.60f), v3(0.035f, 0.035f, 0.085f), 0.02f);
    mirror = mn(mirror, sd_capsule(p, v3(2.36f, b + 0.66f, 0.53f), v3(2.45f, b + 0.50f, 0.46f), 0.011f));
    res = op_u(res, v2(mirror, 0.0f));
    float carbon = sd_suspension(p, b);
    carbon = mn(carbon, sd_taper(p, 4.78f, 5.40f, v2(b + 0.33f, 0.0f), v2(b + 0.33f, 0.0f), v2(0.07f, 0.065f), v2(0.045f, 0.045f), 0.04f, 0.03f));
    carbon = mn(carbon, sd_rbox(p - v3(3.95f, b + 0.74f, 0.0f), v3(0.55f, 0.10f, 0.008f), 0.006f));
    res = op_u(res, v2(carbon, 1.0f));
    res = op_u(res, v2(sd_rbox(p - v3(5.405f, b + 0.33f, 0.0f), v3(0.012f, 0.028f, 0.05f), 0.006f), 11.0f));
    float exhaust = sd_capsule(p, v3(4.95f, b + 0.44f, 0.0f), v3(5.13f, b + 0.45f, 0.0f), 0.042f);
    exhaust = mx(exhaust, -sd_capsule(p, v3(5.0f, b + 0.44f, 0.0f), v3(5.2f, b + 0.45f, 0.0f), 0.028f));
    res = op_u(res, v2(exhaust, 10.0f));
  }
  if (sd_box(p - v3(3.26f, b + 0.2f, 0.4f), v3(1.75f, 0.22f, 0.42f)) < res.x) res = op_u(res, v2(sd_floor(p, b), 1.0f));
  const float lip = BODY_LIP * BODY_X;
  res.x = res.x * lip;
  if (sd_box(p - v3(0.24f, yw + 0.17f, 0.48f), v3(0.36f, 0.34f, 0.50f)) < dv(res.x, lip))
    res = op_u(res, v2(sd_front_wing(S, p, yw) * BODY_LIP * BODY_X, 7.0f));  // (d * LIP) * X, as written
  if (sd_box(p - v3(5.20f, b + 0.64f, 0.27f), v3(0.46f, 0.56f, 0.29f)) < dv(res.x, lip))
    res = op_u(res, v2(sd_rear_wing(S, p, b, yr) * BODY_LIP * BODY_X, 8.0f));
  res = wheel_set(pworld, res, v3(FA, WR26, FWZ * BODY_Z), FHW26, 0.10f);
  res = wheel_set(pworld, res, v3(RA26, WR26, RWZ * BODY_Z), RHW26, 0.08f);
  return res;
}
__device__ float f1_emission(const Scene& S, V3 pw) {
  const V3 p = body_frame(S, v3(pw.x, pw.y, ab(pw.z)));
  const float b = S.s.ride_h;
  float e = 0.0f;
  if (len2(v2(p.x - FA, p.y - WR)) < 0.21f && ab(p.z - (FWZ - FHW - 0.03f)) < 0.12f) e = mx(e, S.s.heat_brakes);
  if (len2(v2(p.x - RA, p.y - WR)) < 0.21f && ab(p.z - (RWZ - RHW - 0.03f)) < 0.12f) e = mx(e, S.s.heat_brakes * 0.8f);
  if (p.x > 5.02f && sd_capsule(p, v3(4.95f, b + 0.44f, 0.0f), v3(5.16f, b + 0.45f, 0.0f), 0.09f) < 0.0f) e = mx(e, S.s.heat_engine);
  if (p.x > 3.85f && p.x < 4.5f && p.z > 0.10f && p.y > b + 0.12f && p.y < b + 0.45f) e = mx(e, S.s.heat_rad);
  if (p.x > 3.55f && p.x < 4.25f && p.z < 0.13f && p.y > b + 0.42f) e = mx(e, S.s.heat_rad * 1.4f);
  return e;
}

// ---------------------------------------------------------------- baked W17 model (kind 5)
// src/engine/f1.ts:322-394 and the rig functions of src/engine/car-model.ts:59-136.
constexpr float W17_H = 0.015f, W17_BASE_RIDE = 0.092f;
constexpr int RIG_HINGES = 71, RIG_ANGLES = 72, RIG_EXTRA = 73, RIG_FLY = 74, RIG_GRIDS = 75;

__device__ __forceinline__ float4 rig_at(const float4* R, int i) { return __ldg(R + i); }
__device__ __forceinline__ float half_at(const uint16_t* t, size_t i) {
  return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short*>(t) + i)));
}
// textureSampleLevel of an r16float texture through the engine's linear,
// clamp-to-edge sampler (engine.ts:270) with f32 weights: c = uvw * size - 0.5,
// i = floor(c), t = c - i, clamped indices, blended along x, then y, then z.
__device__ __forceinline__ int floor_index(float f, int n) { return (int)(f < -1.0f ? -1.0f : (f > (float)n ? (float)n : f)); }
__device__ float sample3(const uint16_t* tex, int w, int h, int d, V3 uvw) {
  const float cx = uvw.x * (float)w - 0.5f, cy = uvw.y * (float)h - 0.5f, cz = uvw.z * (float)d - 0.5f;
  const float fx = floorf(cx), fy = floorf(cy), fz = floorf(cz);
  const float tx = cx - fx, ty = cy - fy, tz = cz - fz;
  const int i = floor_index(fx, w), j = floor_index(fy, h), k = floor_index(fz, d);
  auto at = [&](int x, int y, int z) {
    x = x < 0 ? 0 : (x >= w ? w - 1 : x);
    y = y < 0 ? 0 : (y >= h ? h - 1 : y);
    z = z < 0 ? 0 : (z >= d ? d - 1 : z);
    return half_at(tex, ((size_t)z * (size_t)h + (size_t)y) * (size_t)w + (size_t)x);
  };
  const float c00 = at(i, j, k) * (1.0f - tx) + at(i + 1, j, k) * tx;
  const float c10 = at(i, j + 1, k) * (1.0f - tx) + at(i + 1, j + 1, k) * tx;
  const float c01 = at(i, j, k + 1) * (1.0f - tx) + at(i + 1, j, k + 1) * tx;
  const float c11 = at(i, j + 1, k + 1) * (1.0f - tx) + at(i + 1, j + 1, k + 1) * tx;
  const float c0 = c00 * (1.0f - ty) + c10 * ty, c1 = c01 * (1.0f - ty) + c11 * ty;
  return c0 * (1.0f - tz) + c1 * tz;
}

// rigWeight, rigHinge, rigAngle, rigScale, rigRotate (car-model.ts:70-118); the
// RIG constants (car-model.ts:44-49) as the reference interpolates them
__device__ float rig_weight(uint32_t part, float z) {
  if (part == 1u || part == 2u) {
    const float az = ab(z);
    return sstep(0.16f, 0.22f, az) * (1.0f - sstep(0.5f, 0.56f, az));
  }
  return (part == 3u || part == 4u) ? 1.0f : 0.0f;
}
__device__ V2 rig_hinge(const float4* R, uint32_t part, float z) {
  if (part == 3u) { const float4 g = rig_at(R, RIG_HINGES); return v2(g.z, g.w); }
  if (part == 4u) { const float4 g = rig_at(R, RIG_HINGES); return v2(g.x, g.y); }
  const float f = clmp(ab(z) / 0.01f, 0.0f, 70.0f);
  const uint32_t i = (uint32_t)floorf(f);
  const uint32_t j = (i + 1u) < 70u ? i + 1u : 70u;
  const float4 a = rig_at(R, (int)i), b = rig_at(R, (int)j);
  const float t = f - (float)i;
  return part == 1u ? mix2(v2(a.x, a.y), v2(b.x, b.y), t) : mix2(v2(a.z, a.w), v2(b.z, b.w), t);
}
__device__ float rig_angle(const float4* R, uint32_t part, float z) {
  const float4 an = rig_at(R, RIG_ANGLES);
  float a = 0.0f;
  if (part == 1u) a = an.x;
  else if (part == 2u) a = an.y;
  else if (part == 3u) a = an.z;
  else if (part == 4u) a = an.w;
  if (part == 3u || part == 4u) a = a + rig_at(R, RIG_EXTRA).x * sstep(0.12f, 0.48f, ab(z));
  return a * rig_weight(part, z);
}
__device__ float rig_scale(const float4* R, uint32_t part) {
  const float ey = rig_at(R, RIG_EXTRA).y;
  if (part == 3u) return ey;
  if (part == 1u || part == 2u) return 1.0f - (1.0f - ey) * 0.65f;
  return 1.0f;
}
// rigRotate with dir = -1 (the distance field's direction)
__device__ V3 rig_rotate_back(const Scene& S, V3 p, uint32_t part) {
  if (part == 0u || part > 4u) return p;
  const float a = rig_angle(S.car.rig, part, p.z) * -1.0f;
  const float k = rig_scale(S.car.rig, part);
  const V2 h = rig_hinge(S.car.rig, part, p.z);
  const float c = wtm::cosf(a), s = wtm::sinf(a);
  V2 d = v2(p.x, p.y) - h;
  d = v2(c * d.x - s * d.y, s * d.x + c * d.y);
  d = v2(dv(d.x, k), dv(d.y, k));
  return v3(h.x + d.x, h.y + d.y, p.z);
}
// podWeight, podDeform (car-model.ts:121-135), dir = -1
__device__ float pod_weight(V3 p) {
  return sstep(1.85f, 2.25f, p.x) * (1.0f - sstep(3.55f, 4.05f, p.x)) * sstep(0.12f, 0.2f, p.y) *
         (1.0f - sstep(0.6f, 0.7f, p.y)) * sstep(0.26f, 0.4f, ab(p.z));
}
__device__ V3 pod_deform_back(const Scene& S, V3 p) {
  const float c = rig_at(S.car.rig, RIG_EXTRA).z * pod_weight(p);
  if (c <= 0.0f) return p;
  const float az = ab(p.z);
  const float kz = dv(1.0f, 1.0f - c);
  const float ky = dv(1.0f, 1.0f - 0.45f * c);
  const float nz = az > 0.26f ? 0.26f + (az - 0.26f) * kz : az;
  const float sg = p.z > 0.0f ? 1.0f : (p.z < 0.0f ? -1.0f : 0.0f);
  return v3(p.x, 0.12f + (p.y - 0.12f) * ky, sg * nz);
}
// w17BodyFrame (f1.ts:329-334), with the rake of toBodyFrame
__device__ V3 w17_body_frame(const Scene& S, V3 pw) {
  const float dx = pw.x - FA, dy = pw.y - S.s.ride_h;
  return v3(FA + dx * S.rake_c + dy * S.rake_s, W17_BASE_RIDE - dx * S.rake_s + dy * S.rake_c, pw.z);
}
// sdW17Body (f1.ts:335-341)
__device__ float sd_w17_body(const Scene& S, V3 p) {
  const V3 ext = v3(368.0f * W17_H, 84.0f * W17_H, 67.0f * W17_H);
  const V3 half = ext * 0.5f;
  const float box = sd_box(p - v3(-0.3f + half.x, 0.0f + half.y, 0.0f + half.z), half);
  if (box > 0.0f) return box + 0.07f;
  const V3 uvw = v3(dv(dv(p.x - -0.3f, W17_H) + 0.5f, 368.0f), dv(dv(p.y - 0.0f, W17_H) + 0.5f, 84.0f),
                    dv(dv(p.z - 0.0f, W17_H) + 0.5f, 67.0f));
  return sample3(S.car.body, 368, 84, 67, uvw);
}
// sdW17Part (f1.ts:342-353)
__device__ __noinline__ float sd_w17_part(const Scene& S, V3 pb, uint32_t part) {
  const float4 g0 = rig_at(S.car.rig, RIG_GRIDS + (int)(part - 1u) * 2), g1 = rig_at(S.car.rig, RIG_GRIDS + (int)(part - 1u) * 2 + 1);
  const V3 q = rig_rotate_back(S, pb, part);
  const V3 ext = v3((g1.x - 1.0f) * g0.w, (g1.y - 1.0f) * g0.w, (g1.z - 1.0f) * g0.w);
  const V3 half = ext * 0.5f;
  const float box = sd_box(q - v3(g0.x + half.x, g0.y + half.y, g0.z + half.z), half);
  if (box > 0.0f) return box + 0.03f;
  const V3 cell = v3(dv(q.x - g0.x, g0.w), dv(q.y - g0.y, g0.w), dv(q.z - g0.z, g0.w));
  const float ax = (float)S.car.pdims[0], ay = (float)S.car.pdims[1], az = (float)S.car.pdims[2];
  const V3 uvw = v3(dv(cell.x + 0.5f, ax), dv(cell.y + 0.5f, ay), dv(cell.z + g1.w + 0.5f, az));
  const float sc = rig_scale(S.car.rig, part);
  return sample3(S.car.parts, (int)S.car.pdims[0], (int)S.car.pdims[1], (int)S.car.pdims[2], uvw) * mn(sc, 1.0f);
}
// sdW17 (f1.ts:354-369)
__device__ __noinline__ V2 sd_w17(const Scene& S, V3 pw) {
  const V3 pa = v3(pw.x, pw.y, ab(pw.z));
  const V3 p = w17_body_frame(S, pa);
  const float squeeze = 1.0f - rig_at(S.car.rig, RIG_EXTRA).z * pod_weight(p);
  V2 res = v2(sd_w17_body(S, pod_deform_back(S, p)) * 0.95f * squeeze, 12.0f);
  const float4 fly = rig_at(S.car.rig, RIG_FLY);
  if (fly.z > 0.5f && p.x < 0.85f && p.y < 0.6f)
    res = op_u(res, v2(mn(mn(sd_w17_part(S, p, 1u), sd_w17_part(S, p, 2u)), sd_w17_part(S, p, 5u)) * 0.95f, 7.0f));
  if (fly.w > 0.5f && p.x > 4.4f && p.y > 0.5f)
    res = op_u(res, v2(mn(mn(sd_w17_part(S, p, 3u), sd_w17_part(S, p, 4u)), sd_w17_part(S, p, 6u)) * 0.95f, 8.0f));
  const V3 front = v3(1.0f, 0.36f, 0.779f), rear = v3(4.4f, 0.351f, 0.737f);
  res = op_u(res, v2(mn(sd_tyre(pa, front, 0.175f), sd_cyl_z(pa - front, 0.234f, 0.15f)), 2.0f));
  res = op_u(res, v2(mn(sd_tyre(pa, rear, 0.205f), sd_cyl_z(pa - rear, 0.234f, 0.18f)), 2.0f));
  return res;
}
// w17Duct (f1.ts:374-383)
__device__ float w17_duct(const Scene& S, V3 pw) {
  if (S.s.duct <= 0.0f) return 1e3f;
  const V3 p = pod_deform_back(S, w17_body_frame(S, v3(pw.x, pw.y, ab(pw.z))));
  const float k = S.s.duct;
  const float mouth = sd_capsule(p, v3(2.05f, 0.52f, 0.58f), v3(3.0f, 0.50f, 0.48f), 0.09f * k);
  const float main = sd_capsule(p, v3(2.05f, 0.55f, 0.47f), v3(3.25f, 0.46f, 0.43f), 0.1f * k);
  const float exit = sd_capsule(p, v3(3.25f, 0.46f, 0.43f), v3(4.1f, 0.40f, 0.32f), 0.085f * k);
  return mn(mn(mouth, main), exit);
}
// w17Emission (f1.ts:386-394)
__device__ float w17_emission(const Scene& S, V3 pw) {
  const V3 pa = v3(pw.x, pw.y, ab(pw.z));
  const V3 p = w17_body_frame(S, pa);
  float e = 0.0f;
  if (len2(v2(pa.x - 1.0f, pa.y - 0.36f)) < 0.2f && ab(pa.z - (0.779f - 0.215f)) < 0.1f) e = mx(e, S.s.heat_brakes);
  if (len2(v2(pa.x - 4.4f, pa.y - 0.351f)) < 0.2f && ab(pa.z - (0.737f - 0.245f)) < 0.1f) e = mx(e, S.s.heat_brakes * 0.8f);
  if (len3(p - v3(5.07f, 0.53f, 0.0f)) < 0.1f) e = mx(e, S.s.heat_engine);
  if (p.x > 3.7f && p.x < 4.3f && p.y > 0.2f && p.y < 0.5f && p.z > 0.18f && p.z < 0.48f) e = mx(e, S.s.heat_rad);
  if (p.x > 4.15f && p.x < 4.65f && p.y > 0.5f && p.z < 0.16f) e = mx(e, S.s.heat_rad * 1.4f);
  return e;
}

__device__ V2 scene_sdf(const Scene& S, V3 p) {
  switch (S.s.kind) {
    case WT_KIND_F1: return sd_f1(S, p);
    case WT_KIND_SPHERE: return v2(len3(p - v3(2.6f, 1.0f, 0.0f)) - 0.6f, 6.0f);
    case WT_KIND_CUBE: return v2(sd_rbox(p - v3(2.6f, 1.0f, 0.0f), v3(0.5f, 0.5f, 0.5f), 0.03f), 6.0f);
    case WT_KIND_WING: return v2(sd_wing(p, v2(1.6f, 1.2f), 1.8f, -S.s.aoa, 0.24f, -1.25f, 1.25f), 6.0f);
    case WT_KIND_W17: return S.car.body ? sd_w17(S, p) : v2(1e3f, 0.0f);
    case WT_KIND_BOX:
      return v2(sd_box(p - v3(S.s.box_center[0], S.s.box_center[1], S.s.box_center[2]),
                       v3(S.s.box_half[0], S.s.box_half[1], S.s.box_half[2])), 6.0f);
    default: return v2(1e3f, 0.0f);
  }
}

// Shape plus its shape-wide constants.
Scene make_scene(const wt_shape& shape, const CarView& car = CarView{}) {
  Scene S;
  S.s = shape;
  S.car = car;
  // Shape-wide constants, evaluated once (same functions and operation order as per cell).
  const float th = wtm::atanf((shape.rear_ride - shape.ride_h) / (RA26 - FA));
  S.rake_c = wtm::cosf(th);
  S.rake_s = wtm::sinf(th);
  // Rear-wing variant parameters (f1.ts:260-272).
  const float vr = shape.rear_wing + 0.5f;
  const uint32_t v = (vr == vr && vr > 0.0f) ? (vr >= 4294967296.0f ? 4294967295u : (uint32_t)vr) : 0u;
  S.chord_m = 0.36f; S.ang_m = shape.rear_main; S.rise_m = -0.10f;
  S.chord_f = 0.26f; S.ang_f = shape.rear_flap; S.ep_hx = 0.33f; S.ep_hy = 0.29f;
  if (v == 1u) {
    S.chord_m = 0.42f; S.ang_m = S.ang_m + 3.0f * DEG; S.rise_m = -0.15f;
    S.chord_f = 0.32f; S.ang_f = S.ang_f + 6.0f * DEG; S.ep_hx = 0.36f; S.ep_hy = 0.33f;
  } else if (v == 2u) {
    S.chord_m = 0.27f; S.ang_m = S.ang_m - 5.0f * DEG; S.rise_m = 0.02f;
    S.chord_f = 0.15f; S.ang_f = S.ang_f * 0.55f; S.ep_hx = 0.30f; S.ep_hy = 0.25f;
  }
  S.rear_c = wtm::cosf(S.ang_m);
  S.rear_s = wtm::sinf(S.ang_m);
  return S;
}

}  // namespace
}  // namespace wt
