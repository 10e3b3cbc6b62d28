// The reference's analytic signed-distance scenes on the device
// (src/engine/wgsl.ts:20-76,101-116 primitives and scene switch;
// src/engine/f1.ts:20-320 generic F1, :397-407 heat emission), shared by the
// voxelizer and the renderer.  Every float operation keeps the reference's
// order (units built with -fmad=false); sin, cos and atan are the project's
// functions (wt_fmath.h).  Shape-wide values (rake rotation, rear main-plane
// direction) are computed once on the host by make_scene with the same
// functions, which gives the same bits as evaluating them per point.
#pragma once
#include "wt_fmath.h"
#include "wt_internal.h"
#include "wt_vec.cuh"

namespace wt {
namespace {

// Shape plus host-computed shape-wide constants.
struct Scene {
  wt_shape s;
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
__device__ V2 scene_sdf(const Scene& S, V3 p) {
  switch (S.s.kind) {
    case WT_KIND_F1: return sd_f1(S, p);
    case WT_KIND_SPHERE: return v2(len3(p - v3(2.6f, 1.0f, 0.0f)) - 0.6f, 6.0f);
    case WT_KIND_CUBE: return v2(sd_rbox(p - v3(2.6f, 1.0f, 0.0f), v3(0.5f, 0.5f, 0.5f), 0.03f), 6.0f);
    case WT_KIND_WING: return v2(sd_wing(p, v2(1.6f, 1.2f), 1.8f, -S.s.aoa, 0.24f, -1.25f, 1.25f), 6.0f);
    case WT_KIND_BOX:
      return v2(sd_box(p - v3(S.s.box_center[0], S.s.box_center[1], S.s.box_center[2]),
                       v3(S.s.box_half[0], S.s.box_half[1], S.s.box_half[2])), 6.0f);
    default: return v2(1e3f, 0.0f);
  }
}

// Shape plus its shape-wide constants.
Scene make_scene(const wt_shape& shape) {
  Scene S;
  S.s = shape;
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
