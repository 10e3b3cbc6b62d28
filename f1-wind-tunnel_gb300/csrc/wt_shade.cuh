// The RENDER fragment shader of the reference (src/engine/render-wgsl.ts:36-398,
// with the COLORMAPS chunk src/engine/wgsl.ts:369-428) as device functions:
// colour maps, studio lighting, ray march, soft shadow, ambient occlusion,
// materials and liveries, and render_pixel, the whole fs_main for one pixel.
// Arithmetic follows the WGSL text operation for operation and the WGSL
// builtin definitions (wt_vec.cuh); sin, atan2, exp and pow are the project's
// functions (wt_fmath.h).  Units that include this are built with -fmad=false;
// the result is bit-identical to the reference's shader run on the CPU.
#pragma once
#include "wt_fieldfn.cuh"
#include "wt_render.h"
#include "wt_scene.cuh"

namespace wt {
namespace {


constexpr float FAR = 6.0e4f;
constexpr float PI_F = 3.14159265f;

// ---------------------------------------------------------------- vector helpers
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V2 operator*(V2 a, V2 b) { return v2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ V2 operator/(V2 a, float s) { return v2(a.x / s, a.y / s); }
__device__ __forceinline__ V2 operator/(V2 a, V2 b) { return v2(a.x / b.x, a.y / b.y); }
__device__ __forceinline__ V3 vmin3(V3 a, V3 b) { return v3(mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)); }
__device__ __forceinline__ V3 vmax3(V3 a, V3 b) { return v3(mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)); }
__device__ __forceinline__ V3 vclamp3(V3 e, V3 lo, V3 hi) { return vmin3(vmax3(e, lo), hi); }
__device__ __forceinline__ V3 vmix3(V3 a, V3 b, float t) { return v3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
__device__ __forceinline__ V3 vabs3(V3 a) { return v3(ab(a.x), ab(a.y), ab(a.z)); }
__device__ __forceinline__ V3 nrm3(V3 a) {
  const float l = len3(a);
  return v3(a.x / l, a.y / l, a.z / l);
}
// reflect(e1, e2) = e1 - 2 dot(e2, e1) e2
__device__ __forceinline__ V3 reflect3(V3 e1, V3 e2) { return e1 - (2.0f * dot3(e2, e1)) * e2; }
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
// an RGBA binary16 texel
__device__ __forceinline__ float4 h4(ushort4 v) {
  return make_float4(__half2float(__ushort_as_half(v.x)), __half2float(__ushort_as_half(v.y)),
                     __half2float(__ushort_as_half(v.z)), __half2float(__ushort_as_half(v.w)));
}
__device__ __forceinline__ float stepf(float edge, float x) { return edge <= x ? 1.0f : 0.0f; }
__device__ __forceinline__ V3 c3(const F3& f) { return v3(f.x, f.y, f.z); }
__device__ __forceinline__ uint32_t mn_u(uint32_t a, uint32_t b) { return b < a ? b : a; }
__device__ __forceinline__ V3 tolinear(V3 c) { return v3(wtm::powf(c.x, 2.2f), wtm::powf(c.y, 2.2f), wtm::powf(c.z, 2.2f)); }

// ---------------------------------------------------------------- colour maps (wgsl.ts:369-428)
__device__ V3 turbo(float t0) {
  const float x = clmp(t0, 0.0f, 1.0f);
  const float p0 = 1.0f, p1 = x, p2 = x * x, p3 = x * x * x;
  const float q0 = p2 * p2, q1 = p3 * p2;
  const float r = (p0 * 0.13572138f + p1 * 4.61539260f + p2 * -42.66032258f + p3 * 132.13108234f) +
                  (q0 * -152.94239396f + q1 * 59.28637943f);
  const float g = (p0 * 0.09140261f + p1 * 2.19418839f + p2 * 4.84296658f + p3 * -14.18503333f) +
                  (q0 * 4.27729857f + q1 * 2.82956604f);
  const float b = (p0 * 0.10667330f + p1 * 12.64194608f + p2 * -60.58204836f + p3 * 110.36276771f) +
                  (q0 * -89.90310912f + q1 * 27.34824973f);
  return vclamp3(v3(r, g, b), v3(0.0f, 0.0f, 0.0f), v3(1.0f, 1.0f, 1.0f));
}
__device__ V3 inferno(float t0) {
  const float t = clmp(t0, 0.0f, 1.0f);
  const V3 c0 = v3(0.0002189f, 0.0016510f, -0.0194809f), c1 = v3(0.1065134f, 0.5639564f, 3.9327124f),
           c2 = v3(11.6024931f, -3.9728540f, -15.9423941f), c3 = v3(-41.7039961f, 17.4363989f, 44.3541452f),
           c4 = v3(77.1629357f, -33.4023589f, -81.8073093f), c5 = v3(-71.3194282f, 32.6260643f, 73.2095199f),
           c6 = v3(25.1311262f, -12.2426690f, -23.0703250f);
  const V3 r = c0 + t * (c1 + t * (c2 + t * (c3 + t * (c4 + t * (c5 + t * c6)))));
  return vclamp3(r, v3(0.0f, 0.0f, 0.0f), v3(1.0f, 1.0f, 1.0f));
}
__device__ V3 viridis_like(float t0) {
  const float t = clmp(t0, 0.0f, 1.0f);
  return vmix3(vmix3(v3(0.07f, 0.04f, 0.20f), v3(0.13f, 0.55f, 0.55f), sstep(0.0f, 0.5f, t)), v3(0.99f, 0.91f, 0.15f),
               sstep(0.45f, 1.0f, t));
}
__device__ V3 wake_map(float t0) {
  const float t = clmp(t0, 0.0f, 1.0f);
  V3 c = vmix3(v3(0.02f, 0.03f, 0.06f), v3(0.22f, 0.05f, 0.42f), sstep(0.0f, 0.25f, t));
  c = vmix3(c, v3(0.85f, 0.1f, 0.55f), sstep(0.25f, 0.55f, t));
  c = vmix3(c, v3(1.0f, 0.55f, 0.25f), sstep(0.55f, 0.8f, t));
  return vmix3(c, v3(1.0f, 0.95f, 0.7f), sstep(0.8f, 1.0f, t));
}
__device__ V3 neon(float t0) {
  const float t = clmp(t0, 0.0f, 1.0f);
  V3 c = vmix3(v3(0.01f, 0.02f, 0.08f), v3(0.02f, 0.12f, 0.45f), sstep(0.0f, 0.3f, t));
  c = vmix3(c, v3(0.03f, 0.45f, 0.95f), sstep(0.3f, 0.6f, t));
  c = vmix3(c, v3(0.25f, 0.85f, 1.0f), sstep(0.6f, 0.8f, t));
  return vmix3(c, v3(0.92f, 1.0f, 1.0f), sstep(0.8f, 1.0f, t));
}
__device__ V3 palette(uint32_t id, float t) {
  switch (id) {
    case 1u: return turbo(t * 0.86f + 0.07f);
    case 2u: return inferno(t * 0.92f + 0.04f);
    case 3u: return viridis_like(t);
    case 4u: return wake_map(t);
    default: return neon(t);
  }
}

// ---------------------------------------------------------------- scene pass
struct Mat {
  V3 albedo;
  float rough, metal, coat;
  V3 emit;
};
__device__ __forceinline__ Mat mat(V3 a, float r, float m, float c, V3 e) {
  Mat o;
  o.albedo = a; o.rough = r; o.metal = m; o.coat = c; o.emit = e;
  return o;
}
__device__ __forceinline__ V3 zero3() { return v3(0.0f, 0.0f, 0.0f); }

// studioEnv, backdrop (render-wgsl.ts:43-61)
__device__ V3 studio_env(V3 d) {
  V3 c = v3(0.004f, 0.005f, 0.007f) + v3(0.018f, 0.020f, 0.025f) * sstep(-0.05f, 0.5f, d.y);
  if (d.y > 0.08f) {
    const float u = d.z / d.y;
    const float v = d.x / d.y;
    float box = 0.0f;
    for (int i = -1; i <= 1; i++) box = box + sstep(0.17f, 0.12f, ab(u - (float)i * 0.75f));
    box = box * sstep(1.9f, 1.6f, ab(v - 0.3f));
    c = c + v3(2.4f, 2.45f, 2.6f) * box * sstep(0.08f, 0.35f, d.y);
  }
  const float rim = sstep(0.80f, 0.95f, d.x) * sstep(0.35f, 0.05f, ab(d.y - 0.18f));
  return c + v3(0.9f, 1.0f, 1.15f) * rim;
}
__device__ V3 backdrop(V3 rd) { return v3(0.006f, 0.007f, 0.010f) + v3(0.010f, 0.012f, 0.016f) * sstep(-0.2f, 0.6f, rd.y); }

// boxHit (render-wgsl.ts:62-67)
__device__ V2 box_hit(V3 ro, V3 rd, V3 bmin, V3 bmax) {
  const V3 inv = v3(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
  const V3 t0 = (bmin - ro) * inv, t1 = (bmax - ro) * inv;
  const V3 tn = vmin3(t0, t1), tf = vmax3(t0, t1);
  return v2(mx(mx(tn.x, tn.y), tn.z), mn(mn(tf.x, tf.y), tf.z));
}

// One out-of-line copy of the scene SDF for the whole pass: the ray march,
// normal, occlusion, shadow and reflection taps all call it, and inlining it
// at each site multiplies the code past the instruction cache.
__device__ __noinline__ V2 sdf(const Scene& S, V3 p) { return scene_sdf(S, p); }


// march (render-wgsl.ts:68-79)
__device__ __noinline__ V2 march(const Scene& S, const SceneArgs& a, V3 ro, V3 rd, int max_steps) {
  const V2 tb = box_hit(ro, rd, c3(a.bmin), c3(a.bmax));
  if (tb.x > tb.y || tb.y < 0.0f) return v2(FAR, 0.0f);
  float t = mx(tb.x, 0.0f);
  for (int i = 0; i < max_steps; i++) {
    const V2 r = sdf(S, ro + rd * t);
    if (r.x < 0.0004f * t + 0.0003f) return v2(t, r.y);
    t = t + r.x * 0.9f;
    if (t > tb.y) break;
  }
  return v2(FAR, 0.0f);
}
// calcNormal (render-wgsl.ts:80-83): e = (1, -1) * 0.0008
__device__ V3 calc_normal(const Scene& S, const SceneArgs& a, V3 p) {
  const float ex = 0.0008f, ey = -0.0008f;
  const V3 xyy = v3(ex, ey, ey), yyx = v3(ey, ey, ex), yxy = v3(ey, ex, ey), xxx = v3(ex, ex, ex);
  const V3 s = xyy * sdf(S, p + xyy).x + yyx * sdf(S, p + yyx).x + yxy * sdf(S, p + yxy).x +
               xxx * sdf(S, p + xxx).x;
  return nrm3(s);
}
// ambientOcc (render-wgsl.ts:84-93)
__device__ float ambient_occ(const Scene& S, const SceneArgs& a, V3 p, V3 n) {
  float occ = 0.0f, sca = 1.0f;
  for (int i = 1; i <= 5; i++) {
    const float hh = 0.012f + 0.03f * (float)i;
    occ = occ + (hh - sdf(S, p + n * hh).x) * sca;
    sca = sca * 0.75f;
  }
  return clmp(1.0f - 2.2f * occ, 0.0f, 1.0f);
}
// softShadow (render-wgsl.ts:94-107)
__device__ float soft_shadow(const Scene& S, const SceneArgs& a, V3 ro, V3 rd) {
  const V2 tb = box_hit(ro, rd, c3(a.bmin), c3(a.bmax));
  if (tb.x > tb.y || tb.y < 0.0f) return 1.0f;
  float t = mx(tb.x, 0.01f);
  float res = 1.0f;
  for (int i = 0; i < 48; i++) {
    const float hh = sdf(S, ro + rd * t).x;
    res = mn(res, 12.0f * hh / t);
    if (res < 0.01f || t > tb.y) break;
    t = t + clmp(hh, 0.01f, 0.2f);
  }
  return clmp(res, 0.0f, 1.0f);
}

// carbonWeave, carbonMat, paintMat, hash2, glossBlack (render-wgsl.ts:111-129)
__device__ float carbon_weave(V3 p, V3 n, float view_dist) {
  const V3 an = vabs3(n);
  V2 uv = v2(p.x, p.y);
  if (an.x > an.y && an.x > an.z) uv = v2(p.y, p.z);
  else if (an.y > an.z) uv = v2(p.x, p.z);
  const V2 g = uv * 75.0f;
  const V2 cell = v2(floorf(g.x), floorf(g.y));
  const V2 f = v2(fractf(g.x), fractf(g.y));
  const bool twill = (to_i32(cell.x + cell.y * 2.0f) & 3) < 2;
  const float s = twill ? f.x : f.y;
  const float detail = clmp(1.6f - view_dist * 0.22f, 0.0f, 1.0f);
  return 0.8f + (0.42f * wtm::sinf(s * PI_F) * (twill ? 1.0f : 0.8f) - 0.08f) * detail;
}
__device__ Mat carbon_mat(V3 p, V3 n, float vd) {
  return mat(v3(0.028f, 0.029f, 0.032f) * carbon_weave(p, n, vd), 0.28f, 0.0f, 0.9f, zero3());
}
__device__ __forceinline__ Mat paint_mat(V3 c) { return mat(c, 0.22f, 0.0f, 1.0f, zero3()); }
__device__ __forceinline__ float hash2(V2 c) { return fractf(wtm::sinf(c.x * 127.1f + c.y * 311.7f) * 43758.5453f); }
__device__ __forceinline__ Mat gloss_black() { return mat(v3(0.009f, 0.0095f, 0.011f), 0.14f, 0.0f, 1.0f, zero3()); }

// noseTipY, noseStartX (src/engine/f1.ts:134-135); endplate tops (f1.ts:215-223)
__device__ __forceinline__ float nose_tip_y(const Scene& S, float b) { return b + (variant(S.s.nose) == 2u ? 0.25f : 0.17f); }
__device__ __forceinline__ float nose_start_x(const Scene& S) { return variant(S.s.nose) == 1u ? 0.34f : 0.10f; }
__device__ __forceinline__ float rear_endplate_top(const Scene& S) {
  const uint32_t k = mn_u(variant(S.s.rear_wing), 2u);
  return k == 0u ? 1.06f : (k == 1u ? 1.10f : 1.02f);
}
__device__ __forceinline__ float front_endplate_top(const Scene& S) {
  const uint32_t k = mn_u(variant(S.s.front_wing), 3u);
  return k == 0u ? 0.20f : (k == 1u ? 0.37f : (k == 2u ? 0.16f : 0.135f));
}

// bodyAxisY, sparkleField, liveryBody (render-wgsl.ts:130-159)
__device__ float body_axis_y(const Scene& S, float x, float b) {
  if (x < 1.26f) return mixf(nose_tip_y(S, b), b + 0.36f, clmp((x - nose_start_x(S)) / (1.26f - nose_start_x(S)), 0.0f, 1.0f));
  return b + mixf(0.36f, 0.42f, clmp((x - 1.26f) / 0.98f, 0.0f, 1.0f));
}
__device__ float sparkle_field(V3 p, float b) {
  const V2 uv = v2(p.x * 10.0f, (p.y - b) * 10.0f + p.z * 7.0f);
  const V2 cell = v2(floorf(uv.x), floorf(uv.y));
  const float r = hash2(cell);
  const V2 hv = v2(hash2(v2(cell.x + 7.3f, cell.y + 7.3f)), hash2(v2(cell.x + 3.1f, cell.y + 3.1f)));
  const V2 f = (v2(fractf(uv.x), fractf(uv.y)) - v2(0.5f, 0.5f)) - (hv - v2(0.5f, 0.5f)) * 0.4f;
  const float size = mixf(0.55f, 0.06f, sstep(3.1f, 4.5f, p.x)) * stepf(0.25f, r);
  const float star = ab(f.x) * ab(f.y) * 30.0f + (ab(f.x) + ab(f.y)) * 0.6f;
  return 1.0f - sstep(size * 0.8f, size, star);
}
__device__ Mat livery_body(const Scene& S, V3 p, float b, V3 silver, V3 teal) {
  if (p.z > 0.5f && p.x < 2.5f && p.y > b + 0.6f) return paint_mat(teal);
  const float cy = body_axis_y(S, p.x, b);
  const bool on_chassis = p.x < 2.75f && p.z < 0.33f && p.y < b + 0.62f;
  const float edge = cy - 0.015f + 0.03f * sstep(0.4f, 2.4f, p.x);
  if (on_chassis && p.x > 0.35f && ab(p.y - edge) < mixf(0.010f, 0.016f, sstep(0.5f, 2.0f, p.x))) return paint_mat(teal);
  if (on_chassis && p.y > edge && p.x < 2.62f - (p.y - b - 0.42f) * 0.6f) return mat(silver, 0.38f, 0.35f, 0.8f, zero3());
  if (p.z > 0.2f && p.x > 2.35f && p.x < 4.4f) {
    const float t = clmp((p.x - 2.35f) / 2.05f, 0.0f, 1.0f);
    const float line = b + 0.53f - 0.15f * (p.x - 2.45f);
    if (ab(p.y - line) < mixf(0.04f, 0.007f, t)) return paint_mat(teal);
  }
  const bool on_cover = p.x > 3.05f && p.x < 4.7f && p.y > b + 0.42f && p.z < 0.32f;
  if (on_cover && sparkle_field(p, b) > 0.5f) return mat(silver, 0.38f, 0.35f, 0.8f, zero3());
  return gloss_black();
}

// louvres (render-wgsl.ts:160-178): cooling slots painted onto the mesh's bodywork.
__device__ Mat louvres(const SceneArgs& a, V3 p, V3 n, const Mat mt) {
  if (a.cooling == 0u) return mt;
  const bool open = a.cooling == 2u;
  const float az = ab(p.z);
  float slot = 0.0f;
  const float x0 = open ? 3.05f : 3.35f;
  const float x1 = open ? 3.95f : 3.85f;
  if (p.x > x0 && p.x < x1 && az > 0.16f && az < 0.48f && p.y > 0.45f && n.y > 0.55f) {
    const float f = fractf(p.x / 0.045f);
    slot = ((open ? 0.55f : 0.32f) >= f ? 1.0f : 0.0f) * sstep(0.16f, 0.2f, az) * (1.0f - sstep(0.44f, 0.48f, az));
  }
  if (open && p.x > 3.6f && p.x < 4.25f && az > 0.08f && az < 0.32f && p.y > 0.5f && p.y < 0.8f && ab(n.z) > 0.5f) {
    slot = mx(slot, (0.4f >= fractf(p.x / 0.05f) ? 1.0f : 0.0f) * sstep(0.52f, 0.56f, p.y) *
                        (1.0f - sstep(0.74f, 0.78f, p.y)));
  }
  if (slot <= 0.0f) return mt;
  return mat(vmix3(mt.albedo, v3(0.004f, 0.004f, 0.004f), slot), mixf(mt.rough, 0.9f, slot), mt.metal * (1.0f - slot),
             mt.coat * (1.0f - slot), mt.emit);
}

// materialAt (render-wgsl.ts:180-255).  With the baked mesh (meshMode) only
// reflections reach it past the wings: a neutral dark body stands in.
__device__ __noinline__ Mat material_at(const Scene& S, const SceneArgs& a, float m, V3 pw, V3 n, float vd) {
  const V3 pabs = v3(pw.x, pw.y, ab(pw.z));
  const V3 p = a.is_f1 != 0u ? body_frame(S, pabs) : pabs;
  const float b = S.s.ride_h;
  const V3 accent = c3(a.accent_lin);
  const V3 paint = c3(a.paint_lin);
  if (m < 0.5f) {
    if (a.is_f1 != 0u) return livery_body(S, p, b, paint, accent);
    if (a.carbon_body != 0u) return carbon_mat(p, n, vd);
    return paint_mat(paint);
  }
  if (m < 1.5f) return carbon_mat(p, n, vd);
  if (m < 2.5f) {
    const bool front = pabs.x < 2.7f;
    const V3 wc = front ? v3(FA, WR26, FWZ * BODY_Z) : v3(RA26, WR26, RWZ * BODY_Z);
    const float hw = front ? FHW26 : RHW26;
    const V3 q = pabs - wc;
    const float r = len2(v2(q.x, q.y));
    const float ang = wtm::atan2f(q.y, q.x);
    V3 alb = v3(0.016f, 0.016f, 0.018f);
    if (ab(q.z) > hw - 0.05f) {
      const float aa = fractf(ang / (2.0f * PI_F) * 2.0f);
      const bool word = fractf(aa * 7.0f) < 0.62f && (aa < 0.42f || (aa > 0.5f && aa < 0.92f));
      if (r > 0.291f && r < 0.313f && word) alb = v3(0.24f, 0.245f, 0.25f);
      if (r > 0.321f && r < 0.326f) alb = v3(0.05f, 0.05f, 0.05f);
    }
    return mat(alb, 0.82f, 0.0f, 0.0f, zero3());
  }
  if (m < 3.5f) {
    const V3 q = p - v3(2.67f, b + 0.71f, 0.0f);
    if (p.x < 2.62f && q.y > -0.028f && q.y < 0.03f) {
      const float shift = sstep(-0.5f, 0.6f, n.y * 1.5f + q.z * 5.0f);
      const V3 tint = vmix3(vmix3(v3(0.05f, 0.75f, 0.95f), v3(0.15f, 0.25f, 1.0f), sstep(0.0f, 0.5f, shift)),
                            v3(0.65f, 0.15f, 0.85f), sstep(0.5f, 1.0f, shift));
      return mat(tint, 0.05f, 1.0f, 1.0f, tint * 0.22f);
    }
    if ((ab(q.y + 0.032f) < 0.005f || ab(q.y - 0.034f) < 0.005f) && p.x < 2.63f) return paint_mat(v3(0.02f, 0.02f, 0.02f));
    V3 alb = v3(0.06f, 0.48f, 0.80f);
    const float swoosh = q.y * 0.9f - q.x * 0.55f;
    if (q.y < -0.07f) alb = v3(0.012f, 0.014f, 0.02f);
    else if (ab(swoosh + 0.015f) < 0.018f && q.x > -0.04f) alb = v3(0.01f, 0.03f, 0.09f);
    else if (ab(swoosh + 0.04f) < 0.005f && q.x > -0.02f) alb = accent;
    if (q.y > 0.08f && p.z < 0.022f) alb = v3(0.01f, 0.03f, 0.09f);
    if (q.y > 0.08f && ab(p.z - 0.026f) < 0.004f) alb = accent;
    return mat(alb, 0.16f, 0.0f, 1.0f, zero3());
  }
  if (m < 4.5f) return mat(v3(0.05f, 0.05f, 0.055f), 0.35f, 0.3f, 0.6f, zero3());
  if (m < 6.5f) return mat(v3(0.55f, 0.57f, 0.60f), 0.35f, 0.0f, 0.6f, zero3());
  if (m < 7.5f) {
    const float yw = 0.19f + b * 0.45f;
    const float end_z = 0.94f - 0.01f;
    if (p.z > end_z && p.y > yw + front_endplate_top(S) - 0.035f) return paint_mat(accent);
    if (p.z > end_z) return gloss_black();
    return carbon_mat(p, n, vd);
  }
  if (m < 8.5f) {
    if (p.z > 0.495f && p.y > b + rear_endplate_top(S) - 0.06f) return paint_mat(accent);
    return carbon_mat(p, n, vd);
  }
  if (a.mesh_mode != 0u) return mat(v3(0.02f, 0.021f, 0.024f), 0.3f, 0.0f, 0.8f, zero3());
  if (m > 11.5f) return mat(v3(0.02f, 0.021f, 0.024f), 0.3f, 0.0f, 0.8f, zero3());
  if (m < 9.5f && m > 8.5f) {
    const bool front = pabs.x < 2.7f;
    const V3 wc = front ? v3(FA, WR26, FWZ * BODY_Z) : v3(RA26, WR26, RWZ * BODY_Z);
    const V3 q = pabs - wc;
    const float spokes = 0.75f + 0.25f * sstep(0.2f, 0.8f, ab(wtm::sinf(wtm::atan2f(q.y, q.x) * 5.0f)));
    if (len2(v2(q.x, q.y)) < 0.05f) return mat(v3(0.035f, 0.036f, 0.04f), 0.3f, 0.8f, 0.5f, zero3());
    return mat(v3(0.07f, 0.072f, 0.08f) * spokes, 0.32f, 0.8f, 0.4f, zero3());
  }
  if (m < 10.5f) {
    const V3 tint = vmix3(v3(0.55f, 0.42f, 0.25f), v3(0.25f, 0.30f, 0.55f), sstep(4.98f, 5.12f, p.x));
    return mat(tint, 0.3f, 1.0f, 0.0f, zero3());
  }
  return mat(v3(0.3f, 0.0f, 0.0f), 0.2f, 0.0f, 1.0f, v3(4.0f, 0.12f, 0.08f));
}

// shadeSurface (render-wgsl.ts:257-283)
__device__ __noinline__ V3 shade_surface(const Scene& S, const SceneArgs& a, V3 p, V3 n, V3 rd, const Mat mt, bool fast) {
  const V3 key = c3(a.key);
  float sh = 1.0f, ao = 1.0f;
  const float lift = a.mesh_mode != 0u ? 0.045f : 0.004f;
  if (!fast) {
    sh = soft_shadow(S, a, p + n * lift, key);
    ao = ambient_occ(S, a, p + n * (lift - 0.004f), n);
  }
  const float ndl = mx(dot3(n, key), 0.0f);
  const float fill = mx(dot3(n, c3(a.fill_a)), 0.0f) * 0.18f + mx(dot3(n, c3(a.fill_b)), 0.0f) * 0.18f;
  const float amb = (0.45f + 0.55f * n.y) * 0.22f * ao;
  const V3 h = nrm3(key - rd);
  const float rough = mt.rough;
  const float shin = mixf(12.0f, 900.0f, (1.0f - rough) * (1.0f - rough));
  const V3 f0 = vmix3(v3(0.04f, 0.04f, 0.04f), mt.albedo, mt.metal);
  const float nv = mx(dot3(n, -rd), 0.0f);
  const float p5 = wtm::powf(1.0f - nv, 5.0f);
  const V3 fres = f0 + (v3(1.0f, 1.0f, 1.0f) - f0) * p5;
  const float spec = wtm::powf(mx(dot3(n, h), 0.0f), shin) * (shin + 8.0f) / (8.0f * PI_F);
  const V3 diffuse = mt.albedo * (1.0f - mt.metal);
  const V3 refl = reflect3(rd, n);
  const V3 env = studio_env(refl);
  V3 col = diffuse * (ndl * sh * 2.4f + fill + amb);
  col = col + fres * spec * ndl * sh * 1.6f * (1.0f - rough * 0.6f);
  col = col + env * fres * ao * mixf(1.0f - rough, 1.0f, mt.metal) * 0.9f;
  const float coat_f = 0.04f + 0.96f * p5;
  col = col + env * coat_f * mt.coat * ao * 0.8f;
  return col + mt.emit;
}

// RENDER fs_main (render-wgsl.ts:288-398) for pixel (x, y): colour and hit distance.
// MESH: look.meshMode != 0 (a separate instantiation, so the analytic scenes'
// kernel carries none of the G-buffer code: the pass is bound by instruction
// supply).
template <bool MESH>
__device__ float4 render_pixel(const Scene& S, const SceneArgs& a, uint32_t x, uint32_t y) {
  const float ux = ((float)x + 0.5f) / (float)a.w, uy = ((float)y + 0.5f) / (float)a.h;
  const float ndx = (ux * 2.0f - 1.0f) + a.jitter_x, ndy = (1.0f - uy * 2.0f) + a.jitter_y;
  const V3 rd = nrm3(c3(a.fwd) + ndx * a.tan_half * a.aspect * c3(a.right) + ndy * a.tan_half * c3(a.up));
  const V3 ro = c3(a.pos);
  const V3 key = c3(a.key);

  V3 col = backdrop(rd);
  float t_hit = FAR;
  V2 hit = v2(FAR, 0.0f);
  float4 gn = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ga = gn, gm = gn;
  if constexpr (MESH) {
    // the G-buffer texel under the pixel (it has the scene's size)
    const int gx0 = to_i32(ux * (float)a.w), gy0 = to_i32(uy * (float)a.h);
    const int gx = gx0 < 0 ? 0 : (gx0 > (int)a.w - 1 ? (int)a.w - 1 : gx0);
    const int gy = gy0 < 0 ? 0 : (gy0 > (int)a.h - 1 ? (int)a.h - 1 : gy0);
    const size_t gi = (size_t)gy * a.w + (size_t)gx;
    gn = h4(a.g_normal[gi]);
    if (gn.w > 0.0f) {
      hit = v2(gn.w, 12.0f);
      ga = h4(a.g_albedo[gi]);
      const uchar4 m8 = a.g_material[gi];
      gm = make_float4((float)m8.x / 255.0f, (float)m8.y / 255.0f, (float)m8.z / 255.0f, (float)m8.w / 255.0f);
    }
  } else {
    hit = march(S, a, ro, rd, 220);
  }
  float t_ground = FAR;
  if (rd.y < -1e-4f) t_ground = -ro.y / rd.y;

  if (hit.x < t_ground && hit.x < FAR) {
    const V3 p = ro + rd * hit.x;
    const float vd = hit.x;
    V3 n;
    Mat mt;
    if constexpr (MESH) {
      n = nrm3(v3(gn.x, gn.y, gn.z));
      if (dot3(n, rd) > 0.0f) n = -n;
      const V3 alb = v3(ga.x, ga.y, ga.z);
      mt = louvres(a, p, n, mat(alb, ga.w, gm.x, gm.y, alb * gm.z));
    } else {
      n = calc_normal(S, a, p);
      mt = material_at(S, a, hit.y, p, n, vd);
    }
    if (a.surf_mode == 1u) {
      V3 probe = p + n * a.g.h * 0.8f;
      Sample s = sample_flow(a.g, probe);
      for (int k = 0; k < 4 && s.fluid <= 0.0f; k++) {
        probe = probe + n * a.g.h;
        s = sample_flow(a.g, probe);
      }
      if (s.fluid > 0.0f) {
        const float v = clmp(field_value(a.g, a.view, a.palette, s, probe), 0.0f, 1.0f);
        const float iso = 1.0f - 0.18f * (1.0f - sstep(0.0f, 0.035f, ab(fractf(v * 14.0f) - 0.5f) - 0.44f));
        mt = mat(tolinear(palette(a.palette, v)) * iso, 0.55f, 0.0f, 0.25f, zero3());
      }
    }
    col = shade_surface(S, a, p, n, rd, mt, false);
    t_hit = hit.x;
  } else if (t_ground < FAR) {
    const V3 p = ro + rd * t_ground;
    const V3 up = v3(0.0f, 1.0f, 0.0f);
    const float pool = wtm::expf(-((p.x - 2.8f) * (p.x - 2.8f)) / 14.0f - (p.z * p.z) / 5.0f);
    V3 gc = v3(0.006f, 0.0065f, 0.008f) + v3(0.030f, 0.032f, 0.038f) * pool;
    const bool belt = ab(p.z) < 1.15f && p.x > -0.6f && p.x < 6.2f;
    if (belt) {
      const float stripe = fractf((p.x - a.time * a.road_speed) * 1.2f);
      gc = gc * 0.75f + v3(0.006f, 0.006f, 0.006f) * sstep(0.0f, 0.08f, stripe) * sstep(0.2f, 0.12f, stripe);
      gc = gc + v3(0.05f, 0.05f, 0.055f) * (1.0f - sstep(0.0f, 0.012f, ab(ab(p.z) - 1.15f))) * pool;
    }
    const float sh = soft_shadow(S, a, p + up * 0.005f, key);
    const float ao = clmp(sdf(S, p).x * 2.6f + 0.12f, 0.0f, 1.0f);
    col = gc * (0.35f + 0.65f * sh) * mixf(0.25f, 1.0f, ao);
    const V3 rdir = reflect3(rd, up);
    const float fres = 0.02f + 0.22f * wtm::powf(1.0f - ab(rd.y), 5.0f);
    V3 refl = studio_env(rdir) * 0.35f;
    const V2 rh = march(S, a, p + up * 0.002f, rdir, 90);
    if (rh.x < FAR) {
      const V3 rp = p + rdir * rh.x;
      const V3 rn = calc_normal(S, a, rp);
      const float vd = t_ground + rh.x;
      refl = shade_surface(S, a, rp, rn, rdir, material_at(S, a, rh.y, rp, rn, vd), true) * wtm::expf(-rh.x * 2.2f);
    }
    col = col + refl * fres * ao;
    const float fog_t = 1.0f - wtm::expf(-t_ground * 0.03f);
    col = vmix3(col, backdrop(rd), fog_t);
    t_hit = t_ground;
  }

  if (a.slice_axis > 0u && a.show_flow != 0u) {
    const uint32_t axis = a.slice_axis - 1u;
    const float rda = axis == 0u ? rd.x : (axis == 1u ? rd.y : rd.z);
    const float roa = axis == 0u ? ro.x : (axis == 1u ? ro.y : ro.z);
    if (ab(rda) > 1e-5f) {
      const float ts = (a.slice_pos - roa) / rda;
      if (ts > 0.0f && ts < t_hit) {
        const V3 p = ro + rd * ts;
        const V3 dmin = v3(a.g.ox, 0.0f, -(a.g.oz + (float)a.g.nz * a.g.h));
        const V3 dmax = v3(a.g.ox + (float)a.g.nx * a.g.h, a.g.oy + (float)a.g.ny * a.g.h, a.g.oz + (float)a.g.nz * a.g.h);
        const V3 lo = vmax3(dmin, v3(-1.5f, 0.0f, -2.2f)), hi = vmin3(dmax, v3(8.5f, 2.6f, 2.2f));
        if (p.x >= lo.x && p.y >= lo.y && p.z >= lo.z && p.x <= hi.x && p.y <= hi.y && p.z <= hi.z) {
          const Sample s = sample_flow(a.g, p);
          if (s.fluid > 0.05f) {
            const float v = clmp(field_value(a.g, a.view, a.palette, s, p), 0.0f, 1.0f);
            const V3 cc = tolinear(palette(a.palette, v));
            const float iso = ab(fractf(v * 12.0f) - 0.5f);
            const float contour = 1.0f - sstep(0.0f, 0.06f, iso) * 0.2f;
            col = vmix3(col, cc * 0.8f * contour, a.slice_alpha);
            t_hit = ts;
          }
        }
      }
    }
  }
  return make_float4(col.x, col.y, col.z, mn(t_hit, FAR));
}

}  // namespace
}  // namespace wt
