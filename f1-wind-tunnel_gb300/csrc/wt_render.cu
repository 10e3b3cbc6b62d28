// The reference's render passes as CUDA kernels into headless render targets
// (src/engine/render-wgsl.ts; targets and pass order src/engine/engine.ts:290-327,
// 714-725):
//   scene pass    RENDER fs_main (render-wgsl.ts:288-398): ray march of the scene
//                 SDF, materials, studio lighting, ground reflection, flow slice
//   TAA resolve   TAA fs_main (render-wgsl.ts:456-518)
//   glow pass     PARTICLES_DRAW (src/engine/wgsl.ts:597-659) and STREAM_DRAW
//                 (render-wgsl.ts:578-645) quads, rasterized and added up
//   bloom         BLUR fs_main (render-wgsl.ts:401-418), horizontal then vertical
//   present       PRESENT fs_main (render-wgsl.ts:420-454) into RGBA8
// Each full-screen pass runs one thread per texel of its target with
// uv = ((x + 0.5) / w, (y + 0.5) / h).  Float targets are binary16 RGBA, written
// with round-to-nearest-even as the GPU stores rgba16float.
//
// Arithmetic follows the WGSL text operation for operation and the WGSL builtin
// definitions (wt_vec.cuh); sin, atan2, exp and pow are the project's functions
// (wt_fmath.h), shared with the CPU model.  Built with -fmad=false, so every
// target matches the reference's shaders run on the CPU bit for bit.
//
// The glow pass rasterizes each quad as two triangles with the fixed-function
// rules of the WebGPU pipeline written out (viewport transform, edge functions
// with a tie rule that draws a pixel on a shared edge once, depth clip,
// perspective-correct varyings).  Additive blending is evaluated as an exact sum:
// each fragment's value is rounded to a multiple of 2^-32 and added into 64-bit
// integers with atomics, then the total is rounded once to binary16.  The result
// does not depend on fragment order, so the kernel is deterministic.
#include <cuda_fp16.h>

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
__device__ __forceinline__ float stepf(float edge, float x) { return edge <= x ? 1.0f : 0.0f; }
__device__ __forceinline__ V3 c3(const F3& f) { return v3(f.x, f.y, f.z); }
__device__ __forceinline__ uint32_t mn_u(uint32_t a, uint32_t b) { return b < a ? b : a; }
__device__ __forceinline__ float h2f(unsigned short u) { return __half2float(__ushort_as_half(u)); }
__device__ __forceinline__ unsigned short f2h(float x) { return __half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ float4 load_tex(const ushort4* t, uint32_t w, int x, int y) {
  const ushort4 v = t[(size_t)y * w + (size_t)x];
  return make_float4(h2f(v.x), h2f(v.y), h2f(v.z), h2f(v.w));
}
__device__ __forceinline__ ushort4 pack(float r, float g, float b, float a) {
  ushort4 o;
  o.x = f2h(r); o.y = f2h(g); o.z = f2h(b); o.w = f2h(a);
  return o;
}
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

struct Ctx {
  const Scene& S;
  const SceneArgs& a;
};

// march (render-wgsl.ts:68-79)
__device__ V2 march(const Ctx& c, V3 ro, V3 rd, int max_steps) {
  const V2 tb = box_hit(ro, rd, c3(c.a.bmin), c3(c.a.bmax));
  if (tb.x > tb.y || tb.y < 0.0f) return v2(FAR, 0.0f);
  float t = mx(tb.x, 0.0f);
  for (int i = 0; i < max_steps; i++) {
    const V2 r = scene_sdf(c.S, ro + rd * t);
    if (r.x < 0.0004f * t + 0.0003f) return v2(t, r.y);
    t = t + r.x * 0.9f;
    if (t > tb.y) break;
  }
  return v2(FAR, 0.0f);
}
// calcNormal (render-wgsl.ts:80-83): e = (1, -1) * 0.0008
__device__ V3 calc_normal(const Ctx& c, V3 p) {
  const float ex = 0.0008f, ey = -0.0008f;
  const V3 xyy = v3(ex, ey, ey), yyx = v3(ey, ey, ex), yxy = v3(ey, ex, ey), xxx = v3(ex, ex, ex);
  const V3 s = xyy * scene_sdf(c.S, p + xyy).x + yyx * scene_sdf(c.S, p + yyx).x + yxy * scene_sdf(c.S, p + yxy).x +
               xxx * scene_sdf(c.S, p + xxx).x;
  return nrm3(s);
}
// ambientOcc (render-wgsl.ts:84-93)
__device__ float ambient_occ(const Ctx& c, V3 p, V3 n) {
  float occ = 0.0f, sca = 1.0f;
  for (int i = 1; i <= 5; i++) {
    const float hh = 0.012f + 0.03f * (float)i;
    occ = occ + (hh - scene_sdf(c.S, p + n * hh).x) * sca;
    sca = sca * 0.75f;
  }
  return clmp(1.0f - 2.2f * occ, 0.0f, 1.0f);
}
// softShadow (render-wgsl.ts:94-107)
__device__ float soft_shadow(const Ctx& c, V3 ro, V3 rd) {
  const V2 tb = box_hit(ro, rd, c3(c.a.bmin), c3(c.a.bmax));
  if (tb.x > tb.y || tb.y < 0.0f) return 1.0f;
  float t = mx(tb.x, 0.01f);
  float res = 1.0f;
  for (int i = 0; i < 48; i++) {
    const float hh = scene_sdf(c.S, ro + rd * t).x;
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

// materialAt (render-wgsl.ts:180-255) for the analytic scenes (look.meshMode == 0).
__device__ Mat material_at(const Ctx& c, float m, V3 pw, V3 n, float vd) {
  const Scene& S = c.S;
  const SceneArgs& a = c.a;
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

// shadeSurface (render-wgsl.ts:257-283); lift = 0.004 without the baked mesh
__device__ V3 shade_surface(const Ctx& c, V3 p, V3 n, V3 rd, const Mat& mt, bool fast) {
  const V3 key = c3(c.a.key);
  float sh = 1.0f, ao = 1.0f;
  const float lift = 0.004f;
  if (!fast) {
    sh = soft_shadow(c, p + n * lift, key);
    ao = ambient_occ(c, p + n * (lift - 0.004f), n);
  }
  const float ndl = mx(dot3(n, key), 0.0f);
  const float fill = mx(dot3(n, c3(c.a.fill_a)), 0.0f) * 0.18f + mx(dot3(n, c3(c.a.fill_b)), 0.0f) * 0.18f;
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

// RENDER fs_main (render-wgsl.ts:288-398), one thread per pixel.
__global__ void __launch_bounds__(64) scene_kernel(const Scene S, const SceneArgs a) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.w || y >= a.h) return;
  const Ctx c{S, a};
  const float ux = ((float)x + 0.5f) / (float)a.w, uy = ((float)y + 0.5f) / (float)a.h;
  const float ndx = (ux * 2.0f - 1.0f) + a.jitter_x, ndy = (1.0f - uy * 2.0f) + a.jitter_y;
  const V3 rd = nrm3(c3(a.fwd) + ndx * a.tan_half * a.aspect * c3(a.right) + ndy * a.tan_half * c3(a.up));
  const V3 ro = c3(a.pos);
  const V3 key = c3(a.key);

  V3 col = backdrop(rd);
  float t_hit = FAR;
  const V2 hit = march(c, ro, rd, 220);
  float t_ground = FAR;
  if (rd.y < -1e-4f) t_ground = -ro.y / rd.y;

  if (hit.x < t_ground && hit.x < FAR) {
    const V3 p = ro + rd * hit.x;
    const float vd = hit.x;
    const V3 n = calc_normal(c, p);
    Mat mt = material_at(c, hit.y, p, n, vd);
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
    col = shade_surface(c, p, n, rd, mt, false);
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
    const float sh = soft_shadow(c, p + up * 0.005f, key);
    const float ao = clmp(scene_sdf(S, p).x * 2.6f + 0.12f, 0.0f, 1.0f);
    col = gc * (0.35f + 0.65f * sh) * mixf(0.25f, 1.0f, ao);
    const V3 rdir = reflect3(rd, up);
    const float fres = 0.02f + 0.22f * wtm::powf(1.0f - ab(rd.y), 5.0f);
    V3 refl = studio_env(rdir) * 0.35f;
    const V2 rh = march(c, p + up * 0.002f, rdir, 90);
    if (rh.x < FAR) {
      const V3 rp = p + rdir * rh.x;
      const V3 rn = calc_normal(c, rp);
      const float vd = t_ground + rh.x;
      refl = shade_surface(c, rp, rn, rdir, material_at(c, rh.y, rp, rn, vd), true) * wtm::expf(-rh.x * 2.2f);
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
  a.scene[(size_t)y * a.w + x] = pack(col.x, col.y, col.z, mn(t_hit, FAR));
}

// ---------------------------------------------------------------- TAA resolve (render-wgsl.ts:456-518)
__device__ __forceinline__ V3 tm(V3 c) { return c / (1.0f + mx(c.x, mx(c.y, c.z))); }
__device__ __forceinline__ V3 itm(V3 c) { return c / mx(1e-4f, 1.0f - mx(c.x, mx(c.y, c.z))); }
__device__ __forceinline__ int iclampi(int e, int lo, int hi) { return e < lo ? lo : (e > hi ? hi : e); }

__global__ void taa_kernel(const TaaArgs a) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.w || y >= a.h) return;
  const float ux = ((float)x + 0.5f) / (float)a.w, uy = ((float)y + 0.5f) / (float)a.h;
  const int sx = (int)a.w, sy = (int)a.h;
  const int px = iclampi(to_i32(ux * (float)sx), 0, sx - 1), py = iclampi(to_i32(uy * (float)sy), 0, sy - 1);
  const float4 c0 = load_tex(a.cur, a.w, px, py);
  V3 mu = zero3(), m2 = zero3();
  float closest = c0.w;
  for (int j = -1; j <= 1; j++)
    for (int i = -1; i <= 1; i++) {
      const float4 s = load_tex(a.cur, a.w, iclampi(px + i, 0, sx - 1), iclampi(py + j, 0, sy - 1));
      const V3 t = tm(v3(s.x, s.y, s.z));
      mu = mu + t;
      m2 = m2 + t * t;
      closest = mn(closest, s.w);
    }
  mu = mu / 9.0f;
  const V3 var = vmax3(m2 / 9.0f - mu * mu, zero3());
  const V3 sigma = v3(__fsqrt_rn(var.x), __fsqrt_rn(var.y), __fsqrt_rn(var.z));
  const V3 lo = mu - sigma * 1.25f, hi = mu + sigma * 1.25f;

  const float ndx = ux * 2.0f - 1.0f, ndy = 1.0f - uy * 2.0f;
  const V3 rd = nrm3(c3(a.fwd) + ndx * a.tan_half * a.aspect * c3(a.right) + ndy * a.tan_half * c3(a.up));
  const V3 wp = c3(a.cam_pos) + rd * mn(closest, 1.0e4f);
  const float* m = a.m;
  const float cx = m[0] * wp.x + m[4] * wp.y + m[8] * wp.z + m[12] * 1.0f;
  const float cy = m[1] * wp.x + m[5] * wp.y + m[9] * wp.z + m[13] * 1.0f;
  const float cw = m[3] * wp.x + m[7] * wp.y + m[11] * wp.z + m[15] * 1.0f;
  const float pux = cx / cw * 0.5f + 0.5f, puy = 0.5f - cy / cw * 0.5f;
  const bool valid = cw > 0.0f && pux >= 0.0f && puy >= 0.0f && pux <= 1.0f && puy <= 1.0f;

  const V3 cur3 = tm(v3(c0.x, c0.y, c0.z));
  V3 outc = cur3;
  if (valid && a.blend < 1.0f) {
    // histAt: bilinear of the history at puv with clamped texel indices
    const float hx = pux * (float)sx - 0.5f, hy = puy * (float)sy - 0.5f;
    const int i0 = to_i32(floorf(hx)), j0 = to_i32(floorf(hy));
    const float fx = hx - (float)i0, fy = hy - (float)j0;
    const float4 ta = load_tex(a.hist, a.w, iclampi(i0, 0, sx - 1), iclampi(j0, 0, sy - 1));
    const float4 tb = load_tex(a.hist, a.w, iclampi(i0 + 1, 0, sx - 1), iclampi(j0, 0, sy - 1));
    const float4 tc = load_tex(a.hist, a.w, iclampi(i0, 0, sx - 1), iclampi(j0 + 1, 0, sy - 1));
    const float4 td = load_tex(a.hist, a.w, iclampi(i0 + 1, 0, sx - 1), iclampi(j0 + 1, 0, sy - 1));
    const V3 hab = vmix3(v3(ta.x, ta.y, ta.z), v3(tb.x, tb.y, tb.z), fx);
    const V3 hcd = vmix3(v3(tc.x, tc.y, tc.z), v3(td.x, td.y, td.z), fx);
    const V3 hh = vclamp3(tm(vmix3(hab, hcd, fy)), lo, hi);
    const V2 dm = v2((pux - ux) * (float)sx, (puy - uy) * (float)sy);
    const float motion = len2(dm);
    const float w = clmp(a.blend + motion * 0.04f, a.blend, 1.0f);
    outc = vmix3(hh, cur3, w);
  }
  const V3 o = itm(outc);
  a.out[(size_t)y * a.w + x] = pack(o.x, o.y, o.z, c0.w);
}

// ---------------------------------------------------------------- bloom blur (render-wgsl.ts:401-418)
__global__ void blur_kernel(const BlurArgs a) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.dw || y >= a.dh) return;
  const float ux = ((float)x + 0.5f) / (float)a.dw, uy = ((float)y + 0.5f) / (float)a.dh;
  const int sx = (int)a.sw, sy = (int)a.sh;
  const float bx = ux * (float)sx, by = uy * (float)sy;
  V3 acc = zero3();
  float wsum = 0.0f;
  for (int k = -6; k <= 6; k++) {
    const float w = a.wk[k + 6];
    const float fk = (float)k;
    const int qx = iclampi(to_i32(bx + a.dir_x * fk * a.spacing), 0, sx - 1);
    const int qy = iclampi(to_i32(by + a.dir_y * fk * a.spacing), 0, sy - 1);
    const float4 s = load_tex(a.src, a.sw, qx, qy);
    acc = acc + v3(s.x, s.y, s.z) * w;
    wsum = wsum + w;
  }
  const V3 o = acc / wsum * a.gain;
  a.dst[(size_t)y * a.dw + x] = pack(o.x, o.y, o.z, 1.0f);
}

// ---------------------------------------------------------------- present (render-wgsl.ts:420-454)
__device__ V3 bilinear(const ushort4* t, uint32_t w, uint32_t h, float ux, float uy) {
  const float px = ux * (float)w - 0.5f, py = uy * (float)h - 0.5f;
  const int i0 = to_i32(floorf(px)), j0 = to_i32(floorf(py));
  const float fx = px - (float)i0, fy = py - (float)j0;
  const int mx_ = (int)w - 1, my_ = (int)h - 1;
  const float4 ta = load_tex(t, w, iclampi(i0, 0, mx_), iclampi(j0, 0, my_));
  const float4 tb = load_tex(t, w, iclampi(i0 + 1, 0, mx_), iclampi(j0, 0, my_));
  const float4 tc = load_tex(t, w, iclampi(i0, 0, mx_), iclampi(j0 + 1, 0, my_));
  const float4 td = load_tex(t, w, iclampi(i0 + 1, 0, mx_), iclampi(j0 + 1, 0, my_));
  return vmix3(vmix3(v3(ta.x, ta.y, ta.z), v3(tb.x, tb.y, tb.z), fx), vmix3(v3(tc.x, tc.y, tc.z), v3(td.x, td.y, td.z), fx), fy);
}
__device__ __forceinline__ float aces1(float x) {
  return clmp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
}
__device__ __forceinline__ unsigned char unorm8(float x) {
  if (!(x == x)) return 0;
  return (unsigned char)rintf(clmp(x, 0.0f, 1.0f) * 255.0f);
}
// 1 / 2.2 as WGSL constant-evaluates the AbstractFloat quotient (in double, rounded once)
constexpr float INV_GAMMA = 0x1.d1745ep-2f;

__global__ void present_kernel(const PresentArgs a) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.w || y >= a.h) return;
  const float ux = ((float)x + 0.5f) / (float)a.w, uy = ((float)y + 0.5f) / (float)a.h;
  const V3 c = bilinear(a.scene, a.w, a.h, ux, uy);
  const int gx = iclampi(to_i32(ux * (float)a.gw), 0, (int)a.gw - 1), gy = iclampi(to_i32(uy * (float)a.gh), 0, (int)a.gh - 1);
  const float4 g4 = load_tex(a.glow, a.gw, gx, gy);
  const V3 bl = bilinear(a.bloom_tex, a.bw, a.bh, ux, uy);
  const V3 hdr = c * a.exposure + v3(g4.x, g4.y, g4.z) + bl * a.bloom;
  V3 o = v3(wtm::powf(aces1(hdr.x), INV_GAMMA), wtm::powf(aces1(hdr.y), INV_GAMMA), wtm::powf(aces1(hdr.z), INV_GAMMA));
  const float dx = ux - 0.5f, dy = uy - 0.5f;
  o = o * (1.0f - (dx * dx + dy * dy) * 0.6f);
  uchar4 r;
  r.x = unorm8(o.x); r.y = unorm8(o.y); r.z = unorm8(o.z); r.w = unorm8(1.0f);
  a.out[(size_t)y * a.w + x] = r;
}

// ---------------------------------------------------------------- glow pass
struct Vtx {
  float X, Y, nz, iw;   // framebuffer position, NDC depth, 1 / clip w
  float c[4], side, dist;
};

__device__ __forceinline__ float4 mul4(const float* m, float x, float y, float z, float w) {
  return make_float4(m[0] * x + m[4] * y + m[8] * z + m[12] * w, m[1] * x + m[5] * y + m[9] * z + m[13] * w,
                     m[2] * x + m[6] * y + m[10] * z + m[14] * w, m[3] * x + m[7] * y + m[11] * z + m[15] * w);
}
__device__ __forceinline__ Vtx to_vtx(const DrawArgs& a, float px, float py, float pz, float pw) {
  Vtx v;
  const float nx = px / pw, ny = py / pw;
  v.nz = pz / pw;
  v.X = (nx * 0.5f + 0.5f) * (float)a.w;
  v.Y = (0.5f - ny * 0.5f) * (float)a.h;
  v.iw = 1.0f / pw;
  return v;
}

// Corner k of the quad (vertex_index 0, 1, 2, 5 of the 6-vertex list; 3 and 4
// repeat 0 and 2): (along, side).
__device__ __forceinline__ V2 corner(int k) {
  return k == 0 ? v2(0.0f, -1.0f) : (k == 1 ? v2(1.0f, -1.0f) : (k == 2 ? v2(1.0f, 1.0f) : v2(0.0f, 1.0f)));
}

// PARTICLES_DRAW vs_main (wgsl.ts:615-650) for the four corners of instance ii.
__device__ bool particle_corners(const DrawArgs& a, uint32_t ii, Vtx* out) {
  const uint32_t pi = ii % a.count;
  const bool mirror = ii >= a.count;
  const float4 ppos = a.data[2 * pi], pvel = a.data[2 * pi + 1];
  if (pvel.w < 0.0f) return false;
  V3 head = v3(ppos.x, ppos.y, ppos.z), vel = v3(pvel.x, pvel.y, pvel.z);
  if (mirror) {
    head.z = -head.z;
    vel.z = -vel.z;
  }
  const V3 tail = head - vel * a.trail;
  const float4 ca = mul4(a.m, tail.x, tail.y, tail.z, 1.0f), cb = mul4(a.m, head.x, head.y, head.z, 1.0f);
  if (ca.w < 0.05f || cb.w < 0.05f) return false;
  const V2 res = v2(a.res_x, a.res_y);
  const V2 sa = v2(ca.x, ca.y) / ca.w * res * 0.5f, sb = v2(cb.x, cb.y) / cb.w * res * 0.5f;
  V2 dir = sb - sa;
  const float len = len2(dir);
  dir = len > 1e-3f ? dir / len : v2(1.0f, 0.0f);
  const V2 nrm = v2(-dir.y, dir.x);
  const float fade = clmp(ppos.w / a.fade_in, 0.0f, 1.0f);
  const V3 pc = palette(a.palette, pvel.w);
  float heat_boost = 1.0f;
  if (a.palette == 2u) heat_boost = mixf(0.25f, 4.0f, sstep(0.08f, 0.6f, pvel.w));
  for (int k = 0; k < 4; k++) {
    const V2 cn = corner(k);
    const float along = cn.x;
    const float w = a.width;
    const V2 sp = mix2(sa, sb, along) + nrm * cn.y * w * 0.5f + dir * (along * 2.0f - 1.0f) * w * 0.5f;
    const float cw = mixf(ca.w, cb.w, along);
    const float cz = mixf(ca.z / ca.w, cb.z / cb.w, along);
    const V2 q = sp / (res * 0.5f) * cw;
    Vtx v = to_vtx(a, q.x, q.y, cz * cw, cw);
    v.c[0] = pc.x; v.c[1] = pc.y; v.c[2] = pc.z;
    v.c[3] = a.alpha * fade * heat_boost * mixf(0.15f, 1.0f, along);
    v.side = cn.y;
    const V3 pm = v3(mixf(tail.x, head.x, along), mixf(tail.y, head.y, along), mixf(tail.z, head.z, along));
    v.dist = len3(c3(a.cam_pos) - pm);
    out[k] = v;
  }
  return true;
}

// hash1 (render-wgsl.ts:596-600)
__device__ __forceinline__ float hash1(uint32_t n) {
  const uint32_t s = n * 747796405u + 2891336453u;
  const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (float)((w >> 22u) ^ w) / 4294967296.0f;  // the reference's 4294967295.0 as f32
}

// STREAM_DRAW vs_main (render-wgsl.ts:601-637) for the four corners of instance ii.
__device__ bool stream_corners(const DrawArgs& a, uint32_t ii, Vtx* out) {
  const uint32_t segs = a.steps - 1u;
  const uint32_t seg = ii % segs;
  const uint32_t line_all = ii / segs;
  const bool mirror = line_all >= a.lines;
  const uint32_t line = line_all % a.lines;
  float4 pa = a.data[line * a.steps + seg], pb = a.data[line * a.steps + seg + 1u];
  if (pa.w < 0.0f || pb.w < 0.0f) return false;
  if (mirror) {
    pa.z = -pa.z;
    pb.z = -pb.z;
  }
  const float4 ca = mul4(a.m, pa.x, pa.y, pa.z, 1.0f), cb = mul4(a.m, pb.x, pb.y, pb.z, 1.0f);
  if (ca.w < 0.05f || cb.w < 0.05f) return false;
  const V2 res = v2(a.res_x, a.res_y);
  const V2 sa = v2(ca.x, ca.y) / ca.w * res * 0.5f, sb = v2(cb.x, cb.y) / cb.w * res * 0.5f;
  V2 dir = sb - sa;
  const float len = len2(dir);
  dir = len > 1e-4f ? dir / len : v2(1.0f, 0.0f);
  const V2 nrm = v2(-dir.y, dir.x);
  const float hl = hash1(line * 7u + 3u);
  for (int k = 0; k < 4; k++) {
    const V2 cn = corner(k);
    const float along = cn.x;
    const V2 sp = mix2(sa, sb, along) + nrm * cn.y * a.width * 0.5f + dir * (along * 2.0f - 1.0f) * a.width * 0.3f;
    const float cw = mixf(ca.w, cb.w, along);
    const float cz = mixf(ca.z / ca.w, cb.z / cb.w, along);
    const V2 q = sp / (res * 0.5f) * cw;
    Vtx v = to_vtx(a, q.x, q.y, cz * cw, cw);
    const float t = (float)seg + along;
    const float phase = fractf(t * 0.011f - a.time * 0.42f + hl);
    const float pulse = wtm::powf(phase, 14.0f) * a.pulse;
    const float fade_in = sstep(0.0f, 14.0f, t);
    const float fade_out = 1.0f - sstep((float)a.steps * 0.8f, (float)a.steps, t);
    const float vv = mixf(pa.w, pb.w, along);
    const V3 col = palette(a.palette, vv) * a.intensity * (0.55f + pulse) * fade_in * fade_out;
    v.c[0] = col.x; v.c[1] = col.y; v.c[2] = col.z; v.c[3] = 0.0f;
    v.side = cn.y;
    const V3 pm = v3(mixf(pa.x, pb.x, along), mixf(pa.y, pb.y, along), mixf(pa.z, pb.z, along));
    v.dist = len3(c3(a.cam_pos) - pm);
    out[k] = v;
  }
  return true;
}

__device__ __forceinline__ bool edge_owned(float dx, float dy) { return dy > 0.0f || (dy == 0.0f && dx < 0.0f); }
__device__ __forceinline__ unsigned long long fixed32(float v) {
  return (unsigned long long)__double2ll_rn((double)v * 4294967296.0);
}

// Rasterize triangle (v0, v1, v2) and shade its fragments (the fragment shaders
// of wgsl.ts:652-658 and render-wgsl.ts:638-644).
__device__ void raster_triangle(const DrawArgs& a, const Vtx& v0, const Vtx& v1, const Vtx& v2) {
  const float A = (v1.X - v0.X) * (v2.Y - v0.Y) - (v2.X - v0.X) * (v1.Y - v0.Y);
  if (!(A > 0.0f) && !(A < 0.0f)) return;
  const float sg = A > 0.0f ? 1.0f : -1.0f;
  const float aa = A > 0.0f ? A : -A;
  const float minx = fminf(v0.X, fminf(v1.X, v2.X)), maxx = fmaxf(v0.X, fmaxf(v1.X, v2.X));
  const float miny = fminf(v0.Y, fminf(v1.Y, v2.Y)), maxy = fmaxf(v0.Y, fmaxf(v1.Y, v2.Y));
  // pixel centres inside the bounding box, clamped to the target (and to [-1, size] so
  // that far-off coordinates convert to int exactly)
  const int x0 = (int)ceilf(fminf(fmaxf(minx - 0.5f, 0.0f), (float)a.w));
  const int x1 = (int)floorf(fmaxf(fminf(maxx - 0.5f, (float)(a.w - 1)), -1.0f));
  const int y0 = (int)ceilf(fminf(fmaxf(miny - 0.5f, 0.0f), (float)a.h));
  const int y1 = (int)floorf(fmaxf(fminf(maxy - 0.5f, (float)(a.h - 1)), -1.0f));
  const bool own0 = edge_owned((v2.X - v1.X) * sg, (v2.Y - v1.Y) * sg);
  const bool own1 = edge_owned((v0.X - v2.X) * sg, (v0.Y - v2.Y) * sg);
  const bool own2 = edge_owned((v1.X - v0.X) * sg, (v1.Y - v0.Y) * sg);
  for (int py = y0; py <= y1; py++)
    for (int px = x0; px <= x1; px++) {
      const float Px = (float)px + 0.5f, Py = (float)py + 0.5f;
      const float e0 = ((v2.X - v1.X) * (Py - v1.Y) - (v2.Y - v1.Y) * (Px - v1.X)) * sg;
      const float e1 = ((v0.X - v2.X) * (Py - v2.Y) - (v0.Y - v2.Y) * (Px - v2.X)) * sg;
      const float e2 = ((v1.X - v0.X) * (Py - v0.Y) - (v1.Y - v0.Y) * (Px - v0.X)) * sg;
      if (e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) continue;
      if ((e0 == 0.0f && !own0) || (e1 == 0.0f && !own1) || (e2 == 0.0f && !own2)) continue;
      const float b0 = e0 / aa, b1 = e1 / aa, b2 = e2 / aa;
      const float z = b0 * v0.nz + b1 * v1.nz + b2 * v2.nz;
      if (!(z >= 0.0f && z <= 1.0f)) continue;
      const float q0 = b0 * v0.iw, q1 = b1 * v1.iw, q2 = b2 * v2.iw;
      const float qs = q0 + q1 + q2;
      const float w0 = q0 / qs, w1 = q1 / qs, w2 = q2 / qs;
      const float side = w0 * v0.side + w1 * v1.side + w2 * v2.side;
      const float dist = w0 * v0.dist + w1 * v1.dist + w2 * v2.dist;
      // fragment: scene depth at the pixel (pos.xy / res * size of the scene target)
      const int sx = iclampi(to_i32(Px / a.res_x * (float)a.w), 0, (int)a.w - 1);
      const int sy = iclampi(to_i32(Py / a.res_y * (float)a.h), 0, (int)a.h - 1);
      const float scene_dist = h2f(a.scene[(size_t)sy * a.w + sx].w);
      float cr, cg, cb, ca;
      if (a.kind == 0) {
        if (dist > scene_dist + 0.03f) continue;
        const float c0 = w0 * v0.c[0] + w1 * v1.c[0] + w2 * v2.c[0];
        const float c1 = w0 * v0.c[1] + w1 * v1.c[1] + w2 * v2.c[1];
        const float c2 = w0 * v0.c[2] + w1 * v1.c[2] + w2 * v2.c[2];
        const float c3v = w0 * v0.c[3] + w1 * v1.c[3] + w2 * v2.c[3];
        const float al = c3v * (1.0f - side * side);
        cr = c0 * al; cg = c1 * al; cb = c2 * al; ca = al;
      } else {
        if (dist > scene_dist + 0.02f) continue;
        const float c0 = w0 * v0.c[0] + w1 * v1.c[0] + w2 * v2.c[0];
        const float c1 = w0 * v0.c[1] + w1 * v1.c[1] + w2 * v2.c[1];
        const float c2 = w0 * v0.c[2] + w1 * v1.c[2] + w2 * v2.c[2];
        const float al = 1.0f - side * side;
        cr = c0 * al; cg = c1 * al; cb = c2 * al; ca = al;
      }
      unsigned long long* o = a.acc + ((size_t)py * a.w + px) * 4;
      atomicAdd(o + 0, fixed32(cr));
      atomicAdd(o + 1, fixed32(cg));
      atomicAdd(o + 2, fixed32(cb));
      atomicAdd(o + 3, fixed32(ca));
    }
}

// One thread per quad instance: its four corners, then triangles (0, 1, 2) and
// (3, 4, 5) = corners (0, 2, 3).
__global__ void glow_draw_kernel(const DrawArgs a) {
  const uint32_t ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= a.instances) return;
  Vtx v[4];
  const bool live = a.kind == 0 ? particle_corners(a, ii, v) : stream_corners(a, ii, v);
  if (!live) return;  // culled: every vertex at (2, 2, 2, 1), zero area
  raster_triangle(a, v[0], v[1], v[2]);
  raster_triangle(a, v[0], v[2], v[3]);
}

__global__ void glow_resolve_kernel(const unsigned long long* __restrict__ acc, ushort4* __restrict__ glow, uint32_t texels) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= texels) return;
  float c[4];
  for (int k = 0; k < 4; k++) c[k] = __double2float_rn(__ll2double_rn((long long)acc[4 * (size_t)i + k]) * 0x1p-32);
  glow[i] = pack(c[0], c[1], c[2], c[3]);
}

dim3 tiles(uint32_t w, uint32_t h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

}  // namespace

cudaError_t launch_render_scene(const SceneArgs& a, cudaStream_t s) {
  const Scene S = make_scene(a.shape);
  const dim3 b(8, 8);
  scene_kernel<<<tiles(a.w, a.h, b), b, 0, s>>>(S, a);
  return cudaGetLastError();
}

cudaError_t launch_taa(const TaaArgs& a, cudaStream_t s) {
  const dim3 b(16, 8);
  taa_kernel<<<tiles(a.w, a.h, b), b, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_blur(const BlurArgs& a, cudaStream_t s) {
  const dim3 b(16, 8);
  blur_kernel<<<tiles(a.dw, a.dh, b), b, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_present(const PresentArgs& a, cudaStream_t s) {
  const dim3 b(16, 8);
  present_kernel<<<tiles(a.w, a.h, b), b, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_glow_draw(const DrawArgs& a, cudaStream_t s) {
  if (a.instances == 0) return cudaSuccess;
  glow_draw_kernel<<<(a.instances + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_glow_resolve(const unsigned long long* acc, ushort4* glow, uint32_t texels, cudaStream_t s) {
  glow_resolve_kernel<<<(texels + 255) / 256, 256, 0, s>>>(acc, glow, texels);
  return cudaGetLastError();
}

}  // namespace wt
