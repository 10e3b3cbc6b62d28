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

#include "wt_render.h"
#include "wt_shade.cuh"

namespace wt {
namespace {

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

// One thread per pixel.  16 blocks of 64 per SM (64 registers, a few spills): the
// march waits on latency that more resident warps hide (3.85 -> 3.65 ms per frame).
template <bool MESH>
__global__ void __launch_bounds__(64, 16) scene_kernel(const Scene S, const SceneArgs a) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.w || y >= a.h) return;
  const float4 c = render_pixel<MESH>(S, a, x, y);
  a.scene[(size_t)y * a.w + x] = pack(c.x, c.y, c.z, c.w);
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
  const Scene S = make_scene(a.shape, a.car);
  const dim3 b(8, 8);
  if (a.mesh_mode != 0u) scene_kernel<true><<<tiles(a.w, a.h, b), b, 0, s>>>(S, a);
  else scene_kernel<false><<<tiles(a.w, a.h, b), b, 0, s>>>(S, a);
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
