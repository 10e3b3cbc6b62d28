// The car mesh G-buffer pass: the reference's MESH_DRAW pipeline
// (src/engine/render-wgsl.ts:647-760) over the draws of MeshCar
// (src/engine/mesh-car.ts:46-213) into the G-buffer (src/engine/engine.ts:
// 297-303, 716), as CUDA kernels.
//
// The reference draws triangle after triangle with a depth test against the
// buffer as it stands.  Here the result is formed without any ordering between
// threads and is still the sequential one:
//   vertex pass   one thread per corner of every draw: MESH_DRAW vs_main
//                 (rig rotations, sidepod squeeze, fly-away, rake, jitter)
//   opaque draws  visibility: each covered pixel that passes 'less' against
//                 the depth at the start of the run of opaque draws takes the
//                 64-bit atomic minimum of (depth bits, triangle sequence), so
//                 the nearest fragment wins and, among equal depths, the first
//                 drawn, which is what 'less' with depth writes keeps; then one
//                 thread per pixel evaluates the winning fragment (fs_main) and
//                 writes albedo, normal-distance, material and depth
//   decal draws   (no depth write, so the test depends on the opaque depth
//                 only) the passing fragments of each pixel are counted, laid
//                 out by a prefix sum, collected, and blended per pixel in
//                 triangle order with DECAL_BLEND (mesh-car.ts:22-25)
// Triangles whose screen footprint is large go to a second launch that gives
// each one a block of threads.
//
// Fixed-function stages follow the WebGPU pipeline as the glow pass does
// (viewport, edge functions with the shared-edge rule, depth clip,
// perspective-correct varyings), plus: clipping to z >= 0 in clip space;
// depth32float with the decal depth bias (depthBias -4, slopeScale -1,
// mesh-car.ts:150); textureSample derivatives from the 2 x 2 pixel quad; the
// texture filter of wt_texfilter.h.  Built with -fmad=false: the targets equal
// the CPU pipeline that runs the reference's own MESH_DRAW shader bit for bit.
#include <cuda_fp16.h>

#include <cub/device/device_scan.cuh>

#include "wt_mesh.h"
#include "wt_scene.cuh"

namespace wt {
namespace {

constexpr uint32_t KEEP = 0xffffffffu;  // visibility key: the pixel keeps its earlier fragment
constexpr int BIG_PIXELS = 1024;        // bounding boxes above this are split into tiles
constexpr int TILE = 32;                // pixels per side of a tile of a large triangle

// A corner after the vertex shader: position and, when ATTR, the varyings
// (world xyz, normal xyz, uv).  Coverage and depth need the position only.
template <bool ATTR>
struct CornerT {
  float4 pos;
  float a[ATTR ? 8 : 1];
};
using Corner = CornerT<true>;
constexpr int nattr(bool attr) { return attr ? 8 : 0; }

// ---------------------------------------------------------------- vertex stage
// rigRotate with dir = +1, rigRotateDir and podDeform with dir = +1
// (src/engine/car-model.ts:106-135)
__device__ V3 rig_rotate_fwd(const float4* R, V3 p, uint32_t part) {
  if (part == 0u || part > 4u) return p;
  const float a = rig_angle(R, part, p.z) * 1.0f;
  const float k = rig_scale(R, part);
  const V2 h = rig_hinge(R, part, p.z);
  const float c = wtm::cosf(a), s = wtm::sinf(a);
  V2 d = v2(p.x, p.y) - h;
  d = v2(d.x * k, d.y * k);
  d = v2(c * d.x - s * d.y, s * d.x + c * d.y);
  return v3(h.x + d.x, h.y + d.y, p.z);
}
__device__ V3 rig_rotate_dir(const float4* R, V3 v, uint32_t part, float z) {
  const float a = rig_angle(R, part, z);
  const float c = wtm::cosf(a), s = wtm::sinf(a);
  return v3(c * v.x - s * v.y, s * v.x + c * v.y, v.z);
}
__device__ V3 pod_deform_fwd(const float4* R, V3 p) {
  const float c = rig_at(R, RIG_EXTRA).z * pod_weight(p);
  if (c <= 0.0f) return p;
  const float az = ab(p.z);
  const float kz = 1.0f - c;
  const float ky = 1.0f - 0.45f * c;
  const float nz = az > 0.26f ? 0.26f + (az - 0.26f) * kz : az;
  const float sg = p.z > 0.0f ? 1.0f : (p.z < 0.0f ? -1.0f : 0.0f);
  return v3(p.x, 0.12f + (p.y - 0.12f) * ky, sg * nz);
}

// vs_main (render-wgsl.ts:702-738) for vertex_index vi of draw d
__device__ Corner mesh_vs(const MeshArgs& a, const MeshDraw& d, uint32_t vi) {
  const uint32_t i = a.indices[d.first_index + vi];
  const float4 va = a.verts[2 * (size_t)i], vb = a.verts[2 * (size_t)i + 1];
  const uint32_t tag = a.tags[i];
  const uint32_t part = tag & 7u, assembly = tag >> 3u;
  V3 p = v3(va.x, va.y, va.z), nrm = v3(vb.x, vb.y, vb.z);
  if (part != 0u) {
    nrm = rig_rotate_dir(a.rig, nrm, part, p.z);
    p = rig_rotate_fwd(a.rig, p, part);
  } else if (assembly == 0u && d.is_body > 0.5f) {
    p = pod_deform_fwd(a.rig, p);
  }
  bool hidden = false;
  if (assembly != 0u) {
    const float4 fly = rig_at(a.rig, RIG_FLY);
    const bool fw = assembly == 1u;
    const float t = fw ? fly.x : fly.y;
    if (t > 0.0f) {
      // flyAway, flyNormal (render-wgsl.ts:676-690)
      const V2 c = fw ? v2(0.2f, 0.28f) : v2(4.85f, 0.85f);
      const float an = (fw ? 4.8f : -5.5f) * t;
      const float ca = wtm::cosf(an), sa = wtm::sinf(an);
      const V2 dd = v2(p.x - c.x, p.y - c.y);
      const V2 r = v2(ca * dd.x - sa * dd.y, sa * dd.x + ca * dd.y);
      const float up = 2.4f * wtm::sinf(mn(t, 1.0f) * 1.5708f) + 0.6f * t;
      const float back = (fw ? 3.0f : 4.5f) * t * t;
      p = v3((c.x + r.x) + back, (c.y + r.y) + up, p.z * (1.0f + 1.2f * t * t) + 0.0f);
      nrm = v3(ca * nrm.x - sa * nrm.y, sa * nrm.x + ca * nrm.y, nrm.z);
      hidden = t >= 0.999f;
    }
  }
  // toWorld, rotateNormal (render-wgsl.ts:692-701): the rake about the front axle
  V3 w = p, n = nrm;
  if (!(d.is_body == 0.0f)) {
    const float c = wtm::cosf(a.rake), s = wtm::sinf(a.rake);
    const float bx = p.x - 1.0f, by = p.y - a.base_ride;
    w = v3(1.0f + c * bx - s * by, a.ride_h + s * bx + c * by, p.z);
    n = v3(c * nrm.x - s * nrm.y, s * nrm.x + c * nrm.y, nrm.z);
  }
  const float* m = a.vp;
  float4 cl;
  cl.x = m[0] * w.x + m[4] * w.y + m[8] * w.z + m[12] * 1.0f;
  cl.y = m[1] * w.x + m[5] * w.y + m[9] * w.z + m[13] * 1.0f;
  cl.z = m[2] * w.x + m[6] * w.y + m[10] * w.z + m[14] * 1.0f;
  cl.w = m[3] * w.x + m[7] * w.y + m[11] * w.z + m[15] * 1.0f;
  cl.x = cl.x + a.jitter[0] * cl.w;
  cl.y = cl.y + a.jitter[1] * cl.w;
  Corner o;
  o.pos = hidden ? make_float4(2.0f, 2.0f, 2.0f, 1.0f) : cl;
  o.a[0] = w.x; o.a[1] = w.y; o.a[2] = w.z;
  o.a[3] = n.x; o.a[4] = n.y; o.a[5] = n.z;
  o.a[6] = va.w; o.a[7] = vb.w;
  return o;
}

__global__ void mesh_vertex_kernel(const MeshArgs a, uint32_t corners) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= corners) return;
  uint32_t lo = 0, hi = a.n_draws;  // the last draw whose corner_base <= c
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (a.draws[mid].corner_base <= c) lo = mid; else hi = mid;
  }
  const MeshDraw& d = a.draws[lo];
  const Corner o = mesh_vs(a, d, c - d.corner_base);
  a.cpos[c] = o.pos;
  a.cattr[2 * (size_t)c] = make_float4(o.a[0], o.a[1], o.a[2], o.a[6]);
  a.cattr[2 * (size_t)c + 1] = make_float4(o.a[3], o.a[4], o.a[5], o.a[7]);
}

template <bool ATTR>
__device__ CornerT<ATTR> load_corner(const MeshArgs& a, size_t c) {
  CornerT<ATTR> o;
  o.pos = a.cpos[c];
  if (ATTR) {
    const float4 q = a.cattr[2 * c], r = a.cattr[2 * c + 1];
    o.a[0] = q.x; o.a[1] = q.y; o.a[2] = q.z;
    o.a[3] = r.x; o.a[4] = r.y; o.a[5] = r.z;
    o.a[6] = q.w; o.a[7] = r.w;
  }
  return o;
}

// ---------------------------------------------------------------- primitive setup
__device__ __forceinline__ float lerpf(float x, float y, float t) { return x + t * (y - x); }
template <bool ATTR>
__device__ CornerT<ATTR> corner_lerp(const CornerT<ATTR>& p, const CornerT<ATTR>& q, float t) {
  CornerT<ATTR> o;
  o.pos = make_float4(lerpf(p.pos.x, q.pos.x, t), lerpf(p.pos.y, q.pos.y, t), lerpf(p.pos.z, q.pos.z, t),
                      lerpf(p.pos.w, q.pos.w, t));
  for (int k = 0; k < nattr(ATTR); k++) o.a[k] = lerpf(p.a[k], q.a[k], t);
  return o;
}
// the part of the triangle with z >= 0 (0, 3 or 4 corners, in order)
template <bool ATTR>
__device__ int clip_near(const CornerT<ATTR>* c, CornerT<ATTR>* out) {
  int n = 0;
  for (int i = 0; i < 3; i++) {
    const CornerT<ATTR>& p = c[i];
    const CornerT<ATTR>& q = c[i == 2 ? 0 : i + 1];
    const bool inp = p.pos.z >= 0.0f, inq = q.pos.z >= 0.0f;
    if (inp) out[n++] = p;
    if (inp != inq) out[n++] = corner_lerp(p, q, p.pos.z / (p.pos.z - q.pos.z));
  }
  return n;
}

template <bool ATTR>
struct SVtxT {
  float X, Y, nz, iw;
  float a[ATTR ? 8 : 1];
};
template <bool ATTR>
struct TriT {
  SVtxT<ATTR> v[3];
  float sg, aa, bias;
  bool own0, own1, own2;
  int x0, x1, y0, y1;
  __device__ void edges(float Px, float Py, float* e) const {
    e[0] = ((v[2].X - v[1].X) * (Py - v[1].Y) - (v[2].Y - v[1].Y) * (Px - v[1].X)) * sg;
    e[1] = ((v[0].X - v[2].X) * (Py - v[2].Y) - (v[0].Y - v[2].Y) * (Px - v[2].X)) * sg;
    e[2] = ((v[1].X - v[0].X) * (Py - v[0].Y) - (v[1].Y - v[0].Y) * (Px - v[0].X)) * sg;
  }
  __device__ bool covers(const float* e) const {
    if (e[0] < 0.0f || e[1] < 0.0f || e[2] < 0.0f) return false;
    return !((e[0] == 0.0f && !own0) || (e[1] == 0.0f && !own1) || (e[2] == 0.0f && !own2));
  }
  __device__ float depth(const float* e) const {
    const float b0 = e[0] / aa, b1 = e[1] / aa, b2 = e[2] / aa;
    return b0 * v[0].nz + b1 * v[1].nz + b2 * v[2].nz;
  }
  __device__ void varyings(const float* e, float* out) const {
    const float b0 = e[0] / aa, b1 = e[1] / aa, b2 = e[2] / aa;
    const float q0 = b0 * v[0].iw, q1 = b1 * v[1].iw, q2 = b2 * v[2].iw;
    const float qs = q0 + q1 + q2;
    const float w0 = q0 / qs, w1 = q1 / qs, w2 = q2 / qs;
    for (int k = 0; k < nattr(ATTR); k++) out[k] = w0 * v[0].a[k] + w1 * v[1].a[k] + w2 * v[2].a[k];
  }
};
using Tri = TriT<true>;
__device__ __forceinline__ bool edge_owned(float dx, float dy) { return dy > 0.0f || (dy == 0.0f && dx < 0.0f); }

template <bool ATTR>
__device__ SVtxT<ATTR> screen(const CornerT<ATTR>& c, uint32_t W, uint32_t H) {
  SVtxT<ATTR> v;
  const float nx = c.pos.x / c.pos.w, ny = c.pos.y / c.pos.w;
  v.nz = c.pos.z / c.pos.w;
  v.X = (nx * 0.5f + 0.5f) * (float)W;
  v.Y = (0.5f - ny * 0.5f) * (float)H;
  v.iw = 1.0f / c.pos.w;
  for (int k = 0; k < nattr(ATTR); k++) v.a[k] = c.a[k];
  return v;
}

// Part s (0 or 1) of triangle tl of draw d, ready to rasterize; false when it
// has no fragments (outside the near plane, w <= 0, zero or NaN area).
template <bool ATTR>
__device__ bool setup_tri(const MeshArgs& a, const MeshDraw& d, uint32_t tl, int s, TriT<ATTR>& T) {
  const size_t c0 = (size_t)d.corner_base + 3 * (size_t)tl;
  const CornerT<ATTR> c0v = load_corner<ATTR>(a, c0), c1v = load_corner<ATTR>(a, c0 + 1),
                      c2v = load_corner<ATTR>(a, c0 + 2);
  if (c0v.pos.z >= 0.0f && c1v.pos.z >= 0.0f && c2v.pos.z >= 0.0f) {  // nothing to clip (kept in registers)
    if (s != 0 || !(c0v.pos.w > 0.0f && c1v.pos.w > 0.0f && c2v.pos.w > 0.0f)) return false;
    T.v[0] = screen(c0v, a.w, a.h);
    T.v[1] = screen(c1v, a.w, a.h);
    T.v[2] = screen(c2v, a.w, a.h);
  } else {
    CornerT<ATTR> c[3] = {c0v, c1v, c2v}, poly[4];
    const int np = clip_near<ATTR>(c, poly);
    if (s + 2 >= np) return false;
    const CornerT<ATTR>* t0 = &poly[0];
    const CornerT<ATTR>* t1 = &poly[s + 1];
    const CornerT<ATTR>* t2 = &poly[s + 2];
    if (!(t0->pos.w > 0.0f && t1->pos.w > 0.0f && t2->pos.w > 0.0f)) return false;
    T.v[0] = screen(*t0, a.w, a.h);
    T.v[1] = screen(*t1, a.w, a.h);
    T.v[2] = screen(*t2, a.w, a.h);
  }
  const SVtxT<ATTR>* v = T.v;
  const float A = (v[1].X - v[0].X) * (v[2].Y - v[0].Y) - (v[2].X - v[0].X) * (v[1].Y - v[0].Y);
  if (!(A > 0.0f) && !(A < 0.0f)) return false;
  T.sg = A > 0.0f ? 1.0f : -1.0f;
  T.aa = A > 0.0f ? A : -A;
  T.bias = 0.0f;
  if (d.blend) {
    const float dzdx = ((v[1].nz - v[0].nz) * (v[2].Y - v[0].Y) - (v[2].nz - v[0].nz) * (v[1].Y - v[0].Y)) / A;
    const float dzdy = ((v[2].nz - v[0].nz) * (v[1].X - v[0].X) - (v[1].nz - v[0].nz) * (v[2].X - v[0].X)) / A;
    const float m = mx(fabsf(dzdx), fabsf(dzdy));
    const float zmax = mx(fabsf(v[0].nz), mx(fabsf(v[1].nz), fabsf(v[2].nz)));
    int e = 0;
    frexpf(zmax, &e);
    T.bias = -4.0f * ldexpf(1.0f, e - 1 - 23) + -1.0f * m;
  }
  const float minx = mn(v[0].X, mn(v[1].X, v[2].X)), maxx = mx(v[0].X, mx(v[1].X, v[2].X));
  const float miny = mn(v[0].Y, mn(v[1].Y, v[2].Y)), maxy = mx(v[0].Y, mx(v[1].Y, v[2].Y));
  T.x0 = (int)ceilf(mn(mx(minx - 0.5f, 0.0f), (float)a.w));
  T.x1 = (int)floorf(mx(mn(maxx - 0.5f, (float)(a.w - 1)), -1.0f));
  T.y0 = (int)ceilf(mn(mx(miny - 0.5f, 0.0f), (float)a.h));
  T.y1 = (int)floorf(mx(mn(maxy - 0.5f, (float)(a.h - 1)), -1.0f));
  T.own0 = edge_owned((v[2].X - v[1].X) * T.sg, (v[2].Y - v[1].Y) * T.sg);
  T.own1 = edge_owned((v[0].X - v[2].X) * T.sg, (v[0].Y - v[2].Y) * T.sg);
  T.own2 = edge_owned((v[1].X - v[0].X) * T.sg, (v[1].Y - v[0].Y) * T.sg);
  return T.x0 <= T.x1 && T.y0 <= T.y1;
}

// the draw a frame-wide triangle sequence number belongs to, among [d0, d1)
__device__ uint32_t find_draw(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri) {
  uint32_t lo = d0, hi = d1;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (a.draws[mid].tri_base <= tri) lo = mid; else hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------- fragment stage
struct Frag {
  float4 albedo, normal_dist, material;
  bool discarded;
};
// fs_main (render-wgsl.ts:748-759) for the fragment of T at pixel (px, py)
__device__ Frag mesh_fs(const MeshArgs& a, const MeshDraw& d, const Tri& T, int px, int py, const float* e) {
  float v[8];
  T.varyings(e, v);
  float4 c = make_float4(d.color[0], d.color[1], d.color[2], d.color[3]);
  if (d.has_tex > 0.5f) {
    // coarse derivatives over the 2 x 2 quad, the varyings extrapolated from T
    const float qx = (float)(px & ~1) + 0.5f, qy = (float)(py & ~1) + 0.5f;
    float e00[3], e10[3], e01[3], a00[8], a10[8], a01[8];
    T.edges(qx, qy, e00);
    T.edges(qx + 1.0f, qy, e10);
    T.edges(qx, qy + 1.0f, e01);
    T.varyings(e00, a00);
    T.varyings(e10, a10);
    T.varyings(e01, a01);
    const MeshTex tx = a.texs[d.tex];
    const wtx::Rgba s = wtx::sample(a.levels + tx.first_level, (int)tx.n_levels, v[6], v[7], a10[6] - a00[6],
                                    a10[7] - a00[7], a01[6] - a00[6], a01[7] - a00[7]);
    c = make_float4(c.x * s.r, c.y * s.g, c.z * s.b, c.w * s.a);
  }
  Frag f;
  f.discarded = c.w < d.alpha_cut;
  if (f.discarded) return f;
  f.albedo = make_float4(c.x, c.y, c.z, d.alpha_cut > 0.0f ? c.w : d.rough);
  const V3 n = v3(v[3], v[4], v[5]);
  const float nl = len3(n);
  const V3 dw = v3(v[0] - a.cam_pos[0], v[1] - a.cam_pos[1], v[2] - a.cam_pos[2]);
  f.normal_dist = make_float4(n.x / nl, n.y / nl, n.z / nl, len3(dw));
  f.material = make_float4(d.metal, d.coat, d.emissive, 1.0f);
  return f;
}

__device__ __forceinline__ unsigned short f2h(float x) { return __half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ float h2f(unsigned short u) { return __half2float(__ushort_as_half(u)); }
__device__ __forceinline__ unsigned char unorm8(float x) {
  if (!(x == x)) return 0;
  return (unsigned char)rintf(clmp(x, 0.0f, 1.0f) * 255.0f);
}
__device__ __forceinline__ unsigned long long vis_key(float z, uint32_t seq) {
  return ((unsigned long long)__float_as_uint(z + 0.0f) << 32) | seq;  // + 0: -0 sorts as 0
}

// ---------------------------------------------------------------- rasterization
// Every pixel of the rectangle [x0, x1] x [y0, y1] (within T's bounding box),
// strided over `lanes` threads.
template <bool ATTR, class Op>
__device__ void raster(const TriT<ATTR>& T, int x0, int x1, int y0, int y1, int lane, int lanes, Op op) {
  const int bw = x1 - x0 + 1;
  const int n = bw * (y1 - y0 + 1);
  for (int i = lane; i < n; i += lanes) {
    const int px = x0 + i % bw, py = y0 + i / bw;
    float e[3];
    T.edges((float)px + 0.5f, (float)py + 0.5f, e);
    if (!T.covers(e)) continue;
    const float z = T.depth(e);
    if (!(z >= 0.0f && z <= 1.0f)) continue;
    op(px, py, e, z);
  }
}

// The visibility operation of the opaque draws: 'less' against the depth the
// run of opaque draws started from; with ATTR the fragment's alpha cut too.
template <bool ATTR>
struct OpaqueOp {
  const MeshArgs* a;
  const MeshDraw* d;
  const TriT<ATTR>* T;
  uint32_t seq;
  __device__ void operator()(int px, int py, const float* e, float z) const {
    const size_t p = (size_t)py * a->w + (size_t)px;
    if (!(z < a->depth[p])) return;
    if constexpr (ATTR) {
      if (mesh_fs(*a, *d, *T, px, py, e).discarded) return;
    }
    atomicMin(a->keys + p, vis_key(z, seq));
  }
};
// The decal test: biased depth, clamped to [0, 1], 'less-equal'; counted or collected.
template <bool ATTR>
struct DecalOp {
  const MeshArgs* a;
  const TriT<ATTR>* T;
  uint32_t seq;
  bool fill;
  __device__ void operator()(int px, int py, const float*, float z) const {
    const size_t p = (size_t)py * a->w + (size_t)px;
    float zb = z + T->bias;
    zb = zb < 0.0f ? 0.0f : (zb > 1.0f ? 1.0f : zb);
    if (!(zb <= a->depth[p])) return;
    if (fill) a->dslots[a->doff[p] + atomicAdd(a->dcur + p, 1u)] = seq;
    else atomicAdd(a->dcount + p, 1u);
  }
};

// kind 0: opaque visibility, 1: decal count, 2: decal fill.  ATTR: the
// varyings are loaded (an opaque draw with an alpha cut shades in this pass).
template <int KIND, bool ATTR>
__device__ void raster_part(const MeshArgs& a, const MeshDraw& d, const TriT<ATTR>& T, uint32_t tri, int s, int x0,
                            int x1, int y0, int y1, int lane, int lanes) {
  const uint32_t seq = tri * 2u + (uint32_t)s;
  if (KIND == 0) raster(T, x0, x1, y0, y1, lane, lanes, OpaqueOp<ATTR>{&a, &d, &T, seq});
  else raster(T, x0, x1, y0, y1, lane, lanes, DecalOp<ATTR>{&a, &T, seq, KIND == 2});
}
template <bool ATTR>
__device__ __forceinline__ uint32_t tiles_x(const TriT<ATTR>& T) { return (uint32_t)(T.x1 - T.x0 + TILE) / TILE; }
template <bool ATTR>
__device__ __forceinline__ uint32_t tiles_y(const TriT<ATTR>& T) { return (uint32_t)(T.y1 - T.y0 + TILE) / TILE; }

template <int KIND, bool ATTR>
__device__ void raster_triangle(const MeshArgs& a, const MeshDraw& d, uint32_t tri) {
  for (int s = 0; s < 2; s++) {
    TriT<ATTR> T;
    if (!setup_tri(a, d, tri - d.tri_base, s, T)) continue;
    if ((T.x1 - T.x0 + 1) * (T.y1 - T.y0 + 1) > BIG_PIXELS) {
      const unsigned long long old = atomicAdd(a.big_count, (1ull << 32) | (tiles_x(T) * tiles_y(T)));
      const uint32_t slot = (uint32_t)(old >> 32);
      if (slot < a.big_cap) a.big[slot] = make_uint4(tri, (uint32_t)s, (uint32_t)old, 0u);  // never full: 2 per triangle
      continue;
    }
    raster_part<KIND, ATTR>(a, d, T, tri, s, T.x0, T.x1, T.y0, T.y1, 0, 1);
  }
}

template <int KIND, bool ATTR>
__device__ void raster_tile(const MeshArgs& a, const MeshDraw& d, uint4 b, uint32_t u) {
  TriT<ATTR> T;
  if (!setup_tri(a, d, b.x - d.tri_base, (int)b.y, T)) return;
  const uint32_t t = u - b.z, tx = tiles_x(T);
  const int x0 = T.x0 + (int)(t % tx) * TILE, y0 = T.y0 + (int)(t / tx) * TILE;
  raster_part<KIND, ATTR>(a, d, T, b.x, (int)b.y, x0, min(x0 + TILE - 1, T.x1), y0, min(y0 + TILE - 1, T.y1),
                          threadIdx.x, blockDim.x);
}

// One thread per triangle of draws [d0, d1).  A large footprint is deferred as
// TILE x TILE tiles: one 64-bit atomic gives the part its list slot (high word)
// and the sequence number of its first tile (low word), so the list is ordered
// by first tile and a tile finds its part by binary search.
template <int KIND>
__global__ void mesh_raster_kernel(const MeshArgs a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1) {
  const uint32_t tri = tri0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (tri >= tri1) return;
  const MeshDraw& d = a.draws[find_draw(a, d0, d1, tri)];
  if (KIND == 0 && d.alpha_cut > 0.0f) raster_triangle<KIND, true>(a, d, tri);
  else raster_triangle<KIND, false>(a, d, tri);
}

// The tiles of the deferred large triangles, a block each (grid-strided).
template <int KIND>
__global__ void mesh_raster_big_kernel(const MeshArgs a, uint32_t d0, uint32_t d1) {
  const unsigned long long count = *a.big_count;
  const uint32_t n = min((uint32_t)(count >> 32), a.big_cap), tiles = (uint32_t)count;
  for (uint32_t u = blockIdx.x; u < tiles; u += gridDim.x) {
    uint32_t lo = 0, hi = n;  // the last part whose first tile is <= u
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (a.big[mid].z <= u) lo = mid; else hi = mid;
    }
    const uint4 b = a.big[lo];
    const MeshDraw& d = a.draws[find_draw(a, d0, d1, b.x)];
    if (KIND == 0 && d.alpha_cut > 0.0f) raster_tile<KIND, true>(a, d, b, u);
    else raster_tile<KIND, false>(a, d, b, u);
  }
}

__global__ void mesh_keys_kernel(const MeshArgs a) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)a.w * a.h) return;
  a.keys[p] = ((unsigned long long)__float_as_uint(a.depth[p] + 0.0f) << 32) | KEEP;
}

__global__ void mesh_clear_kernel(const MeshArgs a) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)a.w * a.h) return;
  a.depth[p] = 1.0f;
  a.g_albedo[p] = make_ushort4(0, 0, 0, 0);
  a.g_normal[p] = make_ushort4(0, 0, 0, 0);
  a.g_material[p] = make_uchar4(0, 0, 0, 0);
}

// The winning fragment of each pixel after a run of opaque draws.
__global__ void mesh_resolve_kernel(const MeshArgs a, uint32_t d0, uint32_t d1) {
  const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
  if (px >= a.w || py >= a.h) return;
  const size_t p = (size_t)py * a.w + px;
  const uint32_t seq = (uint32_t)(a.keys[p] & 0xffffffffull);
  if (seq == KEEP) return;
  const uint32_t tri = seq >> 1;
  const MeshDraw& d = a.draws[find_draw(a, d0, d1, tri)];
  Tri T;
  if (!setup_tri(a, d, tri - d.tri_base, (int)(seq & 1u), T)) return;  // cannot happen: it drew this pixel
  float e[3];
  T.edges((float)px + 0.5f, (float)py + 0.5f, e);
  const float z = T.depth(e);
  const Frag f = mesh_fs(a, d, T, (int)px, (int)py, e);
  a.g_albedo[p] = make_ushort4(f2h(f.albedo.x), f2h(f.albedo.y), f2h(f.albedo.z), f2h(f.albedo.w));
  a.g_normal[p] = make_ushort4(f2h(f.normal_dist.x), f2h(f.normal_dist.y), f2h(f.normal_dist.z), f2h(f.normal_dist.w));
  a.g_material[p] = make_uchar4(unorm8(f.material.x), unorm8(f.material.y), unorm8(f.material.z), unorm8(f.material.w));
  a.depth[p] = z;
}

// Each pixel's decal fragments in triangle order, blended into the albedo.
__global__ void mesh_decal_blend_kernel(const MeshArgs a, uint32_t d0, uint32_t d1) {
  const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
  if (px >= a.w || py >= a.h) return;
  const size_t p = (size_t)py * a.w + px;
  const uint32_t n = a.dcount[p];
  if (n == 0u) return;
  const uint32_t* list = a.dslots + a.doff[p];
  const ushort4 g = a.g_albedo[p];
  float r = h2f(g.x), gg = h2f(g.y), b = h2f(g.z);
  long long prev = -1;
  for (uint32_t k = 0; k < n; k++) {
    uint32_t next = KEEP;  // the smallest sequence number above prev (they are distinct)
    for (uint32_t j = 0; j < n; j++) {
      const uint32_t q = list[j];
      if ((long long)q > prev && q < next) next = q;
    }
    prev = next;
    const uint32_t tri = next >> 1;
    const MeshDraw& d = a.draws[find_draw(a, d0, d1, tri)];
    Tri T;
    if (!setup_tri(a, d, tri - d.tri_base, (int)(next & 1u), T)) continue;
    float e[3];
    T.edges((float)px + 0.5f, (float)py + 0.5f, e);
    const Frag f = mesh_fs(a, d, T, (int)px, (int)py, e);
    if (f.discarded) continue;
    const float sa = f.albedo.w;
    r = h2f(f2h(f.albedo.x * sa + r * (1.0f - sa)));
    gg = h2f(f2h(f.albedo.y * sa + gg * (1.0f - sa)));
    b = h2f(f2h(f.albedo.z * sa + b * (1.0f - sa)));
  }
  a.g_albedo[p] = make_ushort4(f2h(r), f2h(gg), f2h(b), g.w);
}

dim3 pixel_grid(const MeshArgs& a, dim3 b) { return dim3((a.w + b.x - 1) / b.x, (a.h + b.y - 1) / b.y); }

}  // namespace

cudaError_t launch_mesh_clear(const MeshArgs& a, cudaStream_t s) {
  const size_t n = (size_t)a.w * a.h;
  mesh_clear_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mesh_vertex(const MeshArgs& a, uint32_t corners, cudaStream_t s) {
  if (corners == 0) return cudaSuccess;
  mesh_vertex_kernel<<<(corners + 127) / 128, 128, 0, s>>>(a, corners);
  return cudaGetLastError();
}

namespace {
template <int KIND>
cudaError_t raster_draws(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.big_count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (tri1 <= tri0) return cudaSuccess;
  mesh_raster_kernel<KIND><<<(tri1 - tri0 + 127) / 128, 128, 0, s>>>(a, d0, d1, tri0, tri1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mesh_raster_big_kernel<KIND><<<1216, 256, 0, s>>>(a, d0, d1);  // 8 blocks per SM, strided over the list
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_mesh_opaque(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                               cudaStream_t s) {
  const size_t n = (size_t)a.w * a.h;
  mesh_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = raster_draws<0>(a, d0, d1, tri0, tri1, s);
  if (e != cudaSuccess) return e;
  const dim3 b(16, 8);
  mesh_resolve_kernel<<<pixel_grid(a, b), b, 0, s>>>(a, d0, d1);
  return cudaGetLastError();
}

cudaError_t launch_mesh_decal_count(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                                    cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.dcount, 0, (size_t)a.w * a.h * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = raster_draws<1>(a, d0, d1, tri0, tri1, s);
  return e;
}

cudaError_t launch_mesh_decal_scan(const MeshArgs& a, void* temp, size_t* temp_bytes, cudaStream_t s) {
  return cub::DeviceScan::ExclusiveSum(temp, *temp_bytes, a.dcount, a.doff, (int64_t)a.w * a.h, s);
}

cudaError_t launch_mesh_decal_blend(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                                    cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.dcur, 0, (size_t)a.w * a.h * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = raster_draws<2>(a, d0, d1, tri0, tri1, s);
  if (e != cudaSuccess) return e;
  const dim3 b(16, 8);
  mesh_decal_blend_kernel<<<pixel_grid(a, b), b, 0, s>>>(a, d0, d1);
  return cudaGetLastError();
}

}  // namespace wt
