// TEST INFRASTRUCTURE ONLY - never linked into the product library.
//
// A minimal C++ model of the WGSL types and builtins that the reference's
// simulation shaders use (src/engine/wgsl.ts, src/engine/f1.ts,
// src/engine/car-model.ts:59-136).  oracle/wgsl_translate.py rewrites the
// shader text itself into C++ that compiles against this header, so the
// reference's own arithmetic runs on the CPU without WebGPU.
//
// Semantics follow the WGSL specification's definitions:
//   min(a,b) = b < a ? b : a          max(a,b) = a < b ? b : a
//   clamp(e,lo,hi) = min(max(e,lo),hi)
//   mix(a,b,t) = a*(1-t) + b*t        smoothstep: t=clamp((x-lo)/(hi-lo),0,1); t*t*(3-2t)
//   length(v) = sqrt(dot(v,v)), dot summed x,y,z,w in order
//   round = ties to even               f32->i32/u32 truncate toward zero, clamped
// sin, cos and atan are implementation-defined in WGSL; they resolve to the
// project's own functions (wt_fmath.h), the same ones the device voxelizer
// uses.  Every arithmetic operation is one IEEE float operation; build with
// -ffp-contract=off.
#pragma once
#include <stdint.h>
#include <string.h>
#include "../f1-wind-tunnel_gb300/csrc/wt_fmath.h"

namespace rt {

typedef float f32;
typedef int32_t i32;
typedef uint32_t u32;
template <class T> using atomic = T;

// ---- scalar conversions -------------------------------------------------
static inline f32 to_f32(f32 x) { return x; }
static inline f32 to_f32(i32 x) { return (f32)x; }
static inline f32 to_f32(u32 x) { return (f32)x; }
static inline f32 to_f32(bool x) { return x ? 1.0f : 0.0f; }
static inline i32 to_i32(i32 x) { return x; }
static inline i32 to_i32(u32 x) { return (i32)x; }
static inline i32 to_i32(bool x) { return x ? 1 : 0; }
static inline i32 to_i32(f32 x) {
  if (!(x == x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (i32)0x80000000u;
  return (i32)x;
}
static inline u32 to_u32(u32 x) { return x; }
static inline u32 to_u32(i32 x) { return (u32)x; }
static inline u32 to_u32(bool x) { return x ? 1u : 0u; }
static inline u32 to_u32(f32 x) {
  if (!(x == x)) return 0u;
  if (x <= 0.0f) return 0u;
  if (x >= 4294967296.0f) return 4294967295u;
  return (u32)x;
}
template <class T> struct conv;
template <> struct conv<f32> { template <class S> static f32 c(S s) { return to_f32(s); } };
template <> struct conv<i32> { template <class S> static i32 c(S s) { return to_i32(s); } };
template <> struct conv<u32> { template <class S> static u32 c(S s) { return to_u32(s); } };
template <> struct conv<bool> { template <class S> static bool c(S s) { return (bool)s; } };
// abstract-int literals (C++ int) and other arithmetic types
template <class T, class S> static inline T cv(S s) { return conv<T>::c(s); }
template <> inline f32 cv<f32, double>(double s) { return (f32)s; }

// ---- vectors ------------------------------------------------------------
template <class T> struct vec2;
template <class T> struct vec3;
template <class T> struct vec4;

// v.swz<i, j, ...>() builds a vector from components i, j, ... (WGSL swizzles).
#define RT_SWIZZLES                                                                                \
  template <int A, int B> vec2<T> swz() const { return vec2<T>((*this)[A], (*this)[B]); }            \
  template <int A, int B, int C> vec3<T> swz() const { return vec3<T>((*this)[A], (*this)[B], (*this)[C]); } \
  template <int A, int B, int C, int D> vec4<T> swz() const {                                       \
    return vec4<T>((*this)[A], (*this)[B], (*this)[C], (*this)[D]);                                  \
  }

template <class T> struct vec2 {
  T x, y;
  vec2() : x(0), y(0) {}
  template <class S> explicit vec2(S s) : x(cv<T>(s)), y(cv<T>(s)) {}
  template <class A, class B> vec2(A a, B b) : x(cv<T>(a)), y(cv<T>(b)) {}
  template <class S> vec2(const vec2<S>& v) : x(cv<T>(v.x)), y(cv<T>(v.y)) {}
  vec2(const vec2& v) = default;
  vec2& operator=(const vec2& v) = default;
  T& operator[](int64_t i) { return i == 0 ? x : y; }
  T operator[](int64_t i) const { return i == 0 ? x : y; }
  RT_SWIZZLES
};
template <class T> struct vec3 {
  T x, y, z;
  vec3() : x(0), y(0), z(0) {}
  template <class S> explicit vec3(S s) : x(cv<T>(s)), y(cv<T>(s)), z(cv<T>(s)) {}
  template <class A, class B, class C> vec3(A a, B b, C c) : x(cv<T>(a)), y(cv<T>(b)), z(cv<T>(c)) {}
  template <class S, class C> vec3(const vec2<S>& ab, C c) : x(cv<T>(ab.x)), y(cv<T>(ab.y)), z(cv<T>(c)) {}
  template <class S> vec3(const vec3<S>& v) : x(cv<T>(v.x)), y(cv<T>(v.y)), z(cv<T>(v.z)) {}
  vec3(const vec3& v) = default;
  vec3& operator=(const vec3& v) = default;
  vec2<T> xy() const { return vec2<T>(x, y); }
  vec2<T> yz() const { return vec2<T>(y, z); }
  T& operator[](int64_t i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int64_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
  RT_SWIZZLES
};
template <class T> struct vec4 {
  T x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  template <class S> explicit vec4(S s) : x(cv<T>(s)), y(cv<T>(s)), z(cv<T>(s)), w(cv<T>(s)) {}
  template <class A, class B, class C, class D>
  vec4(A a, B b, C c, D d) : x(cv<T>(a)), y(cv<T>(b)), z(cv<T>(c)), w(cv<T>(d)) {}
  template <class S, class D> vec4(const vec3<S>& v, D d) : x(cv<T>(v.x)), y(cv<T>(v.y)), z(cv<T>(v.z)), w(cv<T>(d)) {}
  template <class S, class C, class D>
  vec4(const vec2<S>& v, C c, D d) : x(cv<T>(v.x)), y(cv<T>(v.y)), z(cv<T>(c)), w(cv<T>(d)) {}
  template <class S> vec4(const vec4<S>& v) : x(cv<T>(v.x)), y(cv<T>(v.y)), z(cv<T>(v.z)), w(cv<T>(v.w)) {}
  template <class S, class R>
  vec4(const vec2<S>& a, const vec2<R>& b) : x(cv<T>(a.x)), y(cv<T>(a.y)), z(cv<T>(b.x)), w(cv<T>(b.y)) {}
  vec4(const vec4& v) = default;
  vec4& operator=(const vec4& v) = default;
  vec2<T> xy() const { return vec2<T>(x, y); }
  vec2<T> zw() const { return vec2<T>(z, w); }
  vec3<T> xyz() const { return vec3<T>(x, y, z); }
  T& operator[](int64_t i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T operator[](int64_t i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  RT_SWIZZLES
};
typedef vec2<f32> vec2f; typedef vec3<f32> vec3f; typedef vec4<f32> vec4f;
typedef vec2<i32> vec2i; typedef vec3<i32> vec3i; typedef vec4<i32> vec4i;
typedef vec2<u32> vec2u; typedef vec3<u32> vec3u; typedef vec4<u32> vec4u;

#define RT_VOP(OP)                                                                                  \
  template <class T> vec2<T> operator OP(const vec2<T>& a, const vec2<T>& b) { return vec2<T>(a.x OP b.x, a.y OP b.y); } \
  template <class T> vec3<T> operator OP(const vec3<T>& a, const vec3<T>& b) { return vec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
  template <class T> vec4<T> operator OP(const vec4<T>& a, const vec4<T>& b) { return vec4<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); } \
  template <class T, class S> vec2<T> operator OP(const vec2<T>& a, S s) { T b = cv<T>(s); return vec2<T>(a.x OP b, a.y OP b); } \
  template <class T, class S> vec3<T> operator OP(const vec3<T>& a, S s) { T b = cv<T>(s); return vec3<T>(a.x OP b, a.y OP b, a.z OP b); } \
  template <class T, class S> vec4<T> operator OP(const vec4<T>& a, S s) { T b = cv<T>(s); return vec4<T>(a.x OP b, a.y OP b, a.z OP b, a.w OP b); } \
  template <class T, class S> vec2<T> operator OP(S s, const vec2<T>& b) { T a = cv<T>(s); return vec2<T>(a OP b.x, a OP b.y); } \
  template <class T, class S> vec3<T> operator OP(S s, const vec3<T>& b) { T a = cv<T>(s); return vec3<T>(a OP b.x, a OP b.y, a OP b.z); } \
  template <class T, class S> vec4<T> operator OP(S s, const vec4<T>& b) { T a = cv<T>(s); return vec4<T>(a OP b.x, a OP b.y, a OP b.z, a OP b.w); } \
  template <class T, class S> vec2<T>& operator OP##=(vec2<T>& a, const S& b) { a = a OP b; return a; } \
  template <class T, class S> vec3<T>& operator OP##=(vec3<T>& a, const S& b) { a = a OP b; return a; } \
  template <class T, class S> vec4<T>& operator OP##=(vec4<T>& a, const S& b) { a = a OP b; return a; }
RT_VOP(+)
RT_VOP(-)
RT_VOP(*)
RT_VOP(/)
#undef RT_VOP
template <class T> vec2<T> operator-(const vec2<T>& a) { return vec2<T>(-a.x, -a.y); }
template <class T> vec3<T> operator-(const vec3<T>& a) { return vec3<T>(-a.x, -a.y, -a.z); }
template <class T> vec4<T> operator-(const vec4<T>& a) { return vec4<T>(-a.x, -a.y, -a.z, -a.w); }

// Component-wise comparisons give bool vectors (WGSL), reduced by all()/any().
#define RT_VCMP(OP)                                                                                \
  template <class T> vec2<bool> operator OP(const vec2<T>& a, const vec2<T>& b) { return vec2<bool>(a.x OP b.x, a.y OP b.y); } \
  template <class T> vec3<bool> operator OP(const vec3<T>& a, const vec3<T>& b) { return vec3<bool>(a.x OP b.x, a.y OP b.y, a.z OP b.z); }
RT_VCMP(<)
RT_VCMP(<=)
RT_VCMP(>)
RT_VCMP(>=)
#undef RT_VCMP
static inline bool all(const vec2<bool>& v) { return v.x && v.y; }
static inline bool all(const vec3<bool>& v) { return v.x && v.y && v.z; }

// mat4x4f: four columns; m * v = c0 v.x + c1 v.y + c2 v.z + c3 v.w, summed in that order.
struct mat4x4f {
  vec4<f32> c[4];
};
static inline vec4<f32> operator*(const mat4x4f& m, const vec4<f32>& v) {
  vec4<f32> r;
  r.x = m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w;
  r.y = m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w;
  r.z = m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w;
  r.w = m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w;
  return r;
}

// ---- fixed-size arrays ---------------------------------------------------
template <class T, int N> struct array {
  T a[N];
  array() { for (int i = 0; i < N; i++) a[i] = T(); }
  template <class... A> explicit array(A... xs) : a{cv_elem(xs)...} {}
  template <class S> static T cv_elem(const S& s) { return T(s); }
  static T cv_elem(int s) { return cv<T>(s); }
  static T cv_elem(double s) { return (T)s; }
  T& operator[](int64_t i) { return a[i]; }
  const T& operator[](int64_t i) const { return a[i]; }
};

// ---- storage buffers: a shared pointer binding ----------------------------
template <class T> struct storage {
  T* p = nullptr;
  T& operator[](int64_t i) const { return p[i]; }
};
// A 3-D r16float texture (the baked W17 model: body SDF and parts atlas),
// w x h x d binary16 texels, x fastest; no data = the engine's unwritten
// texture, which samples as 0.
struct texture3d {
  int w = 1, h = 1, d = 1;
  const uint16_t* p = nullptr;
};
struct sampler { int dummy = 0; };
static inline f32 half_bits_to_f32(uint16_t b) {
  const uint32_t sign = (uint32_t)(b >> 15) << 31, e = (b >> 10) & 0x1fu, m = b & 0x3ffu;
  uint32_t u;
  if (e == 0x1fu) u = sign | 0x7f800000u | (m << 13);
  else if (e != 0) u = sign | ((e + 112u) << 23) | (m << 13);
  else if (m == 0) u = sign;
  else {  // subnormal: m * 2^-24, exact in binary32
    f32 v = (f32)m * 5.9604644775390625e-8f;
    memcpy(&u, &v, 4);
    u |= sign;
  }
  f32 r;
  memcpy(&r, &u, 4);
  return r;
}
// textureSampleLevel with a linear, clamp-to-edge sampler at level 0 (the
// engine's carSamp, engine.ts:270), written out with f32 weights: texel
// coordinate c = uvw * size - 0.5, i = floor(c), t = c - i, indices clamped to
// the texture, blended along x, then y, then z with mix(a, b, t) = a (1 - t) + b t.
// (A GPU's filter hardware uses reduced-precision weights; WebGPU leaves that
// precision to the implementation.)
static inline f32 texel3(const texture3d& t, int x, int y, int z) {
  x = x < 0 ? 0 : (x >= t.w ? t.w - 1 : x);
  y = y < 0 ? 0 : (y >= t.h ? t.h - 1 : y);
  z = z < 0 ? 0 : (z >= t.d ? t.d - 1 : z);
  return half_bits_to_f32(t.p[((size_t)z * (size_t)t.h + (size_t)y) * (size_t)t.w + (size_t)x]);
}
static inline int floor_index(f32 f, int n) { return (int)(f < -1.0f ? -1.0f : (f > (f32)n ? (f32)n : f)); }
static inline vec4f textureSampleLevel(const texture3d& t, const sampler&, vec3f uvw, f32) {
  if (!t.p) return vec4f(0.0f);
  const f32 cx = uvw.x * (f32)t.w - 0.5f, cy = uvw.y * (f32)t.h - 0.5f, cz = uvw.z * (f32)t.d - 0.5f;
  const f32 fx = __builtin_floorf(cx), fy = __builtin_floorf(cy), fz = __builtin_floorf(cz);
  const f32 tx = cx - fx, ty = cy - fy, tz = cz - fz;
  const int i = floor_index(fx, t.w), j = floor_index(fy, t.h), k = floor_index(fz, t.d);
  const f32 c00 = texel3(t, i, j, k) * (1.0f - tx) + texel3(t, i + 1, j, k) * tx;
  const f32 c10 = texel3(t, i, j + 1, k) * (1.0f - tx) + texel3(t, i + 1, j + 1, k) * tx;
  const f32 c01 = texel3(t, i, j, k + 1) * (1.0f - tx) + texel3(t, i + 1, j, k + 1) * tx;
  const f32 c11 = texel3(t, i, j + 1, k + 1) * (1.0f - tx) + texel3(t, i + 1, j + 1, k + 1) * tx;
  const f32 c0 = c00 * (1.0f - ty) + c10 * ty, c1 = c01 * (1.0f - ty) + c11 * ty;
  return vec4f(c0 * (1.0f - tz) + c1 * tz, 0.0f, 0.0f, 1.0f);
}
static inline vec3u textureDimensions(const texture3d& t) { return vec3u((u32)t.w, (u32)t.h, (u32)t.d); }
// A 2-D render target read by textureLoad: w x h texels of RGBA f32 (already
// rounded to the target format by whoever wrote it).
struct texture2d {
  int w = 1, h = 1;
  const f32* p = nullptr;
};
static inline vec2u textureDimensions(const texture2d& t) { return vec2u((u32)t.w, (u32)t.h); }
// textureSample (implicit level of detail) is the rasterizer's: the driver that
// runs a fragment shader installs a hook that knows the fragment's derivatives.
typedef vec4f (*sample_hook_fn)(const texture2d&, vec2f);
inline thread_local sample_hook_fn sample_hook = nullptr;
static inline vec4f textureSample(const texture2d& t, const sampler&, vec2f uv) { return sample_hook(t, uv); }
static inline vec4f textureLoad(const texture2d& t, vec2i q, i32) {
  if (!t.p || q.x < 0 || q.y < 0 || q.x >= t.w || q.y >= t.h) return vec4f(0.0f);
  const f32* e = t.p + ((size_t)q.y * (size_t)t.w + (size_t)q.x) * 4;
  return vec4f(e[0], e[1], e[2], e[3]);
}

// ---- builtins -----------------------------------------------------------
static inline f32 abs(f32 x) { return x < 0.0f ? -x : (x == 0.0f ? 0.0f : x); }
static inline i32 abs(i32 x) { return x < 0 ? (i32)(0u - (u32)x) : x; }
template <class T> vec2<T> abs(const vec2<T>& v) { return vec2<T>(abs(v.x), abs(v.y)); }
template <class T> vec3<T> abs(const vec3<T>& v) { return vec3<T>(abs(v.x), abs(v.y), abs(v.z)); }

static inline f32 min(f32 a, f32 b) { return b < a ? b : a; }
static inline f32 max(f32 a, f32 b) { return a < b ? b : a; }
static inline i32 min(i32 a, i32 b) { return b < a ? b : a; }
static inline i32 max(i32 a, i32 b) { return a < b ? b : a; }
static inline u32 min(u32 a, u32 b) { return b < a ? b : a; }
static inline u32 max(u32 a, u32 b) { return a < b ? b : a; }
template <class T> vec2<T> min(const vec2<T>& a, const vec2<T>& b) { return vec2<T>(min(a.x, b.x), min(a.y, b.y)); }
template <class T> vec3<T> min(const vec3<T>& a, const vec3<T>& b) { return vec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <class T> vec2<T> max(const vec2<T>& a, const vec2<T>& b) { return vec2<T>(max(a.x, b.x), max(a.y, b.y)); }
template <class T> vec3<T> max(const vec3<T>& a, const vec3<T>& b) { return vec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
template <class T> T clamp(const T& e, const T& lo, const T& hi) { return min(max(e, lo), hi); }

static inline f32 mix(f32 a, f32 b, f32 t) { return a * (1.0f - t) + b * t; }
template <class T> vec2<T> mix(const vec2<T>& a, const vec2<T>& b, f32 t) { return vec2<T>(mix(a.x, b.x, t), mix(a.y, b.y, t)); }
template <class T> vec3<T> mix(const vec3<T>& a, const vec3<T>& b, f32 t) { return vec3<T>(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t)); }
template <class T> vec4<T> mix(const vec4<T>& a, const vec4<T>& b, f32 t) { return vec4<T>(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t), mix(a.w, b.w, t)); }
static inline f32 smoothstep(f32 lo, f32 hi, f32 x) {
  f32 t = clamp((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
template <class T> static inline T select(const T& f, const T& t, bool c) { return c ? t : f; }

static inline f32 sqrt(f32 x) { return __builtin_sqrtf(x); }
static inline f32 floor(f32 x) { return __builtin_floorf(x); }
template <class T> vec2<T> floor(const vec2<T>& v) { return vec2<T>(floor(v.x), floor(v.y)); }
template <class T> vec3<T> floor(const vec3<T>& v) { return vec3<T>(floor(v.x), floor(v.y), floor(v.z)); }
static inline f32 round(f32 x) { return __builtin_rintf(x); }
static inline f32 sign(f32 x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
static inline f32 sin(f32 x) { return wtm::sinf(x); }
static inline f32 cos(f32 x) { return wtm::cosf(x); }
static inline f32 atan(f32 x) { return wtm::atanf(x); }
static inline f32 atan2(f32 y, f32 x) { return wtm::atan2f(y, x); }
static inline f32 exp(f32 x) { return wtm::expf(x); }
static inline f32 exp2(f32 x) { return wtm::exp2f(x); }
static inline f32 log2(f32 x) { return wtm::log2f(x); }
static inline f32 pow(f32 x, f32 y) { return wtm::powf(x, y); }
static inline vec3f pow(const vec3f& x, const vec3f& y) { return vec3f(pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)); }
static inline vec3f sqrt(const vec3f& v) { return vec3f(sqrt(v.x), sqrt(v.y), sqrt(v.z)); }
// fract(e) = e - floor(e)
static inline f32 fract(f32 x) { return x - floor(x); }
static inline vec2f fract(const vec2f& v) { return vec2f(fract(v.x), fract(v.y)); }
static inline vec3f fract(const vec3f& v) { return vec3f(fract(v.x), fract(v.y), fract(v.z)); }
// step(edge, x) = 1 if edge <= x else 0
static inline f32 step(f32 edge, f32 x) { return edge <= x ? 1.0f : 0.0f; }

static inline f32 dot(const vec2f& a, const vec2f& b) { return a.x * b.x + a.y * b.y; }
static inline f32 dot(const vec3f& a, const vec3f& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f32 dot(const vec4f& a, const vec4f& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline f32 length(f32 x) { return abs(x); }
template <class V> static inline f32 length(const V& v) { return sqrt(dot(v, v)); }
// normalize(e) = e / length(e), one IEEE division per component
template <class V> static inline V normalize(const V& v) { return v / length(v); }
// reflect(e1, e2) = e1 - 2 dot(e2, e1) e2;  distance(a, b) = length(a - b)
static inline vec3f reflect(const vec3f& e1, const vec3f& e2) { return e1 - (2.0f * dot(e2, e1)) * e2; }
template <class V> static inline f32 distance(const V& a, const V& b) { return length(a - b); }

template <class T> static inline T bitcast(f32 x) { T r; memcpy(&r, &x, 4); return r; }

// Atomics: relaxed read-modify-write on plain memory, two's-complement wrap.
template <class T> static inline T atomicAdd(T* p, T v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
template <class T> static inline void atomicStore(T* p, T v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }
template <class T> static inline T atomicLoad(T* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }

}  // namespace rt

#define RT_USING                                                                                 \
  using rt::f32; using rt::i32; using rt::u32; using rt::atomic; using rt::array; using rt::storage; \
  using rt::vec2f; using rt::vec3f; using rt::vec4f; using rt::vec2i; using rt::vec3i; using rt::vec4i; \
  using rt::vec2u; using rt::vec3u; using rt::vec4u; using rt::texture3d; using rt::sampler;         \
  using rt::to_f32; using rt::to_i32; using rt::to_u32; using rt::abs; using rt::min; using rt::max; \
  using rt::clamp; using rt::mix; using rt::smoothstep; using rt::select; using rt::sqrt;            \
  using rt::floor; using rt::normalize; using rt::round; using rt::sign; using rt::sin; using rt::cos; using rt::atan;    \
  using rt::dot; using rt::length; using rt::bitcast; using rt::atomicAdd; using rt::atomicStore;   \
  using rt::atomicLoad; using rt::textureSampleLevel; using rt::textureDimensions;                 \
  using rt::texture2d; using rt::textureLoad; using rt::mat4x4f; using rt::all; using rt::atan2;    \
  using rt::exp; using rt::exp2; using rt::log2; using rt::pow; using rt::fract; using rt::step;     \
  using rt::reflect; using rt::distance; using rt::textureSample;
