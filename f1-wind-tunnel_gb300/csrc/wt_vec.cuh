// Small float vectors and the WGSL builtins in the form the reference shaders
// define them (min/max by comparison, clamp = min(max()), mix(a, b, t) =
// a (1 - t) + b t, smoothstep with a correctly rounded division, dot summed
// x, y, z in order, length = sqrt(dot), float -> int truncating and saturating),
// shared by the voxelizer, the field consumers and the renderer.  Every helper
// is a fixed sequence of IEEE operations; the units that use them are built
// with -fmad=false so that results match the CPU models bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wt {
namespace {

struct V2 { float x, y; };
struct V3 { float x, y, z; };
__host__ __device__ __forceinline__ V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V2 operator*(V2 a, float s) { return v2(a.x * s, a.y * s); }

// WGSL builtin definitions (min, max, abs, clamp, mix, smoothstep, length).
__device__ __forceinline__ float mn(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float mx(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float ab(float x) { return x < 0.0f ? -x : (x == 0.0f ? 0.0f : x); }
__device__ __forceinline__ float clmp(float e, float lo, float hi) { return mn(mx(e, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ V2 mix2(V2 a, V2 b, float t) { return v2(mixf(a.x, b.x, t), mixf(a.y, b.y, t)); }
__device__ __forceinline__ float sstep(float lo, float hi, float x) {
  const float t = clmp(__fdiv_rn(x - lo, hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len2(V2 a) { return __fsqrt_rn(dot2(a, a)); }
__device__ __forceinline__ float len3(V3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ uint32_t variant(float v) {  // u32(v + 0.5), saturating
  const float t = v + 0.5f;
  return (t == t && t > 0.0f) ? __float2uint_rz(t) : 0u;
}
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ V3 normalize3(V3 a) { return divs(a, len3(a)); }
__device__ __forceinline__ float wmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float wmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float wclamp(float e, float lo, float hi) { return wmin(wmax(e, lo), hi); }
__device__ __forceinline__ int iclamp(int e, int lo, int hi) {
  const int m = e < lo ? lo : e;
  return hi < m ? hi : m;
}
__device__ __forceinline__ float wabs(float x) { return x < 0.0f ? -x : (x == 0.0f ? 0.0f : x); }
__device__ __forceinline__ float wmix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ int to_i32(float x) {
  if (!(x == x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int)0x80000000u;
  return (int)x;
}

}  // namespace
}  // namespace wt
