// The reference's field sampling on the device: cellIdx, sampleFlow and
// vorticityAt (FIELD_SAMPLING, src/engine/wgsl.ts:324-366) and the VIEW
// colour values (wgsl.ts:430-457), shared by the field consumers and the
// renderer.  Operation order follows the WGSL text (units built with
// -fmad=false), so results are bit-identical to the reference's shaders run
// on the CPU.
#pragma once
#include "wt_fields.h"
#include "wt_vec.cuh"

namespace wt {
namespace {

struct Sample {
  V3 u;
  float rho, temp, fluid;
};

// cellIdx (wgsl.ts:325-329): the clamped cell index.
__device__ __forceinline__ uint32_t cell_idx(const FieldGrid& g, int x, int y, int z) {
  const int qx = iclamp(x, 0, (int)g.nx - 1), qy = iclamp(y, 0, (int)g.ny - 1), qz = iclamp(z, 0, (int)g.nz - 1);
  return (uint32_t)qx + g.nx * ((uint32_t)qy + g.ny * (uint32_t)qz);
}

// sampleFlow (wgsl.ts:332-357): trilinear over the fluid cells of the 8 corners,
// z mirrored about the symmetry plane.
__device__ Sample sample_flow(const FieldGrid& g, V3 pw) {
  const float zs = (pw.z < 0.0f) ? -1.0f : 1.0f;
  const V3 p = v3(pw.x, pw.y, wabs(pw.z));
  const V3 gg = v3((p.x - g.ox) / g.h - 0.5f, (p.y - g.oy) / g.h - 0.5f, (p.z - g.oz) / g.h - 0.5f);
  const int i0x = to_i32(floorf(gg.x)), i0y = to_i32(floorf(gg.y)), i0z = to_i32(floorf(gg.z));
  const V3 f = v3(gg.x - (float)i0x, gg.y - (float)i0y, gg.z - (float)i0z);
  float ax = 0.0f, ay = 0.0f, az = 0.0f, aw = 0.0f, tacc = 0.0f, wsum = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
    int cz = i0z + oz;
    if (cz < 0) cz = -cz - 1;
    const uint32_t id = cell_idx(g, i0x + ox, i0y + oy, cz);
    const float4 v = __ldg(g.fields + id);
    const float w = ((ox == 1) ? f.x : 1.0f - f.x) * ((oy == 1) ? f.y : 1.0f - f.y) * ((oz == 1) ? f.z : 1.0f - f.z);
    if (v.w > 0.0f) {
      ax = ax + v.x * w; ay = ay + v.y * w; az = az + v.z * w; aw = aw + v.w * w;
      tacc = tacc + __ldg(g.temps + id) * w;
      wsum = wsum + w;
    }
  }
  Sample s;
  if (wsum < 1e-5f) {
    s.u = v3(0.0f, 0.0f, 0.0f);
    s.rho = 1.0f;
    s.temp = 0.0f;
    s.fluid = 0.0f;
    return s;
  }
  s.u = v3(ax / wsum, ay / wsum, (az / wsum) * zs);
  s.rho = aw / wsum;
  s.temp = tacc / wsum;
  s.fluid = wsum;
  return s;
}

// vorticityAt (wgsl.ts:359-366): central differences of sampleFlow at +-h.
__device__ float vorticity_at(const FieldGrid& g, V3 p) {
  const float e = g.h;
  const V3 dx0 = sample_flow(g, sub(p, v3(e, 0.0f, 0.0f))).u, dx1 = sample_flow(g, add(p, v3(e, 0.0f, 0.0f))).u;
  const V3 dy0 = sample_flow(g, sub(p, v3(0.0f, e, 0.0f))).u, dy1 = sample_flow(g, add(p, v3(0.0f, e, 0.0f))).u;
  const V3 dz0 = sample_flow(g, sub(p, v3(0.0f, 0.0f, e))).u, dz1 = sample_flow(g, add(p, v3(0.0f, 0.0f, e))).u;
  const V3 w = mul(v3((dy1.z - dy0.z) - (dz1.y - dz0.y), (dz1.x - dz0.x) - (dx1.z - dx0.z),
                      (dx1.y - dx0.y) - (dy1.x - dy0.x)),
                   0.5f);
  return len3(w);
}

// VIEW helpers (wgsl.ts:435-457)
__device__ float rho_ref(const FieldGrid& g) {
  const float r = __ldg(g.fields + cell_idx(g, 6, (int)g.ny - 6, (int)g.nz - 6)).w;
  return (r > 0.5f) ? r : 1.0f;
}
__device__ float pressure_coef(const FieldGrid& g, const ViewArgs& v, const Sample& s) {
  return (s.rho - rho_ref(g)) / 3.0f / (0.5f * v.uIn * v.uIn);
}
__device__ float field_value(const FieldGrid& g, const ViewArgs& v, uint32_t id, const Sample& s, V3 p) {
  switch (id) {
    case 1u: return (pressure_coef(g, v, s) - v.cpMin) / (v.cpMax - v.cpMin);
    case 2u: {
      const float cp = pressure_coef(g, v, s);
      const float t = s.temp + cp * 0.5f * v.vReal * v.vReal / 1005.0f;
      return (t - v.tMin) / (v.tMax - v.tMin);
    }
    case 3u: return vorticity_at(g, p) / (v.uIn * v.vortMax);
    case 4u: return wclamp((1.0f - s.u.x / v.uIn) / 0.9f, 0.0f, 1.0f);
    default: return len3(s.u) / (v.uIn * v.speedMax);
  }
}

}  // namespace
}  // namespace wt
