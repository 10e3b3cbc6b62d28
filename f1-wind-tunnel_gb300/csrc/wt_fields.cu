// Field consumers of the reference as CUDA kernels into headless buffers:
//   sampleFlow / vorticityAt   FIELD_SAMPLING, src/engine/wgsl.ts:324-366
//   particle pass (RK2)        PARTICLES_SIM, wgsl.ts:516-594 (+ VIEW, wgsl.ts:430-457)
//   streamline pass            STREAM_SIM, src/engine/render-wgsl.ts:520-576
// They read the (u, rho) fields of the last step call and the temperatures.
// Arithmetic follows the WGSL text operation for operation (build with
// -fmad=false) and the WGSL builtin definitions the oracle's runtime models
// (min/max/clamp by comparison, mix(a, b, t) = a (1 - t) + b t, dot summed
// x, y, z, length = sqrt(dot), normalize = componentwise division by the
// length, float -> int truncating and saturating), so results are bit-identical
// to the reference's shaders run on the CPU.  sin/cos come from wt_fmath.h.
#include <cuda_runtime.h>
#include <stdint.h>

#include "wt_fieldfn.cuh"
#include "wt_fields.h"
#include "wt_fmath.h"

namespace wt {
namespace {


// pcg hash and rand (wgsl.ts:531-539)
__device__ __forceinline__ uint32_t pcg(uint32_t v) {
  const uint32_t s = v * 747796405u + 2891336453u;
  const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
__device__ __forceinline__ float rnd(uint32_t& seed) {
  seed = pcg(seed);
  return (float)seed / 4294967296.0f;  // the reference's 4294967295.0 as f32
}

__device__ __forceinline__ V3 domain_max(const FieldGrid& g) {
  return v3(g.ox + (float)g.nx * g.h, g.oy + (float)g.ny * g.h, g.oz + (float)g.nz * g.h);
}

// spawn (wgsl.ts:542-562)
__device__ void spawn(const FieldGrid& g, const PSimArgs& ps, uint32_t i, uint32_t& seed, float4& pos, float4& vel) {
  V3 p;
  if (ps.spawnMode == 1u) {
    const uint32_t lanes = ps.rakeRows * ps.rakeCols;
    const uint32_t lane = i % lanes;
    const uint32_t row = lane / ps.rakeCols, col = lane % ps.rakeCols;
    const float fy = ((float)row + 0.5f) / (float)ps.rakeRows;
    const float fz = ((float)col + 0.5f) / (float)ps.rakeCols;
    p = v3(ps.smin[0], wmix(ps.smin[1], ps.smax[1], fy), wmix(ps.smin[2], ps.smax[2], fz));
    const float r0 = rnd(seed) * 0.12f;
    const float r1 = (rnd(seed) - 0.5f) * 0.012f;
    const float r2 = (rnd(seed) - 0.5f) * 0.012f;
    p = add(p, v3(r0, r1, r2));
  } else {
    const float r0 = rnd(seed), r1 = rnd(seed), r2 = rnd(seed);
    p = v3(ps.smin[0] + r0 * 0.15f, wmix(ps.smin[1], ps.smax[1], r1), wmix(ps.smin[2], ps.smax[2], r2));
  }
  if (ps.scatter != 0u) p.x = wmix(ps.smin[0], domain_max(g).x - g.h * 2.0f, rnd(seed));
  pos = make_float4(p.x, p.y, p.z, 0.0f);
  vel = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

// Particle pass cs_main (wgsl.ts:566-594): one thread per particle.
__global__ void particles_kernel(FieldGrid g, PSimArgs ps, ViewArgs view, float4* __restrict__ parts) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ps.count) return;
  uint32_t seed = pcg(i * 9781u + ps.frame * 6271u + 17u);
  float4 pos = parts[2 * i], vel = parts[2 * i + 1];
  const float max_life = ps.life * (0.6f + 0.4f * (float)(pcg(i * 31u) % 1000u) / 1000.0f);
  const V3 hi = domain_max(g);
  if (ps.scatter != 0u || pos.w > max_life) spawn(g, ps, i, seed, pos, vel);
  const V3 p0 = v3(pos.x, pos.y, pos.z);
  const Sample s1 = sample_flow(g, p0);
  const V3 mid = add(p0, mul(mul(mul(s1.u, g.h), ps.dt), 0.5f));
  const Sample s2 = sample_flow(g, mid);
  V3 d = mul(mul(s2.u, g.h), ps.dt);
  const float dl = len3(d);
  if (dl > g.h * 2.0f) d = mul(d, g.h * 2.0f / dl);
  V3 np = add(p0, d);
  const bool dead = np.x > hi.x - g.h * 1.5f || np.y < 0.0f || np.y > hi.y || np.z > hi.z || s2.fluid < 0.05f;
  if (dead) {
    spawn(g, ps, i, seed, pos, vel);
    pos.w = 0.0f;
    parts[2 * i] = pos;
    parts[2 * i + 1] = vel;
    return;
  }
  if (np.z < 0.0f) np.z = -np.z;
  const Sample sv = sample_flow(g, np);
  parts[2 * i] = make_float4(np.x, np.y, np.z, pos.w + 1.0f);
  parts[2 * i + 1] = make_float4(d.x, d.y, d.z, wclamp(field_value(g, view, ps.colorMode, sv, np), 0.0f, 1.0f));
}

// seedOf (render-wgsl.ts:537-550)
__device__ V3 seed_of(const StreamArgs& st, uint32_t line) {
  if (st.seedMode == 1u) {
    const uint32_t ei = min(line / st.perEmitter, st.emitters - 1u);
    const uint32_t k = line % st.perEmitter;
    const float4 e = make_float4(st.emit[ei][0], st.emit[ei][1], st.emit[ei][2], st.emit[ei][3]);
    const float a = ((float)k + 0.5f) / (float)st.perEmitter * 6.2831853f + st.time * 0.6f;
    const float ring = 0.35f + 0.65f * (float)(k % 3u) / 2.0f;
    const V3 off = mul(mul(v3(0.0f, wtm::cosf(a), wtm::sinf(a)), e.w), ring);
    return add(v3(e.x, e.y, e.z), off);
  }
  const uint32_t row = line / st.cols, col = line % st.cols;
  const float fy = ((float)row + 0.5f) / (float)st.rows;
  const float fz = ((float)col + 0.5f) / (float)st.cols;
  return v3(st.smin[0], wmix(st.smin[1], st.smax[1], fy), wmix(st.smin[2], st.smax[2], fz));
}

// Streamline pass cs_main (render-wgsl.ts:551-575): one line per block of one
// warp, lane 0 only.  A line is a chain of dependent RK2 steps, two field samples
// each; lines packed 32 to a warp would gather from 32 places per load (32 L1
// lookups per instruction) and sit on a couple of SMs.  One line per warp spreads
// the (at most a few hundred) lines over the SMs and leaves each gather a single
// lookup, so each step costs about one L1 round trip per sample.
__global__ void __launch_bounds__(32) streamlines_kernel(FieldGrid g, StreamArgs st, ViewArgs view,
                                                        float4* __restrict__ pts) {
  const uint32_t line = blockIdx.x;
  if (line >= st.lines || threadIdx.x != 0) return;
  const uint32_t base = line * st.steps;
  V3 p = seed_of(st, line);
  bool alive = true;
  const V3 hi = v3(g.ox + (float)g.nx * g.h, g.oy + (float)g.ny * g.h, g.oz + (float)g.nz * g.h);
  for (uint32_t k = 0; k < st.steps; k++) {
    if (!alive) {
      pts[base + k] = make_float4(p.x, p.y, p.z, -1.0f);
      continue;
    }
    const Sample s1 = sample_flow(g, p);
    if (s1.fluid < 0.3f || len3(s1.u) < view.uIn * 0.03f) {
      alive = false;
      pts[base + k] = make_float4(p.x, p.y, p.z, -1.0f);
      continue;
    }
    pts[base + k] = make_float4(p.x, p.y, p.z, wclamp(field_value(g, view, st.colorMode, s1, p), 0.0f, 1.0f));
    const V3 mid = add(p, mul(mul(normalize3(s1.u), st.stepLen), 0.5f));
    const Sample s2 = sample_flow(g, mid);
    V3 dir = s1.u;
    if (s2.fluid > 0.3f) dir = s2.u;
    p = add(p, mul(normalize3(dir), st.stepLen));
    if (p.x > hi.x - g.h * 3.0f || p.y < 0.01f || p.y > hi.y || wabs(p.z) > hi.z) alive = false;
  }
}

__global__ void sample_points_kernel(FieldGrid g, const float* __restrict__ pts, uint32_t n, float* __restrict__ out,
                                     float* __restrict__ vort) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const V3 p = v3(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]);
  const Sample s = sample_flow(g, p);
  out[6 * k + 0] = s.u.x; out[6 * k + 1] = s.u.y; out[6 * k + 2] = s.u.z;
  out[6 * k + 3] = s.rho; out[6 * k + 4] = s.temp; out[6 * k + 5] = s.fluid;
  if (vort) vort[k] = vorticity_at(g, p);
}

}  // namespace

cudaError_t launch_particles(const FieldGrid& g, const PSimArgs& ps, const ViewArgs& v, float4* parts, cudaStream_t s) {
  if (ps.count == 0) return cudaSuccess;
  particles_kernel<<<(ps.count + 127) / 128, 128, 0, s>>>(g, ps, v, parts);
  return cudaGetLastError();
}

cudaError_t launch_streamlines(const FieldGrid& g, const StreamArgs& st, const ViewArgs& v, float4* pts,
                               cudaStream_t s) {
  if (st.lines == 0) return cudaSuccess;
  streamlines_kernel<<<st.lines, 32, 0, s>>>(g, st, v, pts);
  return cudaGetLastError();
}

cudaError_t launch_sample_points(const FieldGrid& g, const float* pts, uint32_t n, float* out, float* vort,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  sample_points_kernel<<<(n + 127) / 128, 128, 0, s>>>(g, pts, n, out, vort);
  return cudaGetLastError();
}

}  // namespace wt
