// TEST INFRASTRUCTURE ONLY - never linked into the product library.
//
// Runs the reference's own simulation shaders (translated to C++ by
// oracle/wgsl_translate.py into oracle/_ref/wgsl_modules.inc) the way
// src/engine/engine.ts dispatches them:
//   constructor buffers        engine.ts:234-242 (fA, fB, solid, emit, fields, tA, tB, forces)
//   reset()                    engine.ts:371-381 (LBM_INIT on fA and fB, temps zeroed)
//   setShape() -> voxelize     engine.ts:426-470
//   frame() LBM loop           engine.ts:708-712 (lbm[s % 2] ping-pong, then heat[0], heat[1])
//   maybeReadForces()          engine.ts:739-761 (read, then zero the accumulator)
// Every dispatch is 1-D with workgroups of 128 invocations; the invocations of
// one workgroup run phase by phase (split at workgroupBarrier), workgroups run
// in parallel on host threads.  Output of this file goes to oracle/_ref/.
#include "wgsl_runtime.hpp"
#include "_ref/wgsl_modules.inc"
#include "../f1-wind-tunnel_gb300/csrc/wt_texfilter.h"

#include <math.h>
#include <stdlib.h>

#include <algorithm>
#include <string.h>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Ref {
  uint32_t nx, ny, nz, n;
  float origin[3], h;
  float uIn = 0.0925f, tau0 = 0.508f, smag = 0.17f;  // engine.ts:110,249
  float cool = 0.004f, diffuse = 0.04f;               // engine.ts:263
  std::vector<float> fA, fB, emit, tA, tB, profile;
  std::vector<uint32_t> solid;
  std::vector<rt::vec4f> fields;
  int32_t forces[12];
};

template <class F>
void dispatch(uint32_t n, int nphases, F run) {
  const int64_t nwg = (n + 127) / 128;
#pragma omp parallel for schedule(static)
  for (int64_t wg = 0; wg < nwg; wg++)
    for (int ph = 0; ph < nphases; ph++)
      for (uint32_t li = 0; li < 128; li++) run(ph, rt::vec3u((uint32_t)(wg * 128 + li), 0u, 0u), li);
}

template <class S>
void set_shape(S& s, const uint32_t* w) {
  float f[24];
  memcpy(f, w, sizeof(f));
  s.kind = w[0]; s.profileMode = w[1]; s.pw = w[2]; s.ph = w[3];
  s.frontFlap = f[4]; s.rearMain = f[5]; s.rearFlap = f[6]; s.rideH = f[7];
  s.aoa = f[8]; s.width = f[9]; s.axisY = f[10]; s.pScale = f[11];
  s.pOrigin = rt::vec2f(f[12], f[13]); s.heatBrakes = f[14]; s.heatEngine = f[15];
  s.heatRad = f[16]; s.frontWing = f[17]; s.rearWing = f[18]; s.sidepod = f[19];
  s.cover = f[20]; s.nose = f[21]; s.rearRide = f[22]; s.duct = f[23];
}

// The W17 model set by wtr_set_car (engine.ts:410-421 setCarModel + the rig of
// setShape, :450-462); absent until set.
struct CarModel {
  std::vector<uint16_t> sdf, parts;
  int pdims[3] = {1, 1, 1};
  float rig[87 * 4];
  bool set = false;
};
CarModel g_car;

// Rig uniform: the car model's, or as the engine creates it before any W17
// model is loaded (engine.ts:273-277).
template <class R>
void set_rig(R& rig) {
  rig = R{};
  if (g_car.set) {
    const float* f = g_car.rig;
    auto v4 = [&](int i) { return rt::vec4f(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]); };
    for (int i = 0; i < 71; i++) rig.front[i] = v4(i);
    rig.hinges = v4(71); rig.angles = v4(72); rig.extra = v4(73); rig.fly = v4(74);
    for (int i = 0; i < 12; i++) rig.grids[i] = v4(75 + i);
    return;
  }
  rig.extra = rt::vec4f(0.0f, 1.0f, 0.0f, 0.0f);
  rig.fly = rt::vec4f(0.0f, 0.0f, 1.0f, 1.0f);
  for (int i = 0; i < 12; i++) rig.grids[i] = rt::vec4f(0.0f, 0.0f, 0.0f, 1.0f);
}
template <class M>
void set_car_textures(M& carSdf, M& carParts) {
  if (g_car.set) {
    carSdf = rt::texture3d{368, 84, 67, g_car.sdf.data()};
    carParts = rt::texture3d{g_car.pdims[0], g_car.pdims[1], g_car.pdims[2], g_car.parts.data()};
  } else {
    carSdf = rt::texture3d{};
    carParts = rt::texture3d{};
  }
}

template <class G>
void set_grid(G& g, const Ref& r) {
  g.dims = rt::vec3u(r.nx, r.ny, r.nz);
  g.n = r.n;
  g.origin = rt::vec3f(r.origin[0], r.origin[1], r.origin[2]);
  g.h = r.h;
}

void run_init(Ref& r, std::vector<float>& fa) {
  namespace M = m_lbm_init;
  set_grid(M::grid, r);
  M::sim.uIn = r.uIn; M::sim.tau0 = r.tau0; M::sim.smag = r.smag; M::sim.pad = 0.0f;
  M::fa.p = fa.data();
  M::fields.p = r.fields.data();
  dispatch(r.n, M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

void run_step(Ref& r, std::vector<float>& fin, std::vector<float>& fout) {
  namespace M = m_lbm_step;
  set_grid(M::grid, r);
  M::sim.uIn = r.uIn; M::sim.tau0 = r.tau0; M::sim.smag = r.smag; M::sim.pad = 0.0f;
  M::fin.p = fin.data();
  M::fout.p = fout.data();
  M::solid.p = r.solid.data();
  M::fields.p = r.fields.data();
  M::forces.p = r.forces;
  M::emit.p = r.emit.data();
  dispatch(r.n, M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

void run_heat(Ref& r, std::vector<float>& tin, std::vector<float>& tout, float dt) {
  namespace M = m_heat;
  set_grid(M::grid, r);
  M::heat.dt = dt; M::heat.cool = r.cool; M::heat.diffuse = r.diffuse; M::heat.pad = 0.0f;
  M::fields.p = r.fields.data();
  M::emit.p = r.emit.data();
  M::tin.p = tin.data();
  M::tout.p = tout.data();
  dispatch(r.n, M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

}  // namespace

extern "C" {

void* wtr_new(int nx, int ny, int nz, float ox, float oy, float oz, float h) {
  Ref* r = new Ref();
  r->nx = nx; r->ny = ny; r->nz = nz; r->n = (uint32_t)nx * ny * nz;
  r->origin[0] = ox; r->origin[1] = oy; r->origin[2] = oz; r->h = h;
  size_t n = r->n;
  r->fA.assign(n * 19, 0.0f); r->fB.assign(n * 19, 0.0f);
  r->solid.assign(n, 0u); r->emit.assign(n, 0.0f);
  r->fields.assign(n, rt::vec4f(0.0f));
  r->tA.assign(n, 0.0f); r->tB.assign(n, 0.0f);
  r->profile.assign(256 * 128, 10.0f);  // engine.ts:245-246
  memset(r->forces, 0, sizeof(r->forces));
  return r;
}

void wtr_free(void* p) { delete (Ref*)p; }

void wtr_set_sim(void* p, float uIn, float tau0, float smag) {
  Ref* r = (Ref*)p; r->uIn = uIn; r->tau0 = tau0; r->smag = smag;
}

void wtr_set_heat(void* p, float cool, float diffuse) {
  Ref* r = (Ref*)p; r->cool = cool; r->diffuse = diffuse;
}

void wtr_reset(void* p) {
  Ref* r = (Ref*)p;
  run_init(*r, r->fA);
  run_init(*r, r->fB);
  std::fill(r->tA.begin(), r->tA.end(), 0.0f);
  std::fill(r->tB.begin(), r->tB.end(), 0.0f);
}

// shape: the 24 32-bit words of the Shape uniform (wgsl.ts:9-18) in declaration order.
void wtr_voxelize(void* p, const uint32_t* w) {
  Ref* r = (Ref*)p;
  namespace M = m_voxelize;
  set_grid(M::grid, *r);
  set_shape(M::shape, w);
  set_rig(M::rig);
  set_car_textures(M::carSdf, M::carParts);
  M::profile.p = r->profile.data();
  M::solid.p = r->solid.data();
  M::emit.p = r->emit.data();
  dispatch(r->n, M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

void wtr_set_solid(void* p, const uint32_t* solid, const float* emit) {
  Ref* r = (Ref*)p;
  memcpy(r->solid.data(), solid, r->n * 4);
  memcpy(r->emit.data(), emit, r->n * 4);
}

// engine.ts:710 - n LBM dispatches, lbm[s % 2]; the engine always issues an even count.
void wtr_steps(void* p, int n) {
  Ref* r = (Ref*)p;
  for (int s = 0; s < n; s++) {
    if (s % 2 == 0) run_step(*r, r->fA, r->fB);
    else run_step(*r, r->fB, r->fA);
  }
}

// engine.ts:711-712 with the heat uniform dt of engine.ts:659-660.
void wtr_heat(void* p, float dt) {
  Ref* r = (Ref*)p;
  run_heat(*r, r->tA, r->tB, dt);
  run_heat(*r, r->tB, r->tA, dt);
}

void wtr_read(void* p, float* fields, uint32_t* solid, float* emit, float* temps, float* fa,
              int32_t* forces, int reset_forces) {
  Ref* r = (Ref*)p;
  size_t n = r->n;
  if (fields) memcpy(fields, r->fields.data(), n * 16);
  if (solid) memcpy(solid, r->solid.data(), n * 4);
  if (emit) memcpy(emit, r->emit.data(), n * 4);
  if (temps) memcpy(temps, r->tA.data(), n * 4);
  if (fa) memcpy(fa, r->fA.data(), n * 19 * 4);
  if (forces) memcpy(forces, r->forces, sizeof(r->forces));
  if (reset_forces) memset(r->forces, 0, sizeof(r->forces));
}

void wtr_write_state(void* p, const float* fa, const float* fields, const float* temps) {
  Ref* r = (Ref*)p;
  size_t n = r->n;
  if (fa) memcpy(r->fA.data(), fa, n * 19 * 4);
  if (fields) memcpy(r->fields.data(), fields, n * 16);
  if (temps) memcpy(r->tA.data(), temps, n * 4);
}

// ---- field consumers: FIELD_SAMPLING, PARTICLES_SIM (wgsl.ts:324-366, 516-594) and
// STREAM_SIM (render-wgsl.ts:520-576) over caller-provided fields / temps.
// g: dims (3 u32), origin (3 f32), h.  view: uIn, vReal, cpMin, cpMax, tMin, tMax,
// speedMax, vortMax.
extern "C++" {
template <class G>
static void set_grid_ext(G& g, const uint32_t* dims, const float* origin, float h) {
  g.dims = rt::vec3u(dims[0], dims[1], dims[2]);
  g.n = dims[0] * dims[1] * dims[2];
  g.origin = rt::vec3f(origin[0], origin[1], origin[2]);
  g.h = h;
}
template <class V>
static void set_view(V& v, const float* w) {
  v.uIn = w[0]; v.vReal = w[1]; v.cpMin = w[2]; v.cpMax = w[3];
  v.tMin = w[4]; v.tMax = w[5]; v.speedMax = w[6]; v.vortMax = w[7];
}
}  // extern "C++"

// sampleFlow at n points: out[6k..6k+5] = (ux, uy, uz, rho, temp, fluid); vort[k] = vorticityAt.
void wtr_sample_flow(const uint32_t* dims, const float* origin, float h, const float* fields, const float* temps,
                     const float* pts, uint32_t n, float* out, float* vort) {
  namespace M = m_particles;
  set_grid_ext(M::grid, dims, origin, h);
  M::fields.p = (rt::vec4f*)fields;
  M::temps.p = (float*)temps;
  for (uint32_t k = 0; k < n; k++) {
    const rt::vec3f p(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]);
    const M::Sample sm = M::sampleFlow(p);
    out[6 * k + 0] = sm.u.x; out[6 * k + 1] = sm.u.y; out[6 * k + 2] = sm.u.z;
    out[6 * k + 3] = sm.rho; out[6 * k + 4] = sm.temp; out[6 * k + 5] = sm.fluid;
    if (vort) vort[k] = M::vorticityAt(p);
  }
}

// One dispatch of the particle pass over `parts` (count x 8 floats: pos.xyzw, vel.xyzw).
// ps: count, spawnMode, colorMode, frame, scatter, rakeRows, rakeCols (u32);
// pf: dt, life, spawnMin[3], spawnMax[3].
void wtr_particles(const uint32_t* dims, const float* origin, float h, const float* fields, const float* temps,
                   const uint32_t* ps, const float* pf, const float* view, float* parts) {
  namespace M = m_particles;
  set_grid_ext(M::grid, dims, origin, h);
  M::fields.p = (rt::vec4f*)fields;
  M::temps.p = (float*)temps;
  M::parts.p = (M::Particle*)parts;
  M::psim.count = ps[0]; M::psim.spawnMode = ps[1]; M::psim.colorMode = ps[2]; M::psim.frame = ps[3];
  M::psim.scatter = ps[4]; M::psim.rakeRows = ps[5]; M::psim.rakeCols = ps[6];
  M::psim.dt = pf[0]; M::psim.life = pf[1];
  M::psim.spawnMin = rt::vec3f(pf[2], pf[3], pf[4]);
  M::psim.spawnMax = rt::vec3f(pf[5], pf[6], pf[7]);
  M::psim.pad = 0.0f;
  set_view(M::view, view);
  dispatch(ps[0], M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

// The streamline pass: lines x steps points (x, y, z, colour or -1) into pts.
// ss: lines, steps, seedMode, colorMode, rows, cols, perEmitter, emitters (u32);
// sf: seedMin[3], seedMax[3], stepLen, time; emit: 8 x (x, y, z, radius).
void wtr_streamlines(const uint32_t* dims, const float* origin, float h, const float* fields, const float* temps,
                     const uint32_t* ss, const float* sf, const float* emit, const float* view, float* pts) {
  namespace M = m_stream;
  set_grid_ext(M::grid, dims, origin, h);
  M::fields.p = (rt::vec4f*)fields;
  M::temps.p = (float*)temps;
  M::pts.p = (rt::vec4f*)pts;
  M::stream.lines = ss[0]; M::stream.steps = ss[1]; M::stream.seedMode = ss[2]; M::stream.colorMode = ss[3];
  M::stream.rows = ss[4]; M::stream.cols = ss[5]; M::stream.perEmitter = ss[6]; M::stream.emitters = ss[7];
  M::stream.seedMin = rt::vec3f(sf[0], sf[1], sf[2]);
  M::stream.seedMax = rt::vec3f(sf[3], sf[4], sf[5]);
  M::stream.stepLen = sf[6]; M::stream.time = sf[7];
  for (int i = 0; i < 8; i++) M::emitters.e[i] = rt::vec4f(emit[4 * i], emit[4 * i + 1], emit[4 * i + 2], emit[4 * i + 3]);
  set_view(M::view, view);
  dispatch(ss[0], M::cs_main_nphases, [](int ph, rt::vec3u gid, uint32_t li) { M::cs_main_run(ph, gid, li); });
}

// ---- render passes (src/engine/render-wgsl.ts; order and targets engine.ts:290-327, 714-725)
//
// Render targets are RGBA f32 arrays, row-major from the top row.  rgba16float
// targets hold values rounded to binary16 (nearest, ties to even) on every
// write, as the GPU stores them; the rgba8unorm output holds
// round(clamp(x, 0, 1) * 255).  A full-screen pass invokes fs_main once per
// texel of its target with uv = ((x + 0.5) / w, (y + 0.5) / h).
extern "C++" {
static float round_half(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  const uint32_t a = u & 0x7fffffffu;
  const float sgn = (u >> 31) ? -1.0f : 1.0f;
  if (a >= 0x7f800000u) return x;                     // inf, NaN
  if (a >= 0x477ff000u) return sgn * __builtin_inff();  // >= 65520 rounds past 65504
  if (a <= 0x33000000u) return sgn * 0.0f;            // <= 2^-25 rounds to zero
  const int e = (int)(a >> 23) - 127;
  const int q = e >= -14 ? e - 10 : -24;              // binary16 quantum at this magnitude
  const float scale = __builtin_ldexpf(1.0f, q);
  float ax;
  memcpy(&ax, &a, 4);
  return sgn * (__builtin_rintf(ax / scale) * scale);
}
static uint8_t unorm8(float x) {
  if (!(x == x)) return 0;
  const float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
  return (uint8_t)__builtin_rintf(c * 255.0f);
}
static rt::vec3f v3(const float* p) { return rt::vec3f(p[0], p[1], p[2]); }
static rt::mat4x4f mat4(const float* m) {
  rt::mat4x4f r;
  for (int c = 0; c < 4; c++) r.c[c] = rt::vec4f(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
  return r;
}
template <class F>
static void full_screen(int w, int h, F fs) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const rt::vec2f uv(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      fs(x, y, uv);
    }
}
}  // extern "C++"

// RENDER fs_main (render-wgsl.ts:288-398) into the rgba16float scene target.
// shape: Shape words; cam: the Cam uniform (20 words: pos, tanHalf, fwd, aspect,
// right, time, up, roadSpeed, jitter.xy, pad, pad); look: the Look uniform (24
// words, render-wgsl.ts:12-19); view: View (8 floats).
void wtr_render_scene(const uint32_t* dims, const float* origin, float h, const float* fields, const float* temps,
                      const uint32_t* shape, const float* cam, const uint32_t* look, const float* view, int w,
                      int hgt, float* scene) {
  namespace M = m_render;
  static std::vector<float> profile(256 * 128, 10.0f);  // engine.ts:245-246
  set_grid_ext(M::grid, dims, origin, h);
  M::fields.p = (rt::vec4f*)fields;
  M::temps.p = (float*)temps;
  M::profile.p = profile.data();
  set_shape(M::shape, shape);
  set_rig(M::rig);
  set_car_textures(M::carSdf, M::carParts);
  M::cam.pos = v3(cam); M::cam.tanHalf = cam[3];
  M::cam.fwd = v3(cam + 4); M::cam.aspect = cam[7];
  M::cam.right = v3(cam + 8); M::cam.time = cam[11];
  M::cam.up = v3(cam + 12); M::cam.roadSpeed = cam[15];
  M::cam.jitter = rt::vec2f(cam[16], cam[17]); M::cam.pad0 = 0.0f; M::cam.pad1 = 0.0f;
  float lf[24];
  memcpy(lf, look, sizeof(lf));
  M::Look& L = M::look;
  L.bmin = v3(lf); L.surfMode = look[3];
  L.bmax = v3(lf + 4); L.palette = look[7];
  L.paint = v3(lf + 8); L.carbonBody = look[11];
  L.accent = v3(lf + 12); L.isF1 = look[15];
  L.sliceAxis = look[16]; L.slicePos = lf[17]; L.sliceAlpha = lf[18]; L.showFlow = look[19];
  L.meshMode = look[20]; L.cooling = look[21]; L.pad1 = 0u; L.pad2 = 0u;
  set_view(M::view, view);
  full_screen(w, hgt, [&](int x, int y, rt::vec2f uv) {
    const rt::vec4f c = M::fs_main(uv);
    float* o = scene + ((size_t)y * w + x) * 4;
    o[0] = round_half(c.x); o[1] = round_half(c.y); o[2] = round_half(c.z); o[3] = round_half(c.w);
  });
}

// The car G-buffer RENDER reads with look.meshMode != 0 (engine.ts:297-303):
// w x h RGBA f32 texels holding the stored values (albedo and normal-distance
// rounded to binary16, material c / 255).  NULL unbinds (textureLoad gives 0).
void wtr_set_gbuffer(int w, int hgt, const float* albedo, const float* normal, const float* material) {
  namespace M = m_render;
  M::gAlbedo = rt::texture2d{w, hgt, albedo};
  M::gNormal = rt::texture2d{w, hgt, normal};
  M::gMaterial = rt::texture2d{w, hgt, material};
}

// The W17 model (engine.ts:410-421 setCarModel and the rig uniform of setShape):
// sdf 368 x 84 x 67 binary16 (x fastest), parts pd[0] x pd[1] x pd[2] binary16,
// rig the 87 vec4 of the Rig uniform (car-model.ts:60-69).  sdf == NULL clears it.
void wtr_set_car(const uint16_t* sdf, const uint16_t* parts, const uint32_t* pd, const float* rig) {
  if (!sdf) {
    g_car = CarModel{};
    return;
  }
  g_car.sdf.assign(sdf, sdf + 368 * 84 * 67);
  for (int i = 0; i < 3; i++) g_car.pdims[i] = (int)pd[i];
  g_car.parts.assign(parts, parts + (size_t)pd[0] * pd[1] * pd[2]);
  memcpy(g_car.rig, rig, sizeof(g_car.rig));
  g_car.set = true;
}

// sceneSdf (the RENDER module's copy of the SDF chunk) at n points: out[2k], out[2k+1].
void wtr_scene_sdf(const uint32_t* shape, const float* pts, uint32_t n, float* out) {
  namespace M = m_render;
  set_shape(M::shape, shape);
  set_rig(M::rig);
  set_car_textures(M::carSdf, M::carParts);
  static std::vector<float> profile(256 * 128, 10.0f);
  M::profile.p = profile.data();
  for (uint32_t k = 0; k < n; k++) {
    const rt::vec2f r = M::sceneSdf(rt::vec3f(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]));
    out[2 * k] = r.x;
    out[2 * k + 1] = r.y;
  }
}

// TAA fs_main (render-wgsl.ts:456-518): cur and hist are w x h rgba16float targets;
// taa: the Taa uniform (32 floats: prevViewProj column-major, camPos, tanHalf,
// fwd, aspect, right, blend, up, pad).
void wtr_taa(const float* cur, const float* hist, int w, int hgt, const float* taa, float* out) {
  namespace M = m_taa;
  M::cur = rt::texture2d{w, hgt, cur};
  M::hist = rt::texture2d{w, hgt, hist};
  M::taa.prevViewProj = mat4(taa);
  M::taa.camPos = v3(taa + 16); M::taa.tanHalf = taa[19];
  M::taa.fwd = v3(taa + 20); M::taa.aspect = taa[23];
  M::taa.right = v3(taa + 24); M::taa.blend = taa[27];
  M::taa.up = v3(taa + 28); M::taa.pad = 0.0f;
  full_screen(w, hgt, [&](int x, int y, rt::vec2f uv) {
    const rt::vec4f c = M::fs_main(uv);
    float* o = out + ((size_t)y * w + x) * 4;
    o[0] = round_half(c.x); o[1] = round_half(c.y); o[2] = round_half(c.z); o[3] = round_half(c.w);
  });
}

// BLUR fs_main (render-wgsl.ts:401-418) from an sw x sh source into a dw x dh
// target; blur: dir.xy, spacing, gain.
void wtr_blur(const float* src, int sw, int sh, const float* blur, int dw, int dh, float* out) {
  namespace M = m_blur;
  M::src = rt::texture2d{sw, sh, src};
  M::blur.dir = rt::vec2f(blur[0], blur[1]); M::blur.spacing = blur[2]; M::blur.gain = blur[3];
  full_screen(dw, dh, [&](int x, int y, rt::vec2f uv) {
    const rt::vec4f c = M::fs_main(uv);
    float* o = out + ((size_t)y * dw + x) * 4;
    o[0] = round_half(c.x); o[1] = round_half(c.y); o[2] = round_half(c.z); o[3] = round_half(c.w);
  });
}

// PRESENT fs_main (render-wgsl.ts:420-454) into the w x h rgba8unorm output:
// scene (the resolved history), glow (gw x gh) and bloom (bw x bh) targets;
// post: bloom, exposure, pad, pad.
void wtr_present(const float* scene, int w, int hgt, const float* glow, int gw, int gh, const float* bloom, int bw,
                 int bh, const float* post, uint8_t* out) {
  namespace M = m_present;
  M::scene = rt::texture2d{w, hgt, scene};
  M::glow = rt::texture2d{gw, gh, glow};
  M::bloomTex = rt::texture2d{bw, bh, bloom};
  M::post.bloom = post[0]; M::post.exposure = post[1]; M::post.pad0 = 0.0f; M::post.pad1 = 0.0f;
  full_screen(w, hgt, [&](int x, int y, rt::vec2f uv) {
    const rt::vec4f c = M::fs_main(uv);
    uint8_t* o = out + ((size_t)y * w + x) * 4;
    o[0] = unorm8(c.x); o[1] = unorm8(c.y); o[2] = unorm8(c.z); o[3] = unorm8(c.w);
  });
}

// ---- the glow pass: PARTICLES_DRAW (wgsl.ts:597-659) and STREAM_DRAW
// (render-wgsl.ts:578-645) instanced quads, additively blended (one, one) into
// the cleared rgba16float glow target (engine.ts:719-722).
//
// Fixed-function stages, as the WebGPU pipeline defines them, in the form both
// this model and the device rasterizer evaluate:
//   * triangle-list topology: vertices 0-2 and 3-5 of each instance;
//   * clip -> NDC n = c.xyz / c.w; framebuffer X = (n.x * 0.5 + 0.5) * W,
//     Y = (0.5 - n.y * 0.5) * H;
//   * area A = (X1-X0)(Y2-Y0) - (X2-X0)(Y1-Y0); none or NaN -> no fragments;
//   * pixel (px, py) is covered when its centre P = (px+0.5, py+0.5) gives edge
//     values e0 = (X2-X1)(Py-Y1) - (Y2-Y1)(Px-X1), e1 = (X0-X2)(Py-Y2) - (Y0-Y2)(Px-X2),
//     e2 = (X1-X0)(Py-Y0) - (Y1-Y0)(Px-X0), multiplied by sign(A), all >= 0,
//     where an edge value of exactly 0 counts only for an edge whose direction
//     (b - a, times sign(A)) has dy > 0, or dy == 0 and dx < 0 (so a pixel on an
//     edge two triangles share is drawn once);
//   * depth clip: z = b0 n0.z + b1 n1.z + b2 n2.z outside [0, 1] -> discarded;
//   * perspective-correct varyings: with b_k = e_k / |A| and q_k = b_k / c_k.w,
//     weight k = q_k / (q0 + q1 + q2), varying = w0 a0 + w1 a1 + w2 a2;
//   * fragment position.xy = P.
// Blending: the (one, one) sum is formed exactly, each fragment's value rounded
// to a multiple of 2^-32 into 64-bit integers, and the total rounded once to
// binary16 (the WebGPU blend unit's intermediate precision is the
// implementation's; an exact sum makes the result independent of fragment order).
extern "C++" {
struct Vtx {
  float X, Y, nz, iw;    // framebuffer position, NDC depth, 1 / clip w
  float a[6];            // varyings: colour (4), side, dist
};
static bool raster_edge_owned(float dx, float dy) { return dy > 0.0f || (dy == 0.0f && dx < 0.0f); }
template <class FS>
static void raster_triangle(const Vtx* v, int W, int H, FS shade) {
  const float A = (v[1].X - v[0].X) * (v[2].Y - v[0].Y) - (v[2].X - v[0].X) * (v[1].Y - v[0].Y);
  if (!(A > 0.0f) && !(A < 0.0f)) return;
  const float sg = A > 0.0f ? 1.0f : -1.0f;
  const float aa = A > 0.0f ? A : -A;
  const float minx = std::min(v[0].X, std::min(v[1].X, v[2].X)), maxx = std::max(v[0].X, std::max(v[1].X, v[2].X));
  const float miny = std::min(v[0].Y, std::min(v[1].Y, v[2].Y)), maxy = std::max(v[0].Y, std::max(v[1].Y, v[2].Y));
  const int x0 = (int)ceilf(std::min(std::max(minx - 0.5f, 0.0f), (float)W));
  const int x1 = (int)floorf(std::max(std::min(maxx - 0.5f, (float)(W - 1)), -1.0f));
  const int y0 = (int)ceilf(std::min(std::max(miny - 0.5f, 0.0f), (float)H));
  const int y1 = (int)floorf(std::max(std::min(maxy - 0.5f, (float)(H - 1)), -1.0f));
  const bool own0 = raster_edge_owned((v[2].X - v[1].X) * sg, (v[2].Y - v[1].Y) * sg);
  const bool own1 = raster_edge_owned((v[0].X - v[2].X) * sg, (v[0].Y - v[2].Y) * sg);
  const bool own2 = raster_edge_owned((v[1].X - v[0].X) * sg, (v[1].Y - v[0].Y) * sg);
  for (int py = y0; py <= y1; py++)
    for (int px = x0; px <= x1; px++) {
      const float Px = (float)px + 0.5f, Py = (float)py + 0.5f;
      const float e0 = ((v[2].X - v[1].X) * (Py - v[1].Y) - (v[2].Y - v[1].Y) * (Px - v[1].X)) * sg;
      const float e1 = ((v[0].X - v[2].X) * (Py - v[2].Y) - (v[0].Y - v[2].Y) * (Px - v[2].X)) * sg;
      const float e2 = ((v[1].X - v[0].X) * (Py - v[0].Y) - (v[1].Y - v[0].Y) * (Px - v[0].X)) * sg;
      if (e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) continue;
      if ((e0 == 0.0f && !own0) || (e1 == 0.0f && !own1) || (e2 == 0.0f && !own2)) continue;
      const float b0 = e0 / aa, b1 = e1 / aa, b2 = e2 / aa;
      const float z = b0 * v[0].nz + b1 * v[1].nz + b2 * v[2].nz;
      if (!(z >= 0.0f && z <= 1.0f)) continue;
      const float q0 = b0 * v[0].iw, q1 = b1 * v[1].iw, q2 = b2 * v[2].iw;
      const float qs = q0 + q1 + q2;
      const float w0 = q0 / qs, w1 = q1 / qs, w2 = q2 / qs;
      float a[6];
      for (int k = 0; k < 6; k++) a[k] = w0 * v[0].a[k] + w1 * v[1].a[k] + w2 * v[2].a[k];
      shade(px, py, Px, Py, z, a);
    }
}
static Vtx make_vtx(rt::vec4f pos, int W, int H, const float* a) {
  Vtx v;
  const float nx = pos.x / pos.w, ny = pos.y / pos.w;
  v.nz = pos.z / pos.w;
  v.X = (nx * 0.5f + 0.5f) * (float)W;
  v.Y = (0.5f - ny * 0.5f) * (float)H;
  v.iw = 1.0f / pos.w;
  for (int k = 0; k < 6; k++) v.a[k] = a[k];
  return v;
}
static void accumulate(std::vector<int64_t>& acc, int W, int px, int py, rt::vec4f c) {
  int64_t* o = acc.data() + ((size_t)py * W + px) * 4;
  o[0] += llrint((double)c.x * 4294967296.0);
  o[1] += llrint((double)c.y * 4294967296.0);
  o[2] += llrint((double)c.z * 4294967296.0);
  o[3] += llrint((double)c.w * 4294967296.0);
}
}  // extern "C++"

// scene: the w x h rgba16float scene target (its alpha is the hit distance);
// parts: count x 8 floats; pdraw: the PDraw uniform (28 words); n_pinst
// instances (0 = no particle draw).  pts: lines x steps x 4 floats; sdraw: the
// SDraw uniform (28 words); n_sinst instances (0 = no streamline draw).
void wtr_glow(const float* scene, int w, int hgt, const float* parts, const uint32_t* pdraw, uint32_t n_pinst,
              const float* pts, const uint32_t* sdraw, uint32_t n_sinst, float* glow) {
  std::vector<int64_t> acc((size_t)w * hgt * 4, 0);
  if (n_pinst) {
    namespace M = m_pdraw;
    float f[28];
    memcpy(f, pdraw, sizeof(f));
    M::pd.viewProj = mat4(f); M::pd.camPos = v3(f + 16); M::pd.width = f[19];
    M::pd.res = rt::vec2f(f[20], f[21]); M::pd.trail = f[22]; M::pd.alpha = f[23];
    M::pd.count = pdraw[24]; M::pd.palette = pdraw[25]; M::pd.fadeIn = f[26]; M::pd.pad = 0.0f;
    M::parts.p = (M::Particle*)parts;
    M::scene = rt::texture2d{w, hgt, scene};
    for (uint32_t ii = 0; ii < n_pinst; ii++)
      for (int t = 0; t < 2; t++) {
        Vtx v[3];
        for (int k = 0; k < 3; k++) {
          const M::VOut o = M::vs_main((uint32_t)(3 * t + k), ii);
          const float a[6] = {o.color.x, o.color.y, o.color.z, o.color.w, o.side, o.dist};
          v[k] = make_vtx(o.pos, w, hgt, a);
        }
        raster_triangle(v, w, hgt, [&](int px, int py, float Px, float Py, float z, const float* a) {
          M::VOut in{};
          in.pos = rt::vec4f(Px, Py, z, 1.0f);
          in.color = rt::vec4f(a[0], a[1], a[2], a[3]);
          in.side = a[4];
          in.dist = a[5];
          M::rt_discarded = false;
          const rt::vec4f c = M::fs_main(in);
          if (!M::rt_discarded) accumulate(acc, w, px, py, c);
        });
      }
  }
  if (n_sinst) {
    namespace M = m_sdraw;
    float f[28];
    memcpy(f, sdraw, sizeof(f));
    M::sd.viewProj = mat4(f); M::sd.camPos = v3(f + 16); M::sd.width = f[19];
    M::sd.res = rt::vec2f(f[20], f[21]); M::sd.time = f[22]; M::sd.intensity = f[23];
    M::sd.lines = sdraw[24]; M::sd.steps = sdraw[25]; M::sd.palette = sdraw[26]; M::sd.pulse = f[27];
    M::pts.p = (rt::vec4f*)pts;
    M::scene = rt::texture2d{w, hgt, scene};
    for (uint32_t ii = 0; ii < n_sinst; ii++)
      for (int t = 0; t < 2; t++) {
        Vtx v[3];
        for (int k = 0; k < 3; k++) {
          const M::VOut o = M::vs_main((uint32_t)(3 * t + k), ii);
          const float a[6] = {o.color.x, o.color.y, o.color.z, 0.0f, o.side, o.dist};
          v[k] = make_vtx(o.pos, w, hgt, a);
        }
        raster_triangle(v, w, hgt, [&](int px, int py, float Px, float Py, float z, const float* a) {
          M::VOut in{};
          in.pos = rt::vec4f(Px, Py, z, 1.0f);
          in.color = rt::vec3f(a[0], a[1], a[2]);
          in.side = a[4];
          in.dist = a[5];
          M::rt_discarded = false;
          const rt::vec4f c = M::fs_main(in);
          if (!M::rt_discarded) accumulate(acc, w, px, py, c);
        });
      }
  }
  for (size_t i = 0; i < acc.size(); i++) glow[i] = round_half((float)((double)acc[i] * 0x1p-32));
}

// ---- the car mesh G-buffer pass: MESH_DRAW (render-wgsl.ts:647-760) draws of
// MeshCar.record (mesh-car.ts:205-207) into the cleared G-buffer (engine.ts:
// 297-303, 716), run the way the WebGPU pipeline defines it: draws in order,
// triangles in order, each fragment tested against the depth buffer as it is
// at that moment.  Fixed-function stages:
//   * triangle list of vertex_index 0..count-1 of each draw, cull none;
//   * clipping to z >= 0 in clip space: the corners in order, a corner with
//     z >= 0 kept, an edge whose ends lie on both sides adding the point at
//     t = z_a / (z_a - z_b) with every output a + t (b - a); the polygon is drawn
//     as the fan (0, 1, 2), (0, 2, 3); a part with a corner at w <= 0 is dropped;
//   * viewport, coverage, tie rule, depth clip and perspective-correct
//     varyings as in the glow pass above;
//   * depth32float cleared to 1.  Opaque draws: 'less', depth written.  Blended
//     draws (the decals): the bias depthBias * 2^(e - 23) + slopeScale * m with
//     depthBias -4, slopeScale -1 (mesh-car.ts:150), e the exponent of the
//     largest |z| of the part and m = max(|dz/dX|, |dz/dY|) from its plane, then
//     clamped to [0, 1], 'less-equal', depth not written;
//   * textureSample's derivatives: the uv differences across the fragment's
//     2 x 2 pixel quad (from its top-left pixel to the right and down
//     neighbours), the varyings there extrapolated from the same triangle;
//     filtering as the texture filter header defines it;
//   * targets: albedo and normalDist rgba16float, material rgba8unorm (the
//     output rounding above).  Blended draws write albedo only, with
//     DECAL_BLEND (mesh-car.ts:22-25): rgb = src.rgb * src.a + dst.rgb *
//     (1 - src.a), alpha kept; the other targets have an empty write mask.
extern "C++" {
struct MVtx {
  float X, Y, nz, iw;  // framebuffer position, NDC depth, 1 / clip w
  float a[8];          // world xyz, normal xyz, uv
};
struct MeshTri {
  MVtx v[3];
  float A, sg, aa;
  // barycentric weights (b) and perspective weights (w) at framebuffer point P
  void edges(float Px, float Py, float* e) const {
    e[0] = ((v[2].X - v[1].X) * (Py - v[1].Y) - (v[2].Y - v[1].Y) * (Px - v[1].X)) * sg;
    e[1] = ((v[0].X - v[2].X) * (Py - v[2].Y) - (v[0].Y - v[2].Y) * (Px - v[2].X)) * sg;
    e[2] = ((v[1].X - v[0].X) * (Py - v[0].Y) - (v[1].Y - v[0].Y) * (Px - v[0].X)) * sg;
  }
  void varyings(const float* e, float* out) const {
    const float b0 = e[0] / aa, b1 = e[1] / aa, b2 = e[2] / aa;
    const float q0 = b0 * v[0].iw, q1 = b1 * v[1].iw, q2 = b2 * v[2].iw;
    const float qs = q0 + q1 + q2;
    const float w0 = q0 / qs, w1 = q1 / qs, w2 = q2 / qs;
    for (int k = 0; k < 8; k++) out[k] = w0 * v[0].a[k] + w1 * v[1].a[k] + w2 * v[2].a[k];
  }
};
struct MeshTexture {
  std::vector<std::vector<uint8_t>> data;
  std::vector<wtx::Level> levels;
};
// halveRgba (mesh-car.ts:30-44)
static std::vector<uint8_t> halve_rgba(const std::vector<uint8_t>& src, int w, int h, int* ow, int* oh) {
  const int nw = std::max(1, w >> 1), nh = std::max(1, h >> 1);
  std::vector<uint8_t> out((size_t)nw * nh * 4);
  for (int y = 0; y < nh; y++) {
    const int y0 = std::min(h - 1, y * 2), y1 = std::min(h - 1, y * 2 + 1);
    for (int x = 0; x < nw; x++) {
      const int x0 = std::min(w - 1, x * 2), x1 = std::min(w - 1, x * 2 + 1);
      for (int c = 0; c < 4; c++)
        out[((size_t)y * nw + x) * 4 + c] =
            (uint8_t)((src[((size_t)y0 * w + x0) * 4 + c] + src[((size_t)y0 * w + x1) * 4 + c] +
                       src[((size_t)y1 * w + x0) * 4 + c] + src[((size_t)y1 * w + x1) * 4 + c] + 2) >> 2);
    }
  }
  *ow = nw;
  *oh = nh;
  return out;
}
static thread_local const MeshTexture* g_mesh_tex = nullptr;
static thread_local float g_mesh_deriv[4];  // du/dx, dv/dx, du/dy, dv/dy of the current fragment
static rt::vec4f mesh_sample(const rt::texture2d&, rt::vec2f uv) {
  const wtx::Rgba c = wtx::sample(g_mesh_tex->levels.data(), (int)g_mesh_tex->levels.size(), uv.x, uv.y,
                                  g_mesh_deriv[0], g_mesh_deriv[1], g_mesh_deriv[2], g_mesh_deriv[3]);
  return rt::vec4f(c.r, c.g, c.b, c.a);
}
static MVtx mesh_vtx(const m_mesh::VOut& o, int W, int H) {
  MVtx v;
  const float nx = o.pos.x / o.pos.w, ny = o.pos.y / o.pos.w;
  v.nz = o.pos.z / o.pos.w;
  v.X = (nx * 0.5f + 0.5f) * (float)W;
  v.Y = (0.5f - ny * 0.5f) * (float)H;
  v.iw = 1.0f / o.pos.w;
  const float a[8] = {o.world.x, o.world.y, o.world.z, o.normal.x, o.normal.y, o.normal.z, o.uv.x, o.uv.y};
  for (int k = 0; k < 8; k++) v.a[k] = a[k];
  return v;
}
static m_mesh::VOut vout_lerp(const m_mesh::VOut& a, const m_mesh::VOut& b, float t) {
  auto l = [t](float x, float y) { return x + t * (y - x); };
  m_mesh::VOut o{};
  o.pos = rt::vec4f(l(a.pos.x, b.pos.x), l(a.pos.y, b.pos.y), l(a.pos.z, b.pos.z), l(a.pos.w, b.pos.w));
  o.world = rt::vec3f(l(a.world.x, b.world.x), l(a.world.y, b.world.y), l(a.world.z, b.world.z));
  o.normal = rt::vec3f(l(a.normal.x, b.normal.x), l(a.normal.y, b.normal.y), l(a.normal.z, b.normal.z));
  o.uv = rt::vec2f(l(a.uv.x, b.uv.x), l(a.uv.y, b.uv.y));
  return o;
}
// the part of triangle c[0..3) with z >= 0, as a polygon of 0, 3 or 4 corners
static int clip_near(const m_mesh::VOut* c, m_mesh::VOut* out) {
  int n = 0;
  for (int i = 0; i < 3; i++) {
    const m_mesh::VOut& a = c[i];
    const m_mesh::VOut& b = c[(i + 1) % 3];
    const bool ina = a.pos.z >= 0.0f, inb = b.pos.z >= 0.0f;
    if (ina) out[n++] = a;
    if (ina != inb) out[n++] = vout_lerp(a, b, a.pos.z / (a.pos.z - b.pos.z));
  }
  return n;
}
}  // extern "C++"

// The G-buffer pass.  verts: nv x 8 floats (position, u, normal, v: the
// vertex buffer of mesh-car.ts:63-77); indices[ni]; vparts: the part tags,
// four per u32 (mesh-car.ts:88-91).  draws: nd records of 16 words in record
// order: the MeshMat uniform (12 words: color, metal, rough, coat, alphaCut,
// emissive, hasTex, isBody, firstIndex), vertex count, texture index (-1: none),
// blend flag, unused.  textures: ntex level-0 RGBA8 images tex[i] of
// tex_dims[2i] x tex_dims[2i+1]; their mip chains are made here.  cam: the
// MeshCam uniform (24 words); rig: the 87 vec4 of the Rig uniform.  The targets
// (w x h; albedo and normal as RGBA f32 holding binary16 values, material RGBA8,
// depth f32) are read and written: the caller clears them.
void wtr_mesh_gbuffer(int w, int hgt, const float* verts, uint32_t nv, const uint32_t* indices, uint32_t ni,
                      const uint32_t* vparts, const uint32_t* draws, int nd, int ntex, const uint32_t* tex_dims,
                      const uint8_t* const* tex, const float* cam, const float* rig, float* albedo, float* normal,
                      uint8_t* material, float* depth) {
  namespace M = m_mesh;
  (void)nv;
  (void)ni;
  std::vector<MeshTexture> texs((size_t)std::max(ntex, 0));
  for (int t = 0; t < ntex; t++) {
    int tw = (int)tex_dims[2 * t], th = (int)tex_dims[2 * t + 1];
    const int n_levels = (int)floor(log2((double)std::max(tw, th))) + 1;
    texs[t].data.emplace_back(tex[t], tex[t] + (size_t)tw * th * 4);
    std::vector<int> ws{tw}, hs{th};
    for (int m = 1; m < n_levels; m++) {
      int nw, nh;
      texs[t].data.push_back(halve_rgba(texs[t].data.back(), ws.back(), hs.back(), &nw, &nh));
      ws.push_back(nw);
      hs.push_back(nh);
    }
    for (int m = 0; m < n_levels; m++) texs[t].levels.push_back(wtx::Level{texs[t].data[m].data(), ws[m], hs[m]});
  }
  float cf[24];
  memcpy(cf, cam, sizeof(cf));
  M::cam.viewProj = mat4(cf);
  M::cam.camPos = v3(cf + 16); M::cam.rideH = cf[19];
  M::cam.jitter = rt::vec2f(cf[20], cf[21]); M::cam.rake = cf[22]; M::cam.baseRide = cf[23];
  {
    auto v4 = [&](int i) { return rt::vec4f(rig[4 * i], rig[4 * i + 1], rig[4 * i + 2], rig[4 * i + 3]); };
    for (int i = 0; i < 71; i++) M::rig.front[i] = v4(i);
    M::rig.hinges = v4(71); M::rig.angles = v4(72); M::rig.extra = v4(73); M::rig.fly = v4(74);
    for (int i = 0; i < 12; i++) M::rig.grids[i] = v4(75 + i);
  }
  M::verts.p = (rt::vec4f*)verts;
  M::indices.p = (uint32_t*)indices;
  M::vparts.p = (uint32_t*)vparts;
  rt::sample_hook = mesh_sample;
  for (int d = 0; d < nd; d++) {
    const uint32_t* r = draws + 16 * d;
    float f[12];
    memcpy(f, r, sizeof(f));
    M::mat.color = rt::vec4f(f[0], f[1], f[2], f[3]);
    M::mat.metal = f[4]; M::mat.rough = f[5]; M::mat.coat = f[6]; M::mat.alphaCut = f[7];
    M::mat.emissive = f[8]; M::mat.hasTex = f[9]; M::mat.isBody = f[10]; M::mat.firstIndex = r[11];
    const uint32_t count = r[12];
    const int texi = (int32_t)r[13];
    const bool blend = r[14] != 0u;
    g_mesh_tex = (texi >= 0 && texi < ntex) ? &texs[texi] : nullptr;
    for (uint32_t t = 0; t + 2 < count; t += 3) {
      M::VOut c[3], poly[4];
      for (int k = 0; k < 3; k++) c[k] = M::vs_main(t + (uint32_t)k);
      const int np = clip_near(c, poly);
      for (int s = 0; s + 2 < np; s++) {
        const M::VOut* tri[3] = {&poly[0], &poly[s + 1], &poly[s + 2]};
        if (!(tri[0]->pos.w > 0.0f && tri[1]->pos.w > 0.0f && tri[2]->pos.w > 0.0f)) continue;
        MeshTri T;
        for (int k = 0; k < 3; k++) T.v[k] = mesh_vtx(*tri[k], w, hgt);
        const MVtx* v = T.v;
        T.A = (v[1].X - v[0].X) * (v[2].Y - v[0].Y) - (v[2].X - v[0].X) * (v[1].Y - v[0].Y);
        if (!(T.A > 0.0f) && !(T.A < 0.0f)) continue;
        T.sg = T.A > 0.0f ? 1.0f : -1.0f;
        T.aa = T.A > 0.0f ? T.A : -T.A;
        float bias = 0.0f;
        if (blend) {
          const float dzdx = ((v[1].nz - v[0].nz) * (v[2].Y - v[0].Y) - (v[2].nz - v[0].nz) * (v[1].Y - v[0].Y)) / T.A;
          const float dzdy = ((v[2].nz - v[0].nz) * (v[1].X - v[0].X) - (v[1].nz - v[0].nz) * (v[2].X - v[0].X)) / T.A;
          const float m = std::max(fabsf(dzdx), fabsf(dzdy));
          const float zmax = std::max(fabsf(v[0].nz), std::max(fabsf(v[1].nz), fabsf(v[2].nz)));
          int e = 0;
          frexpf(zmax, &e);
          bias = -4.0f * ldexpf(1.0f, e - 1 - 23) + -1.0f * m;
        }
        const float minx = std::min(v[0].X, std::min(v[1].X, v[2].X)), maxx = std::max(v[0].X, std::max(v[1].X, v[2].X));
        const float miny = std::min(v[0].Y, std::min(v[1].Y, v[2].Y)), maxy = std::max(v[0].Y, std::max(v[1].Y, v[2].Y));
        const int x0 = (int)ceilf(std::min(std::max(minx - 0.5f, 0.0f), (float)w));
        const int x1 = (int)floorf(std::max(std::min(maxx - 0.5f, (float)(w - 1)), -1.0f));
        const int y0 = (int)ceilf(std::min(std::max(miny - 0.5f, 0.0f), (float)hgt));
        const int y1 = (int)floorf(std::max(std::min(maxy - 0.5f, (float)(hgt - 1)), -1.0f));
        const bool own0 = raster_edge_owned((v[2].X - v[1].X) * T.sg, (v[2].Y - v[1].Y) * T.sg);
        const bool own1 = raster_edge_owned((v[0].X - v[2].X) * T.sg, (v[0].Y - v[2].Y) * T.sg);
        const bool own2 = raster_edge_owned((v[1].X - v[0].X) * T.sg, (v[1].Y - v[0].Y) * T.sg);
        for (int py = y0; py <= y1; py++)
          for (int px = x0; px <= x1; px++) {
            const float Px = (float)px + 0.5f, Py = (float)py + 0.5f;
            float e[3];
            T.edges(Px, Py, e);
            if (e[0] < 0.0f || e[1] < 0.0f || e[2] < 0.0f) continue;
            if ((e[0] == 0.0f && !own0) || (e[1] == 0.0f && !own1) || (e[2] == 0.0f && !own2)) continue;
            const float b0 = e[0] / T.aa, b1 = e[1] / T.aa, b2 = e[2] / T.aa;
            const float z = b0 * v[0].nz + b1 * v[1].nz + b2 * v[2].nz;
            if (!(z >= 0.0f && z <= 1.0f)) continue;
            const size_t pi = (size_t)py * w + px;
            if (blend) {
              float zb = z + bias;
              zb = zb < 0.0f ? 0.0f : (zb > 1.0f ? 1.0f : zb);
              if (!(zb <= depth[pi])) continue;
            } else if (!(z < depth[pi])) {
              continue;
            }
            float a[8];
            T.varyings(e, a);
            if (g_mesh_tex) {
              const float qx = (float)(px & ~1) + 0.5f, qy = (float)(py & ~1) + 0.5f;
              float e00[3], e10[3], e01[3], a00[8], a10[8], a01[8];
              T.edges(qx, qy, e00);
              T.edges(qx + 1.0f, qy, e10);
              T.edges(qx, qy + 1.0f, e01);
              T.varyings(e00, a00);
              T.varyings(e10, a10);
              T.varyings(e01, a01);
              g_mesh_deriv[0] = a10[6] - a00[6]; g_mesh_deriv[1] = a10[7] - a00[7];
              g_mesh_deriv[2] = a01[6] - a00[6]; g_mesh_deriv[3] = a01[7] - a00[7];
            }
            M::VOut in{};
            in.pos = rt::vec4f(Px, Py, z, 1.0f);
            in.world = rt::vec3f(a[0], a[1], a[2]);
            in.normal = rt::vec3f(a[3], a[4], a[5]);
            in.uv = rt::vec2f(a[6], a[7]);
            M::rt_discarded = false;
            const M::GOut g = M::fs_main(in);
            if (M::rt_discarded) continue;
            float* al = albedo + pi * 4;
            if (blend) {
              const float sa = g.albedo.w;
              al[0] = round_half(g.albedo.x * sa + al[0] * (1.0f - sa));
              al[1] = round_half(g.albedo.y * sa + al[1] * (1.0f - sa));
              al[2] = round_half(g.albedo.z * sa + al[2] * (1.0f - sa));
              continue;
            }
            al[0] = round_half(g.albedo.x); al[1] = round_half(g.albedo.y);
            al[2] = round_half(g.albedo.z); al[3] = round_half(g.albedo.w);
            float* nd4 = normal + pi * 4;
            nd4[0] = round_half(g.normalDist.x); nd4[1] = round_half(g.normalDist.y);
            nd4[2] = round_half(g.normalDist.z); nd4[3] = round_half(g.normalDist.w);
            uint8_t* m8 = material + pi * 4;
            m8[0] = unorm8(g.material.x); m8[1] = unorm8(g.material.y);
            m8[2] = unorm8(g.material.z); m8[3] = unorm8(g.material.w);
            depth[pi] = z;
          }
      }
    }
  }
  rt::sample_hook = nullptr;
  g_mesh_tex = nullptr;
}

int wtr_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
