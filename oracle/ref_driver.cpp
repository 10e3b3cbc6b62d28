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

#include <stdlib.h>
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
  float f[24];
  memcpy(f, w, sizeof(f));
  M::Shape& s = M::shape;
  s.kind = w[0]; s.profileMode = w[1]; s.pw = w[2]; s.ph = w[3];
  s.frontFlap = f[4]; s.rearMain = f[5]; s.rearFlap = f[6]; s.rideH = f[7];
  s.aoa = f[8]; s.width = f[9]; s.axisY = f[10]; s.pScale = f[11];
  s.pOrigin = rt::vec2f(f[12], f[13]); s.heatBrakes = f[14]; s.heatEngine = f[15];
  s.heatRad = f[16]; s.frontWing = f[17]; s.rearWing = f[18]; s.sidepod = f[19];
  s.cover = f[20]; s.nose = f[21]; s.rearRide = f[22]; s.duct = f[23];
  // Rig uniform as the engine creates it before any W17 model is loaded (engine.ts:273-277).
  M::rig = M::Rig{};
  M::rig.extra = rt::vec4f(0.0f, 1.0f, 0.0f, 0.0f);
  M::rig.fly = rt::vec4f(0.0f, 0.0f, 1.0f, 1.0f);
  for (int i = 0; i < 12; i++) M::rig.grids[i] = rt::vec4f(0.0f, 0.0f, 0.0f, 1.0f);
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

int wtr_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
