/* wt_napi.c - Node N-API addon exposing libwt to the reference's TypeScript host
 * (src/engine/engine.ts).  Build next to src/engine/ with node-gyp and the
 * binding.gyp beside this file (include path to libwt's include/, -lwt).
 *
 * Every call takes the handle `create` returned (an external that destroys the
 * context when the garbage collector frees it) and maps one engine call:
 *   create        new AeroEngine's buffers (engine.ts:226-345)      wt_create
 *   reset         reset() (engine.ts:371-381)                        wt_reset
 *   setSim        syncSim() (engine.ts:497-501)                      wt_set_sim
 *   setShape      setShape() -> VOXELIZE (engine.ts:426-470)         wt_voxelize
 *   step          frame()'s compute pass (engine.ts:708-712)         wt_step
 *   readForces    maybeReadForces() (engine.ts:739-761)              wt_read_forces
 *   readForcesAsync / collectForces: its asynchronous readback       wt_read_forces_async / wt_forces_collect
 *   debugRead     debugRead() (engine.ts:763-768)                    wt_read_fields
 *   save / load   checkpoint and resume (no reference counterpart)   wt_save / wt_load
 *   resetFrom     warm start from a coarse (u, rho) field            wt_reset_from
 *   render* / mesh*: the headless render passes and the car mesh     wt_render_* / wt_mesh_*
 * Typed arrays pass the engine's uniforms byte for byte (Shape, Sim, Cam, Look,
 * View, Taa, Post, MeshCam, Rig); errors throw with wt_last_error's text. */
#include <node_api.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "wt.h"

#define MAXARGS 8

typedef struct {
  napi_value a[MAXARGS];
  size_t n;
} Args;

static Args args(napi_env env, napi_callback_info info) {
  Args r;
  r.n = MAXARGS;
  memset(r.a, 0, sizeof(r.a));
  napi_get_cb_info(env, info, &r.n, r.a, NULL, NULL);
  return r;
}

static napi_value fail(napi_env env, const wt_ctx* c, int rc) {
  char msg[512];
  const char* text = wt_last_error(c);
  snprintf(msg, sizeof(msg), "libwt error %d: %s", rc, text ? text : "");
  napi_throw_error(env, NULL, msg);
  return NULL;
}

static void* handle(napi_env env, napi_value v) {
  void* p = NULL;
  napi_get_value_external(env, v, &p);
  return p;
}

static void* typed(napi_env env, napi_value v, size_t* bytes) {
  void* p = NULL;
  size_t n = 0;
  napi_typedarray_type t = napi_uint8_array;
  napi_get_typedarray_info(env, v, &t, &n, &p, NULL, NULL);
  if (bytes) {
    size_t elem = 1;
    if (t == napi_int16_array || t == napi_uint16_array) elem = 2;
    if (t == napi_int32_array || t == napi_uint32_array || t == napi_float32_array) elem = 4;
    if (t == napi_float64_array || t == napi_bigint64_array || t == napi_biguint64_array) elem = 8;
    *bytes = n * elem;
  }
  return p;
}

static double num(napi_env env, napi_value v) {
  double d = 0.0;
  napi_get_value_double(env, v, &d);
  return d;
}

static napi_value number(napi_env env, double d) {
  napi_value v = NULL;
  napi_create_double(env, d, &v);
  return v;
}

static void destroy_ctx(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  wt_destroy((wt_ctx*)data);
}

/* create(nx, ny, nz, [ox, oy, oz, h], sim Float32Array(12) | null) -> handle */
static napi_value Create(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_grid g;
  g.nx = (uint32_t)num(env, a.a[0]);
  g.ny = (uint32_t)num(env, a.a[1]);
  g.nz = (uint32_t)num(env, a.a[2]);
  size_t bytes = 0;
  const float* o = (const float*)typed(env, a.a[3], &bytes);
  if (!o || bytes < 16) {
    napi_throw_error(env, NULL, "create: origin and cell size must be a Float32Array(4)");
    return NULL;
  }
  g.origin[0] = o[0];
  g.origin[1] = o[1];
  g.origin[2] = o[2];
  g.h = o[3];
  /* the engine's defaults (engine.ts:249,263; wgsl.ts:260,508) unless a Sim array is given */
  wt_sim s = {0.0925f, 0.508f, 0.17f, 18.0f, 0.4f, 10.0f, 0.25f, 0.004f, 0.04f, 0.35f, WT_STORE_F32, 0};
  const void* sim = a.n > 4 ? typed(env, a.a[4], &bytes) : NULL;
  if (sim && bytes >= sizeof(s)) memcpy(&s, sim, sizeof(s));
  wt_ctx* c = NULL;
  int rc = wt_create(&g, &s, &c);
  if (rc) return fail(env, NULL, rc);
  napi_value ext = NULL;
  napi_create_external(env, c, destroy_ctx, NULL, &ext);
  return ext;
}

static napi_value Reset(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  int rc = wt_reset(c);
  return rc ? fail(env, c, rc) : NULL;
}

/* setSim(handle, Float32Array(12) laid out as wt_sim) */
static napi_value SetSim(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bytes = 0;
  const void* p = typed(env, a.a[1], &bytes);
  wt_sim s;
  if (!p || bytes < sizeof(s)) {
    napi_throw_error(env, NULL, "setSim: expected a Float32Array(12)");
    return NULL;
  }
  memcpy(&s, p, sizeof(s));
  int rc = wt_set_sim(c, &s);
  return rc ? fail(env, c, rc) : NULL;
}

/* setShape(handle, Float32Array(24) with the Shape uniform as engine.ts:429-448 packs it) */
static napi_value SetShape(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bytes = 0;
  const void* p = typed(env, a.a[1], &bytes);
  wt_shape s;
  memset(&s, 0, sizeof(s));
  if (p) memcpy(&s, p, bytes < sizeof(s) ? bytes : sizeof(s));
  int rc = wt_voxelize(c, &s);
  return rc ? fail(env, c, rc) : NULL;
}

/* step(handle, evenSteps): evenSteps LBM steps and the two heat passes of a frame */
static napi_value Step(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  int32_t n = 0;
  napi_get_value_int32(env, a.a[1], &n);
  int rc = wt_step(c, n, 2, (float)n / 2.0f);
  return rc ? fail(env, c, rc) : NULL;
}

/* readForces(handle, Int32Array(12)) -> steps accumulated; the accumulator is reset */
static napi_value ReadForces(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bytes = 0;
  void* out = typed(env, a.a[1], &bytes);
  wt_forces f;
  int rc = wt_read_forces(c, &f, 1);
  if (rc) return fail(env, c, rc);
  if (out) memcpy(out, f.raw, bytes < sizeof(f.raw) ? bytes : sizeof(f.raw));
  return number(env, (double)f.steps);
}

/* readForcesAsync(handle) -> ticket; collectForces(handle, ticket, Int32Array(12)) -> steps */
static napi_value ReadForcesAsync(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  uint64_t ticket = 0;
  int rc = wt_read_forces_async(c, 1, &ticket);
  return rc ? fail(env, c, rc) : number(env, (double)ticket);
}

static napi_value CollectForces(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bytes = 0;
  void* out = typed(env, a.a[2], &bytes);
  wt_forces f;
  int rc = wt_forces_collect(c, (uint64_t)num(env, a.a[1]), &f);
  if (rc) return fail(env, c, rc);
  if (out) memcpy(out, f.raw, bytes < sizeof(f.raw) ? bytes : sizeof(f.raw));
  return number(env, (double)f.steps);
}

/* debugRead(handle, Float32Array(4n) fields, Uint32Array(n) solid, Float32Array(n) temps) */
static napi_value DebugRead(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  wt_info in;
  int rc = wt_info_get(c, &in);
  if (rc) return fail(env, c, rc);
  size_t bf = 0, bs = 0, bt = 0;
  float* fields = (float*)typed(env, a.a[1], &bf);
  uint32_t* solid = (uint32_t*)typed(env, a.a[2], &bs);
  float* temps = (float*)typed(env, a.a[3], &bt);
  if ((fields && bf < in.cells * 16) || (solid && bs < in.cells * 4) || (temps && bt < in.cells * 4)) {
    napi_throw_error(env, NULL, "debugRead: output arrays smaller than the lattice");
    return NULL;
  }
  rc = wt_read_fields(c, fields, solid, temps, NULL, NULL);
  return rc ? fail(env, c, rc) : NULL;
}

/* save(handle, path) / load(handle, path) */
static napi_value path_call(napi_env env, napi_callback_info info, int (*fn)(wt_ctx*, const char*)) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  char path[4096];
  size_t len = 0;
  napi_get_value_string_utf8(env, a.a[1], path, sizeof(path), &len);
  int rc = fn(c, path);
  return rc ? fail(env, c, rc) : NULL;
}
static napi_value Save(napi_env env, napi_callback_info info) { return path_call(env, info, wt_save); }
static napi_value Load(napi_env env, napi_callback_info info) { return path_call(env, info, wt_load); }

/* resetFrom(handle, Float32Array(4 cx cy cz) coarse (u, rho), cx, cy, cz) */
static napi_value ResetFrom(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bytes = 0;
  const float* u = (const float*)typed(env, a.a[1], &bytes);
  const uint32_t cx = (uint32_t)num(env, a.a[2]), cy = (uint32_t)num(env, a.a[3]), cz = (uint32_t)num(env, a.a[4]);
  if (!u || bytes < (size_t)cx * cy * cz * 16) {
    napi_throw_error(env, NULL, "resetFrom: coarse field smaller than cx*cy*cz*4 floats");
    return NULL;
  }
  int rc = wt_reset_from(c, u, cx, cy, cz);
  return rc ? fail(env, c, rc) : NULL;
}

/* Headless render passes.  renderCreate(handle, w, h) -> renderer;
 * renderFrame(renderer, cam, look, view, taa, cur, post): the typed arrays hold
 * the Cam / Look / View / Taa / Post uniforms exactly as engine.ts uploads them;
 * renderRead(renderer, Uint8Array(w*h*4)) copies the presented RGBA8 image. */
static void destroy_renderer(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  wt_render_destroy((wt_renderer*)data);
}

static napi_value RenderCreate(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  wt_renderer* r = NULL;
  int rc = wt_render_create(c, (uint32_t)num(env, a.a[1]), (uint32_t)num(env, a.a[2]), &r);
  if (rc) return fail(env, c, rc);
  napi_value ext = NULL;
  napi_create_external(env, r, destroy_renderer, NULL, &ext);
  return ext;
}

static napi_value RenderFrame(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_renderer* r = (wt_renderer*)handle(env, a.a[0]);
  int32_t cur = 0;
  napi_get_value_int32(env, a.a[5], &cur);
  int rc = wt_render_scene(r, (const wt_cam*)typed(env, a.a[1], NULL), (const wt_look*)typed(env, a.a[2], NULL),
                           (const wt_view*)typed(env, a.a[3], NULL));
  if (!rc) rc = wt_render_taa(r, (const wt_taa*)typed(env, a.a[4], NULL), cur);
  if (!rc) rc = wt_render_glow(r, NULL, 0, NULL, NULL, 0, NULL);
  if (!rc) rc = wt_render_bloom(r);
  if (!rc) rc = wt_render_present(r, (const wt_post*)typed(env, a.a[6], NULL), cur);
  return rc ? fail(env, NULL, rc) : NULL;
}

static napi_value RenderRead(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_renderer* r = (wt_renderer*)handle(env, a.a[0]);
  int rc = wt_render_read(r, WT_TARGET_OUTPUT, typed(env, a.a[1], NULL));
  return rc ? fail(env, NULL, rc) : NULL;
}

/* The car mesh (MeshCar.load's buffers before their upload):
 * meshCreate(handle, verts F32(n*8), indices U32, tags U8) -> mesh;
 * renderMesh(renderer, mesh, meshCam, rig, gurney) before renderFrame with
 * look.meshMode = 1. */
static void destroy_mesh(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  wt_mesh_destroy((wt_mesh*)data);
}

static napi_value MeshCreate(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_ctx* c = (wt_ctx*)handle(env, a.a[0]);
  size_t bv = 0, bi = 0, bt = 0;
  const float* v = (const float*)typed(env, a.a[1], &bv);
  const uint32_t* idx = (const uint32_t*)typed(env, a.a[2], &bi);
  const uint8_t* tags = (const uint8_t*)typed(env, a.a[3], &bt);
  wt_mesh* m = NULL;
  int rc = wt_mesh_create(c, v, (uint32_t)(bv / 32), idx, (uint32_t)(bi / 4), tags, &m);
  if (rc) return fail(env, c, rc);
  napi_value ext = NULL;
  napi_create_external(env, m, destroy_mesh, NULL, &ext);
  return ext;
}

static napi_value RenderMesh(napi_env env, napi_callback_info info) {
  Args a = args(env, info);
  wt_renderer* r = (wt_renderer*)handle(env, a.a[0]);
  wt_mesh* m = (wt_mesh*)handle(env, a.a[1]);
  bool gurney = false;
  napi_get_value_bool(env, a.a[4], &gurney);
  int rc = wt_render_mesh(r, m, (const wt_mesh_cam*)typed(env, a.a[2], NULL), (const wt_rig*)typed(env, a.a[3], NULL),
                          gurney ? 1 : 0);
  return rc ? fail(env, NULL, rc) : NULL;
}

NAPI_MODULE_INIT() {
  napi_property_descriptor d[] = {
      {"create", NULL, Create, NULL, NULL, NULL, napi_default, NULL},
      {"reset", NULL, Reset, NULL, NULL, NULL, napi_default, NULL},
      {"setSim", NULL, SetSim, NULL, NULL, NULL, napi_default, NULL},
      {"setShape", NULL, SetShape, NULL, NULL, NULL, napi_default, NULL},
      {"step", NULL, Step, NULL, NULL, NULL, napi_default, NULL},
      {"readForces", NULL, ReadForces, NULL, NULL, NULL, napi_default, NULL},
      {"readForcesAsync", NULL, ReadForcesAsync, NULL, NULL, NULL, napi_default, NULL},
      {"collectForces", NULL, CollectForces, NULL, NULL, NULL, napi_default, NULL},
      {"debugRead", NULL, DebugRead, NULL, NULL, NULL, napi_default, NULL},
      {"save", NULL, Save, NULL, NULL, NULL, napi_default, NULL},
      {"load", NULL, Load, NULL, NULL, NULL, napi_default, NULL},
      {"resetFrom", NULL, ResetFrom, NULL, NULL, NULL, napi_default, NULL},
      {"renderCreate", NULL, RenderCreate, NULL, NULL, NULL, napi_default, NULL},
      {"renderFrame", NULL, RenderFrame, NULL, NULL, NULL, napi_default, NULL},
      {"renderRead", NULL, RenderRead, NULL, NULL, NULL, napi_default, NULL},
      {"meshCreate", NULL, MeshCreate, NULL, NULL, NULL, napi_default, NULL},
      {"renderMesh", NULL, RenderMesh, NULL, NULL, NULL, napi_default, NULL},
  };
  napi_define_properties(env, exports, sizeof(d) / sizeof(d[0]), d);
  return exports;
}
