// TEST INFRASTRUCTURE ONLY (the checker and the render workload's CPU
// baseline, never the product): the renderer's per-pixel device code
// (f1-wind-tunnel_gb300/csrc/wt_shade.cuh: render_pixel, with the scene SDF,
// field sampling and the project's math functions it calls) compiled for the
// host, so that a CPU test can compare it with the reference's RENDER shader
// translated to C++ at every pixel and at arbitrary SDF points.  CUDA
// qualifiers become plain C++ and the device intrinsics their IEEE host
// equivalents (correctly rounded division and square root, truncating float ->
// unsigned).  Built with -ffp-contract=off like the product.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include <cuda_runtime.h>

static inline float __fsqrt_rn(float x) { return sqrtf(x); }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline unsigned int __float2uint_rz(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 4294967295u;
  return (unsigned int)x;
}
template <class T>
static inline T __ldg(const T* p) { return *p; }
// system headers first: libstdc++ spells its own attributes with __noinline__
#include "wt_fields.h"
#include "wt_internal.h"
#ifndef __noinline__
#define __noinline__ __attribute__((__noinline__))
#endif

#include "wt_shade.cuh"

using namespace wt;

namespace {
// the W17 model of wthm_set_car (host copies the shading code reads)
std::vector<uint16_t> g_body, g_parts;
std::vector<float4> g_rig;
CarView g_car;
}  // namespace

extern "C" {

// The W17 model: body 368 x 84 x 67 and parts pd[0] x pd[1] x pd[2] binary16, rig
// the 87 vec4 of the Rig uniform.  body == NULL clears it.
void wthm_set_car(const uint16_t* body, const uint16_t* parts, const uint32_t* pd, const float* rig) {
  g_car = CarView{};
  if (!body) return;
  g_body.assign(body, body + (size_t)368 * 84 * 67);
  g_parts.assign(parts, parts + (size_t)pd[0] * pd[1] * pd[2]);
  g_rig.resize(87);
  memcpy(g_rig.data(), rig, 87 * sizeof(float4));
  g_car.body = g_body.data();
  g_car.parts = g_parts.data();
  for (int i = 0; i < 3; i++) g_car.pdims[i] = pd[i];
  g_car.rig = g_rig.data();
}

// The car G-buffer of the mesh pass, w x h texels (binary16 albedo and
// normal-distance, RGBA8 material) read when look.mesh_mode != 0; NULL unbinds.
static const uint16_t* g_gb_albedo = nullptr;
static const uint16_t* g_gb_normal = nullptr;
static const uint8_t* g_gb_material = nullptr;
void wthm_set_gbuffer(const uint16_t* albedo, const uint16_t* normal, const uint8_t* material) {
  g_gb_albedo = albedo;
  g_gb_normal = normal;
  g_gb_material = material;
}

// RENDER fs_main over rows [y0, y1) of a w x h target: out[(y*w + x)*4 + k] =
// colour, hit distance (rows outside the range untouched).  shape: wt_shape;
// cam/look/view: the wt_cam / wt_look / wt_view structs; fields (n x 4) and
// temps (n) of a lattice dims[3] at origin[3], spacing h.
void wthm_render(const void* shape, const void* cam_p, const void* look_p, const void* view_p, const uint32_t* dims,
                 const float* origin, float h, const float* fields, const float* temps, uint32_t w, uint32_t hgt,
                 uint32_t y0, uint32_t y1, float* out) {
  wt_cam cam;
  wt_look look;
  wt_view view;
  memcpy(&cam, cam_p, sizeof cam);
  memcpy(&look, look_p, sizeof look);
  memcpy(&view, view_p, sizeof view);
  SceneArgs a{};
  memcpy(&a.shape, shape, sizeof a.shape);
  a.g.nx = dims[0]; a.g.ny = dims[1]; a.g.nz = dims[2];
  a.g.ox = origin[0]; a.g.oy = origin[1]; a.g.oz = origin[2]; a.g.h = h;
  a.g.fields = reinterpret_cast<const float4*>(fields);
  a.g.temps = temps;
  a.view.uIn = view.u_in; a.view.vReal = view.v_real; a.view.cpMin = view.cp_min; a.view.cpMax = view.cp_max;
  a.view.tMin = view.t_min; a.view.tMax = view.t_max; a.view.speedMax = view.speed_max; a.view.vortMax = view.vort_max;
  auto f3 = [](const float* v) { return F3{v[0], v[1], v[2]}; };
  auto f3n = [](float x, float y, float z) {
    const float l = sqrtf(x * x + y * y + z * z);
    return F3{x / l, y / l, z / l};
  };
  a.pos = f3(cam.pos); a.fwd = f3(cam.fwd); a.right = f3(cam.right); a.up = f3(cam.up);
  a.tan_half = cam.tan_half; a.aspect = cam.aspect; a.time = cam.time; a.road_speed = cam.road_speed;
  a.jitter_x = cam.jitter[0]; a.jitter_y = cam.jitter[1];
  a.bmin = f3(look.bmin); a.bmax = f3(look.bmax);
  a.paint_lin = F3{wtm::powf(look.paint[0], 2.2f), wtm::powf(look.paint[1], 2.2f), wtm::powf(look.paint[2], 2.2f)};
  a.accent_lin = F3{wtm::powf(look.accent[0], 2.2f), wtm::powf(look.accent[1], 2.2f), wtm::powf(look.accent[2], 2.2f)};
  a.surf_mode = look.surf_mode; a.palette = look.palette; a.carbon_body = look.carbon_body; a.is_f1 = look.is_f1;
  a.slice_axis = look.slice_axis; a.show_flow = look.show_flow; a.slice_pos = look.slice_pos;
  a.slice_alpha = look.slice_alpha;
  a.mesh_mode = look.mesh_mode; a.cooling = look.cooling;
  a.g_albedo = reinterpret_cast<const ushort4*>(g_gb_albedo);
  a.g_normal = reinterpret_cast<const ushort4*>(g_gb_normal);
  a.g_material = reinterpret_cast<const uchar4*>(g_gb_material);
  if (a.mesh_mode != 0u && !(g_gb_albedo && g_gb_normal && g_gb_material)) return;
  a.key = f3n(-0.32f, 0.90f, 0.30f);
  a.fill_a = f3n(0.6f, 0.35f, -0.7f);
  a.fill_b = f3n(0.6f, 0.35f, 0.7f);
  a.w = w; a.h = hgt;
  a.car = g_car;
  const Scene S = make_scene(a.shape, g_car);
  for (uint32_t y = y0; y < y1 && y < hgt; y++)
    for (uint32_t x = 0; x < w; x++) {
      const float4 c = a.mesh_mode != 0u ? render_pixel<true>(S, a, x, y) : render_pixel<false>(S, a, x, y);
      float* o = out + ((size_t)y * w + x) * 4;
      o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = c.w;
    }
}

// sceneSdf at n points (xyz): out[2k] distance, out[2k+1] material.
void wthm_scene_sdf(const void* shape, const float* pts, uint32_t n, float* out) {
  wt_shape sh;
  memcpy(&sh, shape, sizeof sh);
  const Scene S = make_scene(sh, g_car);
  for (uint32_t k = 0; k < n; k++) {
    const V2 r = scene_sdf(S, v3(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]));
    out[2 * k] = r.x;
    out[2 * k + 1] = r.y;
  }
}

}  // extern "C"
