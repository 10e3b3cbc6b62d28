// Kernel arguments of the render passes (wt_render.cu): the reference's Cam,
// Look, Taa, PDraw, SDraw, Blur and Post uniforms (src/engine/render-wgsl.ts,
// src/engine/wgsl.ts:597-603) resolved into plain values, plus the render
// targets.  Float targets are RGBA binary16 (`ushort4` bit patterns), the output
// is RGBA8.  Not installed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "wt_fields.h"
#include "wt_internal.h"

namespace wt {

struct F3 {
  float x, y, z;
};

struct SceneArgs {
  wt_shape shape;             // the context's shape (Shape uniform)
  CarView car;                // its W17 model, if any
  FieldGrid g;                // fields / temperatures of the last step call
  ViewArgs view;
  // Cam (render-wgsl.ts:5-11)
  F3 pos, fwd, right, up;
  float tan_half, aspect, time, road_speed, jitter_x, jitter_y;
  // Look (render-wgsl.ts:12-19); paint and accent already through toLinear
  F3 bmin, bmax, paint_lin, accent_lin;
  uint32_t surf_mode, palette, carbon_body, is_f1, slice_axis, show_flow;
  float slice_pos, slice_alpha;
  uint32_t mesh_mode, cooling;  // meshMode: surfaces come from the G-buffer below
  // car G-buffer of the mesh pass (engine.ts:297-303), w x h: albedo (rgb, rough)
  // and normal-distance as binary16, material (metal, coat, emissive, 1) as RGBA8
  const ushort4* g_albedo;
  const ushort4* g_normal;
  const uchar4* g_material;
  // normalize(KEY) and the two fill-light directions of shadeSurface
  F3 key, fill_a, fill_b;
  uint32_t w, h;
  ushort4* scene;
};

struct TaaArgs {
  float m[16];                // prevViewProj, column-major
  F3 cam_pos, fwd, right, up;
  float tan_half, aspect, blend;
  uint32_t w, h;
  const ushort4* cur;
  const ushort4* hist;
  ushort4* out;
};

struct BlurArgs {
  float dir_x, dir_y, spacing, gain;
  float wk[13];               // exp(-k^2 / 14), k = -6..6
  uint32_t sw, sh, dw, dh;
  const ushort4* src;
  ushort4* dst;
};

struct PresentArgs {
  float bloom, exposure;
  uint32_t w, h, gw, gh, bw, bh;
  const ushort4* scene;
  const ushort4* glow;
  const ushort4* bloom_tex;
  uchar4* out;
};

// One instanced quad draw of the glow pass.
struct DrawArgs {
  int kind;                   // 0 particles (PARTICLES_DRAW), 1 streamlines (STREAM_DRAW)
  float m[16];                // viewProj, column-major
  F3 cam_pos;
  float width, res_x, res_y;
  float trail, alpha, fade_in;   // particles
  float time, intensity, pulse;  // streamlines
  uint32_t count, palette;       // particles: count; both: palette
  uint32_t lines, steps;         // streamlines
  uint32_t instances;
  const float4* data;         // particles (pos, vel) pairs or line points
  uint32_t w, h;
  const ushort4* scene;
  unsigned long long* acc;    // w*h*4 fixed-point sums
};

cudaError_t launch_render_scene(const SceneArgs& a, cudaStream_t s);
cudaError_t launch_taa(const TaaArgs& a, cudaStream_t s);
cudaError_t launch_blur(const BlurArgs& a, cudaStream_t s);
cudaError_t launch_present(const PresentArgs& a, cudaStream_t s);
cudaError_t launch_glow_draw(const DrawArgs& a, cudaStream_t s);
cudaError_t launch_glow_resolve(const unsigned long long* acc, ushort4* glow, uint32_t texels, cudaStream_t s);

}  // namespace wt
