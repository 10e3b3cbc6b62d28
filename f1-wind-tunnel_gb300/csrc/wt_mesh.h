// Kernel arguments of the car mesh G-buffer pass (wt_mesh.cu): the MESH_DRAW
// pipeline of the reference (src/engine/render-wgsl.ts:647-760, draws of
// MeshCar, src/engine/mesh-car.ts:46-213).  Not installed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "wt_texfilter.h"

namespace wt {

// One draw as the kernels read it: the MeshMat uniform, its range of the index
// list, texture, blend state and its place in the frame's corner and triangle
// sequences.
struct MeshDraw {
  float color[4];
  float metal, rough, coat, alpha_cut, emissive, has_tex, is_body;
  uint32_t first_index, count;
  int32_t tex;           // texture slot, -1 = none
  uint32_t blend;        // decal: biased 'less-equal' test, no depth write, albedo blended
  uint32_t corner_base;  // first corner of the draw among the frame's corners
  uint32_t tri_base;     // sequence number of its first triangle in the frame
  uint32_t pad[3];
};

struct MeshTex {
  uint32_t first_level, n_levels;
};

struct MeshArgs {
  const float4* verts;      // 2 per vertex: position + u, normal + v
  const uint32_t* indices;
  const uint8_t* tags;      // part (bits 0-2) and assembly (bits 3-7) per vertex
  const wtx::Level* levels;
  const MeshTex* texs;
  const MeshDraw* draws;
  uint32_t n_draws;
  // MeshCam (render-wgsl.ts:648-652)
  float vp[16];
  float cam_pos[3], ride_h;
  float jitter[2], rake, base_ride;
  const float4* rig;        // the Rig uniform, 87 vec4
  // frame
  uint32_t w, h;
  float4* cpos;             // vertex shader outputs per corner: clip position,
  float4* cattr;            // and 2 float4 of varyings (world xyz + u, normal xyz + v)
  float* depth;             // depth32float
  unsigned long long* keys; // visibility: depth bits << 32 | triangle sequence * 2 + part
  uint4* big;               // parts with a large footprint: (triangle, part, first tile, 0)
  unsigned long long* big_count;  // parts << 32 | tiles
  uint32_t big_cap;
  ushort4* g_albedo;
  ushort4* g_normal;
  uchar4* g_material;
  uint32_t* dcount;         // decal fragments per pixel, their offsets and fill cursors
  uint32_t* doff;
  uint32_t* dcur;
  uint32_t* dslots;         // decal fragments (triangle sequence * 2 + part), grouped per pixel
};

cudaError_t launch_mesh_clear(const MeshArgs& a, cudaStream_t s);
cudaError_t launch_mesh_vertex(const MeshArgs& a, uint32_t corners, cudaStream_t s);
// Draws [d0, d1), triangles [tri0, tri1) of the frame's sequence, all opaque:
// visibility against the current depth, then one fragment per pixel.
cudaError_t launch_mesh_opaque(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                               cudaStream_t s);
// Draws [d0, d1), all decals: the passing fragments per pixel into dcount.
cudaError_t launch_mesh_decal_count(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                                    cudaStream_t s);
// doff = exclusive prefix sum of dcount (temp == NULL: *temp_bytes receives the scratch size).
cudaError_t launch_mesh_decal_scan(const MeshArgs& a, void* temp, size_t* temp_bytes, cudaStream_t s);
// The fragments into dslots at doff, then each pixel's list blended in order.
cudaError_t launch_mesh_decal_blend(const MeshArgs& a, uint32_t d0, uint32_t d1, uint32_t tri0, uint32_t tri1,
                                    cudaStream_t s);

}  // namespace wt
