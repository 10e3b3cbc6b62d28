// Kernel arguments of the field consumers (wt_fields.cu): the reference's
// Grid / PSim / View / Stream uniforms (src/engine/wgsl.ts:430-434,516-521,
// src/engine/render-wgsl.ts:521-526) over the library's buffers.  Not installed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wt {

struct FieldGrid {
  uint32_t nx, ny, nz;
  float ox, oy, oz, h;
  const float4* fields;  // (ux, uy, uz, rho) of the last step call; rho = 0 in solid cells
  const float* temps;
};

struct ViewArgs {
  float uIn, vReal, cpMin, cpMax, tMin, tMax, speedMax, vortMax;
};

struct PSimArgs {
  uint32_t count, spawnMode, colorMode, frame, scatter, rakeRows, rakeCols;
  float dt, life, smin[3], smax[3];
};

struct StreamArgs {
  uint32_t lines, steps, seedMode, colorMode, rows, cols, perEmitter, emitters;
  float smin[3], smax[3], stepLen, time;
  float emit[8][4];  // emitter centre and radius
};

cudaError_t launch_particles(const FieldGrid& g, const PSimArgs& ps, const ViewArgs& v, float4* parts, cudaStream_t s);
cudaError_t launch_streamlines(const FieldGrid& g, const StreamArgs& st, const ViewArgs& v, float4* pts,
                               cudaStream_t s);
cudaError_t launch_sample_points(const FieldGrid& g, const float* pts, uint32_t n, float* out, float* vort,
                                 cudaStream_t s);

}  // namespace wt
