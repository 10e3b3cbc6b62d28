// Semi-Lagrangian heat advection (HEAT, src/engine/wgsl.ts:460-510): trilinear
// backtrace of the temperature along u*dt, 6-neighbour diffusion mix, source
// mix from the voxelizer's emission field, cooling.  One thread per cell; the
// backtrace gathers stay within a few cells so they hit L1/L2.  The source term
// (the neighbours' largest emission) depends on the flags only and is formed
// once per voxelization (heat_sources_kernel).
// Algorithmic traffic per cell and pass: fields 16 B + source 4 B + tin 4 B read,
// tout 4 B written = 28 B (solid cells read emit instead of the source).  Built with -fmad=false: bit-identical to the CPU model.
#include "wt_internal.h"

namespace wt {
namespace {

__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float mxf(float a, float b) { return a < b ? b : a; }

__device__ __forceinline__ uint32_t idx_of(int x, int y, int z, int nx, int ny, int nz) {
  if (z < 0) z = -z - 1;  // symmetry plane (wgsl.ts:472)
  x = min(max(x, 0), nx - 1);
  y = min(max(y, 0), ny - 1);
  z = min(max(z, 0), nz - 1);
  return (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
}

__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }  // saturating, NaN -> 0

__device__ __forceinline__ int clampi(int v, int n) { return min(max(v, 0), n - 1); }
__device__ __forceinline__ int zmir(int z, int nz) {  // idx_of's z: mirror, then clamp
  if (z < 0) z = -z - 1;
  return min(max(z, 0), nz - 1);
}

__global__ void heat_kernel(HeatArgs a) {
  // chained like the step kernels: the next launch may be scheduled now; wait
  // for the fields and temperatures of the previous launch
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int nx = (int)a.nx, ny = (int)a.ny, nz = (int)a.nz;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const uint32_t idx = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z);
  const float4 fv = a.fields[idx];
  if (fv.w <= 0.0f) {
    a.tout[idx] = a.emit[idx];
    return;
  }
  const float gx = (float)x - fv.x * a.dt, gy = (float)y - fv.y * a.dt, gz = (float)z - fv.z * a.dt;
  const int ix = f2i(floorf(gx)), iy = f2i(floorf(gy)), iz = f2i(floorf(gz));
  const float fx = gx - (float)ix, fy = gy - (float)iy, fz = gz - (float)iz;
  // the eight corners' clamped (and z-mirrored) coordinates, as idx_of forms them
  const uint32_t xs[2] = {(uint32_t)clampi(ix, nx), (uint32_t)clampi(ix + 1, nx)};
  const uint32_t rows[4] = {(uint32_t)nx * ((uint32_t)clampi(iy, ny) + (uint32_t)ny * (uint32_t)zmir(iz, nz)),
                            (uint32_t)nx * ((uint32_t)clampi(iy + 1, ny) + (uint32_t)ny * (uint32_t)zmir(iz, nz)),
                            (uint32_t)nx * ((uint32_t)clampi(iy, ny) + (uint32_t)ny * (uint32_t)zmir(iz + 1, nz)),
                            (uint32_t)nx * ((uint32_t)clampi(iy + 1, ny) + (uint32_t)ny * (uint32_t)zmir(iz + 1, nz))};
  float t = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
    const float w = (ox ? fx : 1.0f - fx) * (oy ? fy : 1.0f - fy) * (oz ? fz : 1.0f - fz);
    const int cx = ix + ox;
    const float tv = cx < 0 ? 0.0f : a.tin[xs[ox] + rows[oy + 2 * oz]];
    t = t + tv * w;
  }
  float nb = 0.0f;
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const int cx = x + off[k][0], cy = y + off[k][1], cz = z + off[k][2];
    nb = nb + (cx < 0 ? 0.0f : a.tin[idx_of(cx, cy, cz, nx, ny, nz)]);
  }
  const float src = a.src[idx];
  t = mixf(t, __fdiv_rn(nb, 6.0f), a.diffuse);
  if (src > 0.0f) t = mixf(t, src, a.src_mix);
  a.tout[idx] = mxf(t * (1.0f - a.cool), 0.0f);
}

// The largest emission among a fluid cell's six neighbours inside the lattice
// (the z = -1 neighbour mirrors onto z = 0), 0 if none emits: what the heat
// pass mixes in (wgsl.ts:493-500).  It changes only with the flags, so it is
// formed once per voxelization instead of in every pass.
__global__ void heat_sources_kernel(const float* __restrict__ emit, float* __restrict__ src, int nx, int ny, int nz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const int cx = x + off[k][0], cy = y + off[k][1], cz = z + off[k][2];
    if (cx >= 0 && cy >= 0 && cx < nx && cy < ny && cz < nz) m = mxf(m, emit[idx_of(cx, cy, cz, nx, ny, nz)]);
  }
  src[(uint32_t)x + (uint32_t)nx * ((uint32_t)y + (uint32_t)ny * (uint32_t)z)] = m;
}

}  // namespace

cudaError_t launch_heat_sources(const float* emit, float* src, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s) {
  const dim3 block(128, 1, 1);
  const dim3 g((nx + 127) / 128, ny, nz);
  heat_sources_kernel<<<g, block, 0, s>>>(emit, src, (int)nx, (int)ny, (int)nz);
  return cudaGetLastError();
}

cudaError_t launch_heat(const HeatArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((a.nx + 127) / 128, a.ny, a.nz);
  cfg.blockDim = dim3(128, 1, 1);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // programmatic dependent launch
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, heat_kernel, a);
}

}  // namespace wt
