// Voxelizer (VOXELIZE, src/engine/wgsl.ts:294-321) and the cell words the
// step kernels read.
//
// The signed-distance scenes are the reference's analytic ones
// (src/engine/wgsl.ts:20-76,101-116 primitives and scene switch;
// src/engine/f1.ts:20-320 generic F1, :397-407 heat emission).  Solid flags
// are a threshold test on the distance at the cell centre, so every float
// operation is kept in the reference's order and this unit is built with
// -fmad=false: flags and emission match the CPU model bit for bit.  sin, cos
// and atan are the project's functions (wt_fmath.h); shape-wide values (rake
// rotation, rear main-plane direction) are computed once on the host with the
// same functions, which gives the same bits as evaluating them per cell.
//
// The cell-word pass stages a tile of solid flags (with a 2-cell halo in x for
// the belt test and 1 in y and z) in shared memory; coordinates are clamped to
// the lattice when loading, which makes the z = -1 halo the z = 0 mirror image
// the reference reads through its symmetry plane (wgsl.ts:218).
#include "wt_internal.h"
#include "wt_lattice.cuh"
#include "wt_scene.cuh"

namespace wt {
namespace {

__global__ void voxelize_kernel(Scene S, uint32_t nx, uint32_t ny, uint32_t nz, float ox, float oy, float oz, float h,
                                uint8_t* __restrict__ solid, float* __restrict__ emit) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  const uint32_t z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const uint32_t idx = x + nx * (y + ny * z);
  const V3 p = v3(ox + ((float)x + 0.5f) * h, oy + ((float)y + 0.5f) * h, oz + ((float)z + 0.5f) * h);
  V2 r = scene_sdf(S, p);
  const bool w17 = S.s.kind == WT_KIND_W17 && S.car.body != nullptr;
  // the W17's cooling ducts are carved out of its body (wgsl.ts:313) and marked
  // with emission -1 (wgsl.ts:319-320): the step relaxes the air there
  const float duct = w17 ? w17_duct(S, p) : 1e3f;
  if (w17 && ab(r.y - 12.0f) < 0.5f) r.x = mx(r.x, -duct);
  const bool inside = r.x < (w17 ? 0.45f : 0.3f) * h && x > 1u && x < nx - 2u;
  uint32_t group = 1u;
  if (ab(r.y - 7.0f) < 0.5f) group = 2u;
  if (ab(r.y - 8.0f) < 0.5f) group = 3u;
  solid[idx] = inside ? (uint8_t)group : (uint8_t)0;
  const float em = S.s.kind == WT_KIND_F1 ? f1_emission(S, p) : (w17 ? w17_emission(S, p) : 0.0f);
  emit[idx] = inside ? em : (w17 && duct < 0.0f ? -1.0f : 0.0f);
}

// ---------------------------------------------------------------- cell words
constexpr int TX = 32, TY = 4, TZ = 2;
constexpr int HX = 2, HY = 1, HZ = 1;
constexpr int SX = TX + 2 * HX, SY = TY + 2 * HY, SZ = TZ + 2 * HZ;

__global__ void cell_words_kernel(const uint8_t* __restrict__ solid, const float* __restrict__ emit,
                                  uint32_t* __restrict__ cellw, uint32_t nx, uint32_t ny, uint32_t nz) {
  __shared__ uint8_t tile[SZ][SY][SX];
  const int x0 = blockIdx.x * TX - HX, y0 = blockIdx.y * TY - HY, z0 = blockIdx.z * TZ - HZ;
  const int tid = threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z);
  for (int k = tid; k < SX * SY * SZ; k += TX * TY * TZ) {
    const int lx = k % SX, ly = (k / SX) % SY, lz = k / (SX * SY);
    const int gx = min(max(x0 + lx, 0), (int)nx - 1);
    const int gy = min(max(y0 + ly, 0), (int)ny - 1);
    const int gz = min(max(z0 + lz, 0), (int)nz - 1);
    tile[lz][ly][lx] = solid[(uint32_t)gx + nx * ((uint32_t)gy + ny * (uint32_t)gz)];
  }
  __syncthreads();
  const uint32_t x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z * TZ + threadIdx.z;
  if (x >= nx || y >= ny || z >= nz) return;
  const uint32_t idx = x + nx * (y + ny * z);
  const int lx = threadIdx.x + HX, ly = threadIdx.y + HY, lz = threadIdx.z + HZ;
  if (tile[lz][ly][lx]) {
    cellw[idx] = CW_SOLID;
    return;
  }
  uint32_t w = 0u;
  const bool duct = emit[idx] < 0.0f;
  bool force = false;
  sfor<19>([&](auto I) {
    constexpr int i = I;
    if constexpr (i != 0) {
      constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
      const int sx = (int)x - cx, sy = (int)y - cy, sz = (int)z - cz;
      // precedence of wgsl.ts:207-221: inlet, outlet, floor, far field come first
      if (sx < 0 || sx >= (int)nx || sy < 0 || sy >= (int)ny || sz >= (int)nz) return;
      if (tile[lz - cz][ly - cy][lx - cx]) {  // z = -1 reads the clamped (mirrored) z = 0 flag
        w |= 1u << i;
        if (!(sz < 0)) force = true;
      }
    }
  });
  if (y == 0u) {  // belt contact patch (wgsl.ts:192-197)
    if (tile[lz][ly][lx - 2] || tile[lz][ly][lx + 2] || tile[lz][ly + 1][lx] || tile[lz - 1][ly][lx] ||
        tile[lz + 1][ly][lx])
      w |= CW_BELT;
  }
  if (duct) w |= CW_DUCT;
  if (force && !duct) w |= CW_FORCE;
  cellw[idx] = w;
}

__global__ void block_flags_kernel(const uint32_t* __restrict__ cellw, uint32_t nx, uint32_t ny,
                                   uint8_t* __restrict__ flags) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  const uint32_t z = blockIdx.z;
  bool f = false;
  if (x < nx && y < ny) f = (cellw[x + nx * (y + ny * z)] & CW_FORCE) != 0u;
  const int any = __syncthreads_or(f);
  if (threadIdx.x == 0 && threadIdx.y == 0)
    flags[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = any ? 1 : 0;
}

__global__ void links_out_kernel(const uint32_t* __restrict__ cellw, uint32_t* __restrict__ links, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t w = cellw[i];
    links[i] = (w & CW_SOLID) ? 0u : (w & (CW_LINKS | CW_BELT));
  }
}
__global__ void solid_u32_kernel(const uint8_t* __restrict__ s, uint32_t* __restrict__ out, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = s[i];
}
__global__ void solid_from_u32_kernel(const uint32_t* __restrict__ in, uint8_t* __restrict__ s, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) s[i] = (uint8_t)(in[i] > 3u ? 3u : in[i]);
}

}  // namespace

// Scene distance at the cell centres of `grid` (the first component of sceneSdf).
__global__ void sdf_sample_kernel(Scene S, uint32_t nx, uint32_t ny, uint32_t nz, float ox, float oy, float oz,
                                  float h, float* __restrict__ out) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
  const uint32_t z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const V3 p = v3(ox + ((float)x + 0.5f) * h, oy + ((float)y + 0.5f) * h, oz + ((float)z + 0.5f) * h);
  out[x + nx * (y + ny * z)] = scene_sdf(S, p).x;
}


cudaError_t launch_sdf_sample(const wt_shape& shape, const wt_grid& grid, float* out, cudaStream_t s) {
  const Scene S = make_scene(shape);
  const dim3 block(32, 4, 1);
  const dim3 g((grid.nx + 31) / 32, (grid.ny + 3) / 4, grid.nz);
  sdf_sample_kernel<<<g, block, 0, s>>>(S, grid.nx, grid.ny, grid.nz, grid.origin[0], grid.origin[1], grid.origin[2],
                                        grid.h, out);
  return cudaGetLastError();
}

cudaError_t launch_voxelize(const wt_shape& shape, const CarView& car, const wt_grid& grid, uint8_t* solid, float* emit,
                            cudaStream_t s) {
  const Scene S = make_scene(shape, car);
  const dim3 block(32, 4, 1);
  const dim3 g((grid.nx + 31) / 32, (grid.ny + 3) / 4, grid.nz);
  voxelize_kernel<<<g, block, 0, s>>>(S, grid.nx, grid.ny, grid.nz, grid.origin[0], grid.origin[1], grid.origin[2],
                                      grid.h, solid, emit);
  return cudaGetLastError();
}

cudaError_t launch_cell_words(const uint8_t* solid, const float* emit, uint32_t* cellw, uint32_t nx, uint32_t ny,
                              uint32_t nz, cudaStream_t s) {
  const dim3 block(TX, TY, TZ);
  const dim3 g((nx + TX - 1) / TX, (ny + TY - 1) / TY, (nz + TZ - 1) / TZ);
  cell_words_kernel<<<g, block, 0, s>>>(solid, emit, cellw, nx, ny, nz);
  return cudaGetLastError();
}

cudaError_t launch_block_flags(const uint32_t* cellw, const StepGeom& g, uint32_t nx, uint32_t ny, uint32_t nz,
                               uint8_t* flags, cudaStream_t s) {
  (void)nz;
  block_flags_kernel<<<g.grid, g.block, 0, s>>>(cellw, nx, ny, flags);
  return cudaGetLastError();
}

cudaError_t launch_links_out(const uint32_t* cellw, uint32_t* links, uint64_t n, cudaStream_t s) {
  links_out_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(cellw, links, n);
  return cudaGetLastError();
}
cudaError_t launch_solid_u32(const uint8_t* solid, uint32_t* out, uint64_t n, cudaStream_t s) {
  solid_u32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(solid, out, n);
  return cudaGetLastError();
}
cudaError_t launch_solid_from_u32(const uint32_t* in, uint8_t* solid, uint64_t n, cudaStream_t s) {
  solid_from_u32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, solid, n);
  return cudaGetLastError();
}

}  // namespace wt
