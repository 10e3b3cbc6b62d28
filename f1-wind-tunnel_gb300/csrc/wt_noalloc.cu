// wt_forces_noalloc: momentum-exchange forces of a population state, for callers
// that cannot allocate device memory.
//
// Who needs it: hosts that hand libwt buffers they allocated themselves and do
// not allow a library to allocate behind their back - an engine that owns all
// GPU memory through its own arena or memory budget, or a renderer that shares
// the lattice through graphics-API interop memory - and code that must not hit
// cudaMalloc (which can synchronise the whole device) in the middle of a frame.
// Such a caller has device pointers to the populations and flags but no
// wt_ctx (creating one allocates).
//
// What it computes: the force the next collide-stream step takes from this
// state.  Per fluid cell it pulls the 19 populations with the reference's
// boundary precedence (src/engine/wgsl.ts:191-229: inlet, outlet from the
// cell's previous velocity, moving belt with its contact mask, far field,
// symmetry mirror, bounce-back), adds the momentum exchange of the
// non-mirrored bounce-back links of non-duct cells (wgsl.ts:221-223), and
// drops the cell's force when the divergence guard fires on its moments
// (wgsl.ts:231-243).  Forces are summed per solid group in FP64 and as the
// reference's i32 fixed-point accumulator.  It is the force path of the step
// kernel (wt_lbm.cu) without the collision.
//
// Scratch: the per-block partial records live in g_probe_scratch, a file-scope
// __device__ array of WT_NOALLOC_BLOCKS + 2 records (96 B each, 98,496 B in all:
// the block records, the result record and the guard counter's record)
// that every GPU which loads the library holds until the process exits.  In
// host code the array's name is only a host-side stand-in, so its device
// address is obtained once per device with cudaGetSymbolAddress (with that
// device current) on the first call on that device, and kept for the process:
// this assumes the device's primary context lives as long as the process (no
// cudaDeviceReset between calls).  Every call overwrites all the records it
// reads (the guard counter it accumulates is cleared at the start of each
// call), so nothing else has to be cleared; the array is shared by all calls, so
// calls that overlap on the GPU (different streams, or different host threads
// on the same device) race and must be serialised by the caller.  The first
// call on a device does that device's set-up (the address lookup), so make it
// before any stream capture begins.  Each call ends by synchronising its stream.
// No cudaMalloc/cudaFree or allocating library routine is called.
#include <string.h>

#include <mutex>

#include "wt_internal.h"
#include "wt_lattice.cuh"

namespace wt {
namespace {

constexpr uint32_t PROBE_THREADS = 256;

static __device__ __align__(256) ForceSlot g_probe_scratch[WT_NOALLOC_BLOCKS + 2];

std::mutex g_probe_mu;
ForceSlot* g_probe_addr[64] = {nullptr};

struct ProbeArgs {
  const float* f;         // 19 * n, f[i * n + idx]
  const uint32_t* solid;  // n
  const float* emit;      // n or null
  const float4* fields;   // n or null: previous (u, rho), read on the outlet column
  uint32_t nx, ny, nz;
  float u_in;
  float guard_uu;
  float feq_in[19];   // feq(i, 1, (u_in, 0, 0))
  float floor_k[19];  // 6 * w_i * c_ix
};

// feq(i, 1, u) in the reference's operation order (wgsl.ts:135-138), zero
// lattice coefficients dropped as in the step kernel.
template <int i>
__device__ __forceinline__ float feq1(float ux, float uy, float uz) {
  constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
  float cu = 0.0f;
  bool first = true;
  if constexpr (cx != 0) { cu = (cx > 0) ? ux : -ux; first = false; }
  if constexpr (cy != 0) { if (first) cu = (cy > 0) ? uy : -uy; else cu = (cy > 0) ? cu + uy : cu - uy; first = false; }
  if constexpr (cz != 0) { if (first) cu = (cz > 0) ? uz : -uz; else cu = (cz > 0) ? cu + uz : cu - uz; }
  const float uu = ux * ux + uy * uy + uz * uz;
  return Wd(i) * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
}

__device__ __forceinline__ bool bad(float x) { return (__float_as_uint(x) & 0x7f800000u) == 0x7f800000u; }

template <int i>
__device__ __forceinline__ void add_link(float v, uint32_t grp, float (&gf)[9]) {
  const float t = 2.0f * (v - Wd(i));
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (grp == (uint32_t)(k + 1)) {
      if constexpr (CXd(i) > 0) gf[3 * k] = gf[3 * k] - t;
      if constexpr (CXd(i) < 0) gf[3 * k] = gf[3 * k] + t;
      if constexpr (CYd(i) > 0) gf[3 * k + 1] = gf[3 * k + 1] - t;
      if constexpr (CYd(i) < 0) gf[3 * k + 1] = gf[3 * k + 1] + t;
      if constexpr (CZd(i) > 0) gf[3 * k + 2] = gf[3 * k + 2] - t;
      if constexpr (CZd(i) < 0) gf[3 * k + 2] = gf[3 * k + 2] + t;
    }
  }
}

__global__ void __launch_bounds__(PROBE_THREADS) probe_kernel(const ProbeArgs a, ForceSlot* scratch,
                                                               unsigned int* guarded) {
  const uint32_t nx = a.nx, ny = a.ny, nz = a.nz;
  const uint32_t nxy = nx * ny, n = nxy * nz;
  const float* __restrict__ f = a.f;
  const uint32_t* __restrict__ solid = a.solid;
  double d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t r[6] = {0, 0, 0, 0, 0, 0};
  unsigned int nguard = 0;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (solid[idx] != 0u) continue;
    const int x = (int)(idx % nx), y = (int)((idx / nx) % ny), z = (int)(idx / nxy);
    const bool duct = a.emit != nullptr && a.emit[idx] < 0.0f;  // no force in duct cells (wgsl.ts:201,223)
    // moving belt: no floor speed under a contact patch (wgsl.ts:191-198)
    float floor_u = a.u_in;
    if (y == 0) {
      const uint32_t row = (uint32_t)z * nxy;
      const uint32_t xl = x < 2 ? 0u : (uint32_t)x - 2u, xr = (uint32_t)x + 2u > nx - 1u ? nx - 1u : (uint32_t)x + 2u;
      const uint32_t zl = z < 1 ? 0u : (uint32_t)z - 1u, zr = (uint32_t)z + 1u > nz - 1u ? nz - 1u : (uint32_t)z + 1u;
      if (solid[row + xl] || solid[row + xr] || solid[idx + nx] || solid[zl * nxy + (uint32_t)x] ||
          solid[zr * nxy + (uint32_t)x])
        floor_u = 0.0f;
    }
    float4 pu = make_float4(a.u_in, 0.0f, 0.0f, 1.0f);
    if (x == (int)nx - 1 && a.fields != nullptr) pu = a.fields[idx];
    float gf[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float rho = 0.0f, mx = 0.0f, my = 0.0f, mz = 0.0f;
    sfor<19>([&](auto I) {  // pull streaming with the boundary precedence of wgsl.ts:203-229
      constexpr int i = I;
      constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
      const int sx = x - cx, sy = y - cy;
      int sz = z - cz;
      float v;
      if (sx < 0) {
        v = a.feq_in[i];
      } else if (sx >= (int)nx) {
        v = feq1<i>(pu.x, pu.y, pu.z);
      } else if (sy < 0) {
        v = f[(size_t)OPPd(i) * n + idx];
        if constexpr (cx != 0) v = v + a.floor_k[i] * floor_u;
      } else if (sy >= (int)ny || sz >= (int)nz) {
        v = a.feq_in[i];
      } else {
        int src = i;
        bool mirrored = false;
        if (sz < 0) { sz = 0; src = ZMIRd(i); mirrored = true; }
        const uint32_t sidx = (uint32_t)sx + nx * (uint32_t)sy + nxy * (uint32_t)sz;
        const uint32_t g = solid[sidx];
        if (g != 0u) {
          v = f[(size_t)OPPd(i) * n + idx];
          if (!mirrored && !duct) add_link<i>(v, g > 3u ? 3u : g, gf);
        } else {
          v = f[(size_t)src * n + sidx];
        }
      }
      // moments in direction order (wgsl.ts:231-235)
      rho = rho + v;
      if constexpr (cx > 0) mx = mx + v;
      if constexpr (cx < 0) mx = mx - v;
      if constexpr (cy > 0) my = my + v;
      if constexpr (cy < 0) my = my - v;
      if constexpr (cz > 0) mz = mz + v;
      if constexpr (cz < 0) mz = mz - v;
    });
    // divergence guard (wgsl.ts:236-243): the step resets the cell and drops its force
    const float den = (rho < 1e-4f) ? 1e-4f : rho;
    const float ux = __fdiv_rn(mx, den), uy = __fdiv_rn(my, den), uz = __fdiv_rn(mz, den);
    const float uu = __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz));
    if (bad(rho) || bad(ux) || bad(uy) || bad(uz) || rho < 0.3f || rho > 3.0f || uu > a.guard_uu) {
      nguard++;
      continue;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) d[k] += (double)gf[k];
#pragma unroll
    for (int g = 0; g < 3; g++) {
      if (gf[3 * g] != 0.0f) r[2 * g] += (uint32_t)__float2int_rn(gf[3 * g] * 10000.0f);
      if (gf[3 * g + 1] != 0.0f) r[2 * g + 1] += (uint32_t)__float2int_rn(gf[3 * g + 1] * 10000.0f);
    }
  }
  if (nguard) atomicAdd(guarded, nguard);
  // fixed-order block reduction: warp shuffles, then warps in index order
  __shared__ double sd[9][PROBE_THREADS / 32];
  __shared__ uint32_t sr[6][PROBE_THREADS / 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
#pragma unroll
    for (int k = 0; k < 9; k++) d[k] += __shfl_down_sync(0xffffffffu, d[k], s);
#pragma unroll
    for (int k = 0; k < 6; k++) r[k] += __shfl_down_sync(0xffffffffu, r[k], s);
  }
  if (lane == 0) {
    for (int k = 0; k < 9; k++) sd[k][warp] = d[k];
    for (int k = 0; k < 6; k++) sr[k][warp] = r[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ForceSlot out;
    for (int k = 0; k < 9; k++) {
      double t = 0.0;
      for (uint32_t w = 0; w < PROBE_THREADS / 32; w++) t += sd[k][w];
      out.f[k] = t;
    }
    for (int k = 0; k < 6; k++) {
      uint32_t t = 0;
      for (uint32_t w = 0; w < PROBE_THREADS / 32; w++) t += sr[k][w];
      out.raw[k] = (int32_t)t;
    }
    scratch[blockIdx.x] = out;  // every record the finish kernel reads is rewritten here
  }
}

// Sums the block records in a fixed order into scratch[WT_NOALLOC_BLOCKS].
__global__ void __launch_bounds__(PROBE_THREADS) probe_finish(ForceSlot* scratch, uint32_t nb) {
  __shared__ double sd[PROBE_THREADS];
  __shared__ uint32_t sr[PROBE_THREADS];
  const uint32_t t = threadIdx.x;
  ForceSlot res;
  for (int k = 0; k < 15; k++) {
    double acc = 0.0;
    uint32_t racc = 0;
    for (uint32_t b = t; b < nb; b += PROBE_THREADS) {
      if (k < 9) acc += scratch[b].f[k];
      else racc += (uint32_t)scratch[b].raw[k - 9];
    }
    sd[t] = acc;
    sr[t] = racc;
    __syncthreads();
    for (uint32_t w = PROBE_THREADS / 2; w > 0; w >>= 1) {
      if (t < w) { sd[t] += sd[t + w]; sr[t] += sr[t + w]; }
      __syncthreads();
    }
    if (t == 0) {
      if (k < 9) res.f[k] = sd[0];
      else res.raw[k - 9] = (int32_t)sr[0];
    }
    __syncthreads();
  }
  if (t == 0) scratch[WT_NOALLOC_BLOCKS] = res;
}

}  // namespace
}  // namespace wt

extern "C" int wt_forces_noalloc(const float* f, const uint32_t* solid, const float* emit, const float* fields,
                                 uint32_t nx, uint32_t ny, uint32_t nz, float u_in, void* stream, wt_forces* out) {
  using namespace wt;
  if (!f || !solid || !out) return WT_ERR_ARG;
  if (nx < 8 || ny < 3 || nz < 3) return WT_ERR_ARG;  // the minimum lattice of wt_create
  if (!(u_in == u_in) || u_in < -1.0f || u_in > 1.0f) return WT_ERR_ARG;
  const uint64_t n = (uint64_t)nx * ny * nz;
  if (n > WT_NOALLOC_MAX_CELLS) return WT_ERR_NOALLOC_LIMIT;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return WT_ERR_DEVICE;
  ForceSlot* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_probe_mu);
    if (!g_probe_addr[dev]) {
      // first call on this device (with it current): device address of the static scratch
      e = cudaGetSymbolAddress((void**)&g_probe_addr[dev], g_probe_scratch);
      if (e != cudaSuccess) {
        g_probe_addr[dev] = nullptr;
        return WT_ERR_CUDA;
      }
    }
    scratch = g_probe_addr[dev];
  }
  ProbeArgs a;
  a.f = f;
  a.solid = solid;
  a.emit = emit;
  a.fields = reinterpret_cast<const float4*>(fields);
  a.nx = nx;
  a.ny = ny;
  a.nz = nz;
  a.u_in = u_in;
  a.guard_uu = guard_threshold();
  for (int i = 0; i < 19; i++) {  // host arithmetic without contraction: the device's bits
    const float cu = (float)CXd(i) * u_in + (float)CYd(i) * 0.0f + (float)CZd(i) * 0.0f;
    const float uu = u_in * u_in + 0.0f * 0.0f + 0.0f * 0.0f;
    a.feq_in[i] = Wd(i) * 1.0f * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
    a.floor_k[i] = 6.0f * Wd(i) * (float)CXd(i);
  }
  // the guard counter is the first word of the record after the result (cleared per call)
  unsigned int* guarded = reinterpret_cast<unsigned int*>(scratch + WT_NOALLOC_BLOCKS + 1);
  if (cudaMemsetAsync(guarded, 0, sizeof(unsigned int), s) != cudaSuccess) return WT_ERR_CUDA;
  uint64_t nb = (n + PROBE_THREADS - 1) / PROBE_THREADS;
  if (nb > WT_NOALLOC_BLOCKS) nb = WT_NOALLOC_BLOCKS;
  probe_kernel<<<(unsigned)nb, PROBE_THREADS, 0, s>>>(a, scratch, guarded);
  if (cudaGetLastError() != cudaSuccess) return WT_ERR_CUDA;
  probe_finish<<<1, PROBE_THREADS, 0, s>>>(scratch, (uint32_t)nb);
  if (cudaGetLastError() != cudaSuccess) return WT_ERR_CUDA;
  ForceSlot rec[2];  // the result record and the guard counter's
  if (cudaMemcpyAsync(rec, scratch + WT_NOALLOC_BLOCKS, sizeof(rec), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return WT_ERR_CUDA;
  const ForceSlot& res = rec[0];
  unsigned int ng = 0;
  memcpy(&ng, &rec[1], sizeof(ng));
  memset(out, 0, sizeof(*out));
  for (int k = 0; k < 9; k++) out->sum[k] = res.f[k];
  for (int g = 0; g < 3; g++) {
    out->raw[3 * g] = res.raw[2 * g];
    out->raw[3 * g + 1] = res.raw[2 * g + 1];
  }
  out->steps = 1;
  out->guarded = ng;
  return WT_OK;
}
