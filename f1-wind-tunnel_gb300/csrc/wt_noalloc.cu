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
// state - per fluid cell and direction, the bounce-back links of the reference
// (src/engine/wgsl.ts:207-223, same boundary precedence, mirrored and duct links
// excluded), summed per solid group in FP64 and as the reference's i32
// fixed-point accumulator.  It is the force path of the step kernel
// (wt_lbm.cu) without the collision.
//
// Scratch: the per-block partial records live in g_probe_scratch, a file-scope
// __device__ array of WT_NOALLOC_BLOCKS + 1 records (96 B each, 98,400 B in all)
// that every GPU which loads the library holds until the process exits.  In
// host code the array's name is only a host-side stand-in, so its device
// address is obtained once per device with cudaGetSymbolAddress (with that
// device current) on the first call on that device; make that first call
// before any stream capture.  Every call overwrites all the records it reads,
// so nothing has to be cleared; the array is shared by all calls, so calls that
// overlap on the GPU (different streams, or different host threads on the same
// device) race and must be serialised by the caller.  No cudaMalloc/cudaFree or
// allocating library routine is called.
#include <string.h>

#include <mutex>

#include "wt_internal.h"
#include "wt_lattice.cuh"

namespace wt {
namespace {

constexpr uint32_t PROBE_THREADS = 256;

static __device__ __align__(256) ForceSlot g_probe_scratch[WT_NOALLOC_BLOCKS + 1];

std::mutex g_probe_mu;
ForceSlot* g_probe_addr[64] = {nullptr};

template <int i>
__device__ __forceinline__ void probe_link(const float* __restrict__ f, uint32_t n, uint32_t idx, uint32_t grp,
                                           float (&gf)[9]) {
  const float v = __ldg(f + (size_t)OPPd(i) * n + idx);
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

__global__ void __launch_bounds__(PROBE_THREADS) probe_kernel(const float* __restrict__ f,
                                                               const uint32_t* __restrict__ solid,
                                                               const float* __restrict__ emit, uint32_t nx,
                                                               uint32_t ny, uint32_t nz, ForceSlot* scratch) {
  const uint32_t n = nx * ny * nz;
  double d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t r[6] = {0, 0, 0, 0, 0, 0};
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (solid[idx] != 0u) continue;
    const int x = (int)(idx % nx), y = (int)((idx / nx) % ny), z = (int)(idx / (nx * ny));
    if (emit != nullptr && emit[idx] < 0.0f) continue;  // duct cells carry no force (wgsl.ts:201,223)
    float gf[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    sfor<19>([&](auto I) {
      constexpr int i = I;
      if constexpr (i != 0) {
        const int sx = x - CXd(i), sy = y - CYd(i), sz = z - CZd(i);
        if (sx < 0 || sx >= (int)nx || sy < 0 || sy >= (int)ny || sz >= (int)nz) return;
        if (sz < 0) return;  // mirrored links carry no force
        const uint32_t g = solid[(uint32_t)sx + nx * ((uint32_t)sy + ny * (uint32_t)sz)];
        if (g != 0u) probe_link<i>(f, n, idx, g > 3u ? 3u : g, gf);
      }
    });
#pragma unroll
    for (int k = 0; k < 9; k++) d[k] += (double)gf[k];
#pragma unroll
    for (int g = 0; g < 3; g++) {
      if (gf[3 * g] != 0.0f) r[2 * g] += (uint32_t)__float2int_rn(gf[3 * g] * 10000.0f);
      if (gf[3 * g + 1] != 0.0f) r[2 * g + 1] += (uint32_t)__float2int_rn(gf[3 * g + 1] * 10000.0f);
    }
  }
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

extern "C" int wt_forces_noalloc(const float* f, const uint32_t* solid, const float* emit, uint32_t nx, uint32_t ny,
                                 uint32_t nz, void* stream, wt_forces* out) {
  using namespace wt;
  if (!f || !solid || !out) return WT_ERR_ARG;
  const uint64_t n = (uint64_t)nx * ny * nz;
  if (nx < 1 || ny < 1 || nz < 1) return WT_ERR_ARG;
  if (n > WT_NOALLOC_MAX_CELLS) return WT_ERR_NOALLOC_LIMIT;
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
  cudaStream_t s = (cudaStream_t)stream;
  uint64_t nb = (n + PROBE_THREADS - 1) / PROBE_THREADS;
  if (nb > WT_NOALLOC_BLOCKS) nb = WT_NOALLOC_BLOCKS;
  probe_kernel<<<(unsigned)nb, PROBE_THREADS, 0, s>>>(f, solid, emit, nx, ny, nz, scratch);
  if (cudaGetLastError() != cudaSuccess) return WT_ERR_CUDA;
  probe_finish<<<1, PROBE_THREADS, 0, s>>>(scratch, (uint32_t)nb);
  if (cudaGetLastError() != cudaSuccess) return WT_ERR_CUDA;
  ForceSlot res;
  if (cudaMemcpyAsync(&res, scratch + WT_NOALLOC_BLOCKS, sizeof(res), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return WT_ERR_CUDA;
  memset(out, 0, sizeof(*out));
  for (int k = 0; k < 9; k++) out->sum[k] = res.f[k];
  for (int g = 0; g < 3; g++) {
    out->raw[3 * g] = res.raw[2 * g];
    out->raw[3 * g + 1] = res.raw[2 * g + 1];
  }
  out->steps = 1;
  return WT_OK;
}
