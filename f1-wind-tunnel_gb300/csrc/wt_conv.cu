// 3-D convolution of the warm-start network as an implicit GEMM on the
// 5th-generation tensor cores (tcgen05, kind::f16 with BF16 operands, FP32
// accumulation in tensor memory).
//
// One kernel, three operand gathers:
//   FWD    D[m][co]        = sum_k A[m][k] B[co][k],  A[m][(t,ci)]  = x[m + off(t)][ci],  B = w[co][(t,ci)]
//   DGRAD  D[m][ci]        = sum_k A[m][k] B[ci][k],  A[m][(t,co)]  = dy[m - off(t)][co], B = wt[ci][(t,co)]
//   WGRAD  D[(t,ci)][co]   = sum_m A[(t,ci)][m] B[co][m], A = x[m + off(t)][ci], B = dy[m][co]
// (m a voxel of the batch's grid, out-of-grid neighbours read as zero).
//
// CTA: 128 threads, a 128 x N tile (N <= 128).  The K dimension runs in
// slices of 64 through two shared-memory stages: all threads gather a slice of
// A (128 rows) and B (N rows) into the canonical K-major, non-swizzled
// core-matrix layout (8 rows x 16 bytes per core matrix; core matrices adjacent
// along K 128 B apart, along M/N 1024 B apart), one thread issues four
// tcgen05.mma (K = 16 each) and commits them to the stage's mbarrier, and the
// next slice is gathered into the other stage meanwhile.  The accumulator
// (128 lanes x N FP32 columns) lives in tensor memory; the epilogue reads it
// with tcgen05.ld (warp w owns lanes 32w..32w+31).  Every mbarrier wait is
// bounded: on expiry the kernel raises g_conv_error, still waits (bounded) for
// its own MMAs, frees its tensor memory and returns.
#include <atomic>
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>

#include "wt_internal.h"
#include "wt_net.h"

namespace wt {

__device__ int g_conv_error;

std::string& net_error() {
  thread_local std::string e;
  return e;
}

namespace {

constexpr int BM = 128, BK = 64, NTHREADS = 128;
constexpr uint32_t STAGE_BYTES = BM * BK * 2;       // one operand slice, 16 KB
constexpr uint32_t SMEM_BYTES = 4 * STAGE_BYTES + 64;  // A0 A1 B0 B1 + barriers + TMEM slot
constexpr uint32_t TMEM_COLS = 128;
constexpr uint32_t WAIT_LIMIT = 1u << 21;

enum Mode { FWD = 0, DGRAD = 1, WGRAD = 2 };

struct GemmArgs {
  uint32_t batch, d, h, w;
  uint32_t cin, cout, taps;
  uint32_t M, N, K;        // GEMM extents
  uint32_t k_chunk;        // K per split (WGRAD; multiple of BK), K otherwise
  const __nv_bfloat16* a;  // FWD x, DGRAD dy, WGRAD x
  const __nv_bfloat16* b;  // FWD w, DGRAD wt, WGRAD dy
  const float* bias;
  void* out;               // FWD bf16 y[M][cout], DGRAD f32 dx[M][cin], WGRAD f32 ws[split][M][N]
  int relu;
  uint32_t stage_wait;     // polls of a K-slice stage wait (WAIT_LIMIT unless a test lowers it)
};

// Poll budget of the pipeline's stage waits for the next launches (see
// wt_net_set_stage_wait_limit); the drain before tensor memory is freed always
// uses WAIT_LIMIT.
std::atomic<uint32_t> g_stage_wait{WAIT_LIMIT};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading (K-direction)
// and stride (M/N-direction) byte offsets, all >> 4; bits 46-47 = 1 (the
// descriptor version of this architecture); no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ int tap_dz(uint32_t t, uint32_t taps) { return taps == 27 ? (int)(t / 9) - 1 : 0; }
__device__ __forceinline__ int tap_dy(uint32_t t, uint32_t taps) { return taps == 27 ? (int)((t / 3) % 3) - 1 : 0; }
__device__ __forceinline__ int tap_dx(uint32_t t, uint32_t taps) { return taps == 27 ? (int)(t % 3) - 1 : 0; }

// Byte offset of 16-byte chunk (row r, k-group g) in the core-matrix layout.
__device__ __forceinline__ uint32_t chunk_off(uint32_t r, uint32_t g) { return ((r >> 3) * 8u + g) * 128u + (r & 7u) * 16u; }

__device__ __forceinline__ uint4 ld16(const __nv_bfloat16* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }


// Grid position of a voxel (x fastest, then y, z, batch item).
struct VoxPos {
  int x, y, z;
  int64_t vox;
  bool ok;
};

__device__ __forceinline__ VoxPos vox_pos(const GemmArgs& p, uint32_t m, uint32_t end) {
  VoxPos r;
  r.ok = m < end;
  const uint32_t mm = r.ok ? m : 0u;
  r.x = (int)(mm % p.w);
  r.y = (int)((mm / p.w) % p.h);
  r.z = (int)((mm / (p.w * p.h)) % p.d);
  r.vox = mm;
  return r;
}

// Index of the voxel r + (dz, dy, dx) in the same batch item, or -1 outside the grid.
__device__ __forceinline__ int64_t nbr(const GemmArgs& p, const VoxPos& r, int dz, int dy, int dx) {
  const int xx = r.x + dx, yy = r.y + dy, zz = r.z + dz;
  if ((unsigned)xx >= p.w || (unsigned)yy >= p.h || (unsigned)zz >= p.d) return -1;
  return r.vox + ((int64_t)dz * p.h + dy) * p.w + dx;
}

// Gather K slice [k0, k0 + 64) of both operands into the stage buffers sa, sb.
//   FWD / DGRAD: thread t owns A row t (a voxel, position precomputed in `row`)
//   and B row t (a weight row); each 16-byte chunk is 8 consecutive channels of
//   one tap, one vector load.
//   WGRAD: K runs over voxels; thread t owns voxel k0 + (t & 63) and half
//   (t >> 6) of the A rows (taps x channels) and B rows (output channels); it
//   loads 8 channels of its voxel with one vector load and stores them into 8
//   rows of the K-major tile (2-byte stores).
// Rows past the MMA's N (B) are never read and not written; K past the range
// is zero in both operands.
template <int MODE>
__device__ __forceinline__ void gather(const GemmArgs& p, const VoxPos& row, uint32_t tile_m, uint32_t n_mma,
                                       uint32_t k0, uint32_t k_end, uint8_t* sa, uint8_t* sb) {
  const uint32_t t = threadIdx.x;
  if constexpr (MODE == FWD || MODE == DGRAD) {
    const uint32_t C = (MODE == FWD) ? p.cin : p.cout;
    const int sg = (MODE == FWD) ? 1 : -1;
    uint32_t tap = k0 / C, c = k0 % C;
#pragma unroll
    for (uint32_t g = 0; g < 8; g++) {
      const uint32_t k = k0 + 8 * g;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (row.ok && k < k_end) {
        const int64_t sv = nbr(p, row, sg * tap_dz(tap, p.taps), sg * tap_dy(tap, p.taps), sg * tap_dx(tap, p.taps));
        if (sv >= 0) v = ld16(p.a + (size_t)sv * C + c);
      }
      *reinterpret_cast<uint4*>(sa + chunk_off(t, g)) = v;
      c += 8;
      if (c >= C) {
        c = 0;
        tap++;
      }
    }
    if (t < n_mma) {
#pragma unroll
      for (uint32_t g = 0; g < 8; g++) {
        const uint32_t k = k0 + 8 * g;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (t < p.N && k < k_end) v = ld16(p.b + (size_t)t * p.K + k);
        *reinterpret_cast<uint4*>(sb + chunk_off(t, g)) = v;
      }
    }
  } else {
    const uint32_t j = t & 63u, half = t >> 6;
    const VoxPos m = vox_pos(p, k0 + j, k_end);
    const uint32_t jo = (j & 7u) * 2u, jg = j >> 3;
    // A rows half*64 .. +63 = (tap, ci) rows tile_m + ...
#pragma unroll
    for (uint32_t q = 0; q < 8; q++) {
      const uint32_t r0 = half * 64u + 8u * q, R0 = tile_m + r0;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (m.ok && R0 < p.M) {
        const uint32_t tap = R0 / p.cin, ci = R0 % p.cin;
        const int64_t sv = nbr(p, m, tap_dz(tap, p.taps), tap_dy(tap, p.taps), tap_dx(tap, p.taps));
        if (sv >= 0) v = ld16(p.a + (size_t)sv * p.cin + ci);
      }
      const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int e = 0; e < 8; e++)
        *reinterpret_cast<uint16_t*>(sa + chunk_off(r0 + e, jg) + jo) = (uint16_t)(w4[e >> 1] >> ((e & 1) * 16));
    }
    // B rows (output channels) half*64 .. +63, only those the MMA reads
#pragma unroll
    for (uint32_t q = 0; q < 8; q++) {
      const uint32_t r0 = half * 64u + 8u * q;
      if (r0 >= n_mma) break;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (m.ok && r0 < p.N) v = ld16(p.b + (size_t)m.vox * p.cout + r0);
      const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int e = 0; e < 8; e++)
        *reinterpret_cast<uint16_t*>(sb + chunk_off(r0 + e, jg) + jo) = (uint16_t)(w4[e >> 1] >> ((e & 1) * 16));
    }
  }
}

template <int MODE>
__global__ void __launch_bounds__(NTHREADS, 1) conv_gemm_kernel(GemmArgs p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  // stage s: A at smem + s * STAGE_BYTES, B at smem + (2 + s) * STAGE_BYTES
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 4 * STAGE_BYTES);  // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 4 * STAGE_BYTES + 16);
  const uint32_t t = threadIdx.x, warp = t >> 5;
  const uint32_t tile_m = blockIdx.x * BM;
  const uint32_t k_begin = blockIdx.y * p.k_chunk;
  const uint32_t k_end = min(p.K, k_begin + p.k_chunk);
  const uint32_t nk = (k_end > k_begin) ? (k_end - k_begin + BK - 1) / BK : 0;
  const uint32_t n_mma = ((p.N + 15) / 16) * 16;
  const uint32_t idesc = idesc_bf16(BM, n_mma);

  if (t == 0) {
    mbar_init(smem_u32(&bars[0]), 1);
    mbar_init(smem_u32(&bars[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const VoxPos row_pos = vox_pos(p, tile_m + t, p.M);  // FWD / DGRAD: this thread's A row (a voxel)
  bool ok = true;
  uint32_t issued = 0;  // K slices whose MMAs were issued (uniform across the block)
  for (uint32_t kt = 0; kt < nk; kt++) {
    const uint32_t s = kt & 1u;
    bool w = true;
    if (kt >= 2) w = mbar_wait(smem_u32(&bars[s]), ((kt >> 1) - 1) & 1u, p.stage_wait);  // MMAs of slice kt-2 done
    if (!__syncthreads_and(w)) {  // the block stops together
      ok = false;
      break;
    }
    uint8_t* const sa = smem + s * STAGE_BYTES;
    uint8_t* const sb = smem + (2u + s) * STAGE_BYTES;
    gather<MODE>(p, row_pos, tile_m, n_mma, k_begin + kt * BK, k_end, sa, sb);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (uint32_t kk = 0; kk < BK / 16; kk++) {
        const uint64_t ad = smem_desc(a0 + kk * 256u, 128u, 1024u);
        const uint64_t bd = smem_desc(b0 + kk * 256u, 128u, 1024u);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[s]))
                   : "memory");
    }
    issued++;
  }
  // All MMAs done: the last commit covers every earlier one of the issuing thread.
  if (issued > 0) {
    const uint32_t last = issued - 1;
    const bool done = mbar_wait(smem_u32(&bars[last & 1u]), (last >> 1) & 1u, WAIT_LIMIT);
    ok = ok && done;
  }
  if (!ok && t == 0) atomicExch(&g_conv_error, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // ---- epilogue: lane = row t of the tile, 16 columns per tcgen05.ld
  const uint32_t row = tile_m + t;
  const uint32_t taddr = tmem + ((warp * 32u) << 16);
  for (uint32_t c0 = 0; c0 < n_mma; c0 += 16) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr + c0)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (!ok || row >= p.M || nk == 0) continue;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const uint32_t col = c0 + j;
      if (col >= p.N) break;
      float v = __uint_as_float(r[j]);
      if constexpr (MODE == FWD) {
        if (p.bias) v += p.bias[col];
        if (p.relu) v = fmaxf(v, 0.0f);
        reinterpret_cast<__nv_bfloat16*>(p.out)[(size_t)row * p.N + col] = __float2bfloat16_rn(v);
      } else if constexpr (MODE == DGRAD) {
        reinterpret_cast<float*>(p.out)[(size_t)row * p.N + col] = v;
      } else {
        reinterpret_cast<float*>(p.out)[((size_t)blockIdx.y * p.M + row) * p.N + col] = v;
      }
    }
  }
  if (nk == 0 && row < p.M) {  // empty K range: the product is zero
    for (uint32_t col = 0; col < p.N; col++) {
      if constexpr (MODE == FWD) {
        float v = p.bias ? p.bias[col] : 0.0f;
        if (p.relu) v = fmaxf(v, 0.0f);
        reinterpret_cast<__nv_bfloat16*>(p.out)[(size_t)row * p.N + col] = __float2bfloat16_rn(v);
      } else if constexpr (MODE == DGRAD) {
        reinterpret_cast<float*>(p.out)[(size_t)row * p.N + col] = 0.0f;
      } else {
        reinterpret_cast<float*>(p.out)[((size_t)blockIdx.y * p.M + row) * p.N + col] = 0.0f;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// dw[co][t][ci] = sum over splits of ws[split][(t, ci)][co].
__global__ void wgrad_reduce_kernel(const float* __restrict__ ws, float* __restrict__ dw, uint32_t splits,
                                    uint32_t rows, uint32_t cout, uint32_t taps, uint32_t cin) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cout) return;
  const uint32_t row = i / cout, co = i % cout;  // row = t * cin + ci
  double s = 0.0;
  for (uint32_t k = 0; k < splits; k++) s += ws[((size_t)k * rows + row) * cout + co];
  const uint32_t tap = row / cin, ci = row % cin;
  dw[((size_t)co * taps + tap) * cin + ci] = (float)s;
}

int nfail(int code, const std::string& m) {
  net_error() = m;
  return code;
}

int check_shape(const wt_conv_shape* s, const char* what) {
  if (!s) return nfail(WT_ERR_ARG, std::string(what) + ": null shape");
  if (s->taps != 27 && s->taps != 1) return nfail(WT_ERR_ARG, std::string(what) + ": taps must be 27 or 1");
  if (s->cin == 0 || s->cout == 0 || s->cin % 8 || s->cout % 8 || s->cin > 128 || s->cout > 128)
    return nfail(WT_ERR_ARG, std::string(what) + ": channel counts must be multiples of 8 in [8, 128]");
  if (s->batch == 0 || s->d == 0 || s->h == 0 || s->w == 0) return nfail(WT_ERR_ARG, std::string(what) + ": empty grid");
  if ((uint64_t)s->batch * s->d * s->h * s->w >= (1ull << 31)) return nfail(WT_ERR_ARG, std::string(what) + ": grid too large");
  return WT_OK;
}

constexpr uint32_t WGRAD_SPLITS_MAX = 64;

uint32_t wgrad_splits(uint64_t voxels) {
  // about 4096 voxels (64 slices of 64) per split, at most WGRAD_SPLITS_MAX
  uint64_t s = (voxels + 4095) / 4096;
  if (s < 1) s = 1;
  if (s > WGRAD_SPLITS_MAX) s = WGRAD_SPLITS_MAX;
  return (uint32_t)s;
}

template <int MODE>
int launch_gemm(const GemmArgs& p, uint32_t splits, cudaStream_t st) {
  cudaError_t ea = cudaFuncSetAttribute(conv_gemm_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  if (ea != cudaSuccess) return nfail(WT_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ea));
  const dim3 grid((p.M + BM - 1) / BM, splits);
  conv_gemm_kernel<MODE><<<grid, NTHREADS, SMEM_BYTES, st>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nfail(WT_ERR_CUDA, std::string("conv kernel launch: ") + cudaGetErrorString(e));
  return WT_OK;
}

GemmArgs base_args(const wt_conv_shape* s) {
  GemmArgs p = {};
  p.batch = s->batch; p.d = s->d; p.h = s->h; p.w = s->w;
  p.cin = s->cin; p.cout = s->cout; p.taps = s->taps;
  p.stage_wait = g_stage_wait.load();
  return p;
}

}  // namespace
}  // namespace wt

using namespace wt;

extern "C" {

int wt_conv3d_forward(const wt_conv_shape* s, const void* x, const void* w, const float* bias, void* y, int relu,
                      void* stream) {
  int rc = check_shape(s, "wt_conv3d_forward");
  if (rc) return rc;
  if (!x || !w || !y) return nfail(WT_ERR_ARG, "wt_conv3d_forward: null tensor");
  GemmArgs p = base_args(s);
  p.M = s->batch * s->d * s->h * s->w;
  p.N = s->cout;
  p.K = s->taps * s->cin;
  p.k_chunk = p.K;
  p.a = static_cast<const __nv_bfloat16*>(x);
  p.b = static_cast<const __nv_bfloat16*>(w);
  p.bias = bias;
  p.out = y;
  p.relu = relu;
  return launch_gemm<FWD>(p, 1, static_cast<cudaStream_t>(stream));
}

int wt_conv3d_backward_data(const wt_conv_shape* s, const void* dy, const void* wt, float* dx, void* stream) {
  int rc = check_shape(s, "wt_conv3d_backward_data");
  if (rc) return rc;
  if (!dy || !wt || !dx) return nfail(WT_ERR_ARG, "wt_conv3d_backward_data: null tensor");
  GemmArgs p = base_args(s);
  p.M = s->batch * s->d * s->h * s->w;
  p.N = s->cin;
  p.K = s->taps * s->cout;
  p.k_chunk = p.K;
  p.a = static_cast<const __nv_bfloat16*>(dy);
  p.b = static_cast<const __nv_bfloat16*>(wt);
  p.out = dx;
  return launch_gemm<DGRAD>(p, 1, static_cast<cudaStream_t>(stream));
}

size_t wt_conv3d_workspace_bytes(const wt_conv_shape* s) {
  if (check_shape(s, "wt_conv3d_workspace_bytes")) return 0;
  const uint64_t vox = (uint64_t)s->batch * s->d * s->h * s->w;
  return (size_t)wgrad_splits(vox) * s->taps * s->cin * s->cout * sizeof(float);
}

int wt_conv3d_backward_weight(const wt_conv_shape* s, const void* x, const void* dy, float* dw, void* workspace,
                              void* stream) {
  int rc = check_shape(s, "wt_conv3d_backward_weight");
  if (rc) return rc;
  if (!x || !dy || !dw || !workspace) return nfail(WT_ERR_ARG, "wt_conv3d_backward_weight: null tensor");
  GemmArgs p = base_args(s);
  const uint64_t vox = (uint64_t)s->batch * s->d * s->h * s->w;
  const uint32_t splits = wgrad_splits(vox);
  p.M = s->taps * s->cin;
  p.N = s->cout;
  p.K = (uint32_t)vox;
  p.k_chunk = (uint32_t)(((vox + splits - 1) / splits + BK - 1) / BK * BK);
  p.a = static_cast<const __nv_bfloat16*>(x);
  p.b = static_cast<const __nv_bfloat16*>(dy);
  p.out = workspace;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = launch_gemm<WGRAD>(p, splits, st);
  if (rc) return rc;
  const uint32_t total = p.M * p.N;
  wgrad_reduce_kernel<<<(total + 255) / 256, 256, 0, st>>>(static_cast<const float*>(workspace), dw, splits, p.M,
                                                           s->cout, s->taps, s->cin);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nfail(WT_ERR_CUDA, std::string("wgrad reduce: ") + cudaGetErrorString(e));
  return WT_OK;
}

int wt_net_check(void) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return nfail(WT_ERR_CUDA, std::string("wt_net_check: ") + cudaGetErrorString(e));
  int flag = 0, zero = 0;
  cudaMemcpyFromSymbol(&flag, g_conv_error, sizeof(int));
  cudaMemcpyToSymbol(g_conv_error, &zero, sizeof(int));
  return flag;
}

const char* wt_net_last_error(void) { return net_error().c_str(); }

uint32_t wt_net_set_stage_wait_limit(uint32_t polls) { return g_stage_wait.exchange(polls); }

}  // extern "C"
