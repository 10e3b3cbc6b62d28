// D3Q19 tables as compile-time functions, cell-word bits and the population
// storage formats.  The velocity order, opposite and z-mirror permutations and
// weights are those of the reference (src/engine/wgsl.ts:123-133); they are
// restated as constexpr functions so that every per-direction branch folds away
// inside the unrolled kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <utility>

namespace wt {

__host__ __device__ constexpr int CXd(int i) {
  return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1 : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int CYd(int i) {
  return (i == 3 || i == 7 || i == 10 || i == 15 || i == 17) ? 1 : (i == 4 || i == 8 || i == 9 || i == 16 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int CZd(int i) {
  return (i == 5 || i == 11 || i == 14 || i == 15 || i == 18) ? 1 : (i == 6 || i == 12 || i == 13 || i == 16 || i == 17) ? -1 : 0;
}
__host__ __device__ constexpr int OPPd(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }
// Reflection z -> -z of direction i.
__host__ __device__ constexpr int ZMIRd(int i) {
  return i == 5 ? 6 : i == 6 ? 5 : i == 11 ? 13 : i == 13 ? 11 : i == 12 ? 14 : i == 14 ? 12
       : i == 15 ? 17 : i == 17 ? 15 : i == 16 ? 18 : i == 18 ? 16 : i;
}
// Weights exactly as the reference's f32 literals.
__host__ __device__ constexpr float Wd(int i) { return i == 0 ? 0.33333334f : (i < 7 ? 0.055555556f : 0.027777778f); }

// Cell word (one u32 per cell, built at voxelization):
//   bit 0      cell is solid
//   bits 1-18  direction i of this fluid cell bounces back off a solid source
//              cell (the `solid[sidx] != 0` branch of wgsl.ts:221, mirror included)
//   bit 19     belt contact: floor speed 0 under this y=0 cell (wgsl.ts:192-197)
//   bit 20     duct cell (emit < 0): no force, axial velocity relaxation (wgsl.ts:201,248)
//   bit 21     at least one force-carrying link (non-mirrored, not a duct cell)
constexpr uint32_t CW_SOLID = 1u;
constexpr uint32_t CW_LINKS = 0x7fffeu;
constexpr uint32_t CW_BELT = 1u << 19;
constexpr uint32_t CW_DUCT = 1u << 20;
constexpr uint32_t CW_FORCE = 1u << 21;

// Compile-time loop: f(std::integral_constant<int, I>) for I = 0..N-1.
template <int... Is, class F>
__device__ __forceinline__ void sfor_impl(std::integer_sequence<int, Is...>, F&& f) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(std::make_integer_sequence<int, N>{}, f);
}

// a / b from r = RN(1/b) by Markstein's correction step (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): q = RN(a r) lies within one ulp of a/b, the remainder
// e = a - q b is exact under a fused multiply-add, and RN(q + e r) = RN(a/b).
// The remainder stays exact (a multiple of 2^-149 at worst) and q normal for
// |a| >= 2^-60 or a = 0 with b in [2^-14, 2^14]; callers keep to that range.
__device__ __forceinline__ float div_rcp(float a, float b, float r) {
  const float q = __fmul_rn(a, r);
  return __fmaf_rn(__fmaf_rn(-q, b, a), r, q);
}

// Population storage.  F32 keeps f_i; F16/BF16 keep f_i - w_i, which is small
// and keeps the significant bits of the deviation from rest.
struct StoreF32 {
  typedef float T;
  static constexpr uint32_t id = 0;
  // step-kernel registers: 56 (no spills; 9 blocks of 128 per SM), measured
  // against 48 (5 blocks of 256, small spills) to 64: 71.2 % -> 73.6 % of HBM
  static constexpr int max_regs = 56;
  __device__ __forceinline__ static float ld(const T* p, float) { return __ldg(p); }
  // L2-coherent load (ld.global.cg): for populations another block may have
  // rewritten earlier in the same launch (the persistent batch kernel)
  __device__ __forceinline__ static float ld_coh(const T* p, float) { return __ldcg(p); }
  __device__ __forceinline__ static float ld_smem(const T* p, float) { return *p; }
  __device__ __forceinline__ static void st(T* p, float v, float) { *p = v; }
};
// F16 keeps (f_i - w_i) * 2^14: the deviations (~1e-2 and below) then stay in
// half's normal range down to ~4e-9 instead of turning subnormal below 6e-5;
// the power-of-two scale adds no rounding.  Both conversions are single fused
// multiply-adds with the same bits as the separate operations: h * 2^-14 and
// v * 2^14, w * 2^14 are exact, so fma(h, 2^-14, w) = RN(w + h 2^-14) and
// fma(v, 2^14, -w 2^14) = RN(2^14 (v - w)) = 2^14 RN(v - w) (|v| < 2^100).
constexpr float F16_SCALE = 16384.0f, F16_INV = 1.0f / 16384.0f;
struct StoreF16 {
  typedef __half T;
  static constexpr uint32_t id = 1;
  // step-kernel registers: 48 (10 blocks of 128 per SM, a few bytes of spills in
  // some variants), measured against 52 and 56 with the moment-form collision:
  // 48.2 -> 50.2 GLUPS at 512x192x160, 45.7 -> 46.5 at 256x96x80 (52 = 56)
  static constexpr int max_regs = 48;
  __device__ __forceinline__ static float ld(const T* p, float w) { return __fmaf_rn(__half2float(__ldg(p)), F16_INV, w); }
  __device__ __forceinline__ static float ld_smem(const T* p, float w) { return __fmaf_rn(__half2float(*p), F16_INV, w); }
  __device__ __forceinline__ static void st(T* p, float v, float w) {
    *p = __float2half_rn(__fmaf_rn(v, F16_SCALE, -(w * F16_SCALE)));
  }
  // the stored deviation itself, in units of 2^-14 (the step kernel's working form)
  static constexpr float S = F16_SCALE;
  __device__ __forceinline__ static float ldd(const T* p) { return __half2float(__ldg(p)); }
  __device__ __forceinline__ static float ldd_coh(const T* p) { return __half2float(__ldcg(p)); }
  __device__ __forceinline__ static void std_(T* p, float d) { *p = __float2half_rn(d); }
};
struct StoreBF16 {
  typedef __nv_bfloat16 T;
  static constexpr uint32_t id = 2;
  // step-kernel registers: 48, as for F16 (45.9 -> 46.6 GLUPS at 256x96x80)
  static constexpr int max_regs = 48;
  __device__ __forceinline__ static float ld(const T* p, float w) { return w + __bfloat162float(__ldg(p)); }
  __device__ __forceinline__ static float ld_smem(const T* p, float w) { return w + __bfloat162float(*p); }
  __device__ __forceinline__ static void st(T* p, float v, float w) { *p = __float2bfloat16_rn(v - w); }
  static constexpr float S = 1.0f;
  __device__ __forceinline__ static float ldd(const T* p) { return __bfloat162float(__ldg(p)); }
  __device__ __forceinline__ static float ldd_coh(const T* p) { return __bfloat162float(__ldcg(p)); }
  __device__ __forceinline__ static void std_(T* p, float d) { *p = __float2bfloat16_rn(d); }
};

}  // namespace wt
