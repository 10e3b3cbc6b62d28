// D3Q19 regularized LBM with Smagorinsky LES: the collide-stream step of the
// reference (LBM_STEP, src/engine/wgsl.ts:157-291) and its init (LBM_INIT,
// wgsl.ts:141-155), as an in-place AA-pattern single lattice.
//
// Storage: one array per direction, pop[i*np + idx].  Two step kinds alternate:
//   gather step  (odd steps 1, 3, ...): state C -> state S
//       reads  f_i(x) = pop[opp(i)][x - c_i]           (neighbour slots)
//       writes f*_j(x) -> pop[j][x + c_j]                (neighbour slots)
//   local step   (even steps 2, 4, ...): state S -> state C
//       reads  f_i(x) = pop[i][x]                        (own slots)
//       writes f*_j(x) -> pop[opp(j)][x]                 (own slots)
// State C ("canonical", after every even number of steps) holds the
// post-collision populations f*_j(x) at pop[opp(j)][x] - the same information
// as the reference's buffer fA after engine.ts:710's even-length loop - and
// does not depend on the link masks, so re-voxelization between calls is exact.
//
// Boundaries keep the reference's precedence (wgsl.ts:207-227): inlet (x<0),
// outlet (x>=nx, feq of the cell's previous velocity), moving floor (y<0,
// bounce-back + 6 w c_x u_floor), far field (y>=ny or z>=nz), symmetry mirror
// (z<0), solid bounce-back, interior.  In AA form the bounce-back, floor and
// mirror values are redirected on write so that every read of the next step
// finds its value: bounce-back/floor -> own slot pop[opp(j)][x]; mirror ->
// pop[zmir(j)][(x + c_jx, y + c_jy, 0)].  Every slot written in a step is read
// in that step only by the writing thread, so the step has no races.
//
// Arithmetic matches the reference operation for operation (no contraction,
// compile with -fmad=false): sums run in the reference's direction order, and
// only products with a zero lattice coefficient are dropped, which leaves every
// finite result bit-identical.
//
// Roofline: 19 loads + 19 stores of the storage type + one 4-byte cell word per
// cell and step (156 B/LUP in f32, 80 B/LUP in f16/bf16); the (u, rho) field
// write (16 B) happens only on the last step of a call.
#include "wt_internal.h"
#include "wt_lattice.cuh"

namespace wt {

namespace {

constexpr int BX_MAX = 256;

struct CellOut {
  float ux, uy, uz, rho;
  bool guard;
};

// feq of wgsl.ts:135-138 with rho = 1 (outlet populations from the previous velocity).
template <int i>
__device__ __forceinline__ float feq_rho1(float ux, float uy, float uz) {
  constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
  float cu = 0.0f;
  bool first = true;
  if constexpr (cx != 0) { cu = (cx > 0) ? ux : -ux; first = false; }
  if constexpr (cy != 0) { if (first) cu = (cy > 0) ? uy : -uy; else cu = (cy > 0) ? cu + uy : cu - uy; first = false; }
  if constexpr (cz != 0) { if (first) cu = (cz > 0) ? uz : -uz; else cu = (cz > 0) ? cu + uz : cu - uz; }
  const float uu = ux * ux + uy * uy + uz * uz;
  return Wd(i) * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
}

// c_i . u with the reference's x, y, z order and zero terms dropped.
template <int i>
__device__ __forceinline__ float cdot(float ux, float uy, float uz) {
  constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
  float cu = 0.0f;
  bool first = true;
  if constexpr (cx != 0) { cu = (cx > 0) ? ux : -ux; first = false; }
  if constexpr (cy != 0) { if (first) cu = (cy > 0) ? uy : -uy; else cu = (cy > 0) ? cu + uy : cu - uy; first = false; }
  if constexpr (cz != 0) { if (first) cu = (cz > 0) ? uz : -uz; else cu = (cz > 0) ? cu + uz : cu - uz; }
  return cu;
}

__device__ __forceinline__ bool is_bad(float x) { return (__float_as_uint(x) & 0x7f800000u) == 0x7f800000u; }

// Moments, divergence guard, duct relaxation, regularized + Smagorinsky collision
// (wgsl.ts:231-272).  f[] in, fo[] out.
__device__ __forceinline__ CellOut collide(const float (&f)[19], float (&fo)[19], float tau0, float u_in, float ks2,
                                           bool duct, const float (&feq_guard)[19], float guard_uu) {
  CellOut o;
  float rho = 0.0f, mx = 0.0f, my = 0.0f, mz = 0.0f;
  sfor<19>([&](auto I) {
    constexpr int i = I;
    rho = rho + f[i];
    if constexpr (CXd(i) > 0) mx = mx + f[i];
    if constexpr (CXd(i) < 0) mx = mx - f[i];
    if constexpr (CYd(i) > 0) my = my + f[i];
    if constexpr (CYd(i) < 0) my = my - f[i];
    if constexpr (CZd(i) > 0) mz = mz + f[i];
    if constexpr (CZd(i) < 0) mz = mz - f[i];
  });
  const float den = (rho < 1e-4f) ? 1e-4f : rho;
  // u = m / den with one correctly rounded reciprocal and Markstein corrections:
  // the quotients only matter for rho in [0.3, 3] (any other rho takes the guard
  // below), where they equal IEEE division for |m| >= 2^-60 or m = 0; a warp
  // holding a smaller nonzero numerator takes IEEE division (no such state
  // arises from populations near w_i, whose sums are multiples of ~2^-30).
  float rcp = __frcp_rn(den);
  float ux = div_rcp(mx, den, rcp), uy = div_rcp(my, den, rcp), uz = div_rcp(mz, den, rcp);
  {
    const uint32_t small = min(min((__float_as_uint(mx) & 0x7fffffffu) - 1u, (__float_as_uint(my) & 0x7fffffffu) - 1u),
                               (__float_as_uint(mz) & 0x7fffffffu) - 1u);  // zero -> 0xffffffff
    const bool tiny = small < 0x21800000u - 1u;                             // 0 < |m| < 2^-60
    if (__any_sync(__activemask(), tiny) && tiny) {
      ux = __fdiv_rn(mx, den); uy = __fdiv_rn(my, den); uz = __fdiv_rn(mz, den);
    }
  }
  float g[19];
  // length(u) > 0.35 (wgsl.ts:238) <=> u.u > guard_uu: sqrt is correctly rounded and
  // monotonic, and guard_uu is the largest float whose square root rounds to <= 0.35f.
  bool guard = is_bad(rho) || is_bad(ux) || is_bad(uy) || is_bad(uz) || rho < 0.3f || rho > 3.0f ||
               (ux * ux + uy * uy + uz * uz) > guard_uu;
  // Divergence guard (wgsl.ts:238-243): rho = 1, u = u_in/2, f = feq(1, u); the
  // equilibria are the same for every cell and come precomputed from the host.
  if (guard) {
    rho = 1.0f;
    rcp = 1.0f;
    ux = u_in * 0.5f; uy = 0.0f; uz = 0.0f;
  }
  sfor<19>([&](auto I) { g[I] = f[I]; });
  if (guard) sfor<19>([&](auto I) { g[I] = feq_guard[I]; });
  if (duct) {
    const float t = 0.04f, tu = 1.0f - 0.04f;
    ux = ux * tu + (0.55f * u_in) * t;
    uy = uy * tu + uy * t;
    uz = uz * tu + uz * t;
  }
  const float uu = ux * ux + uy * uy + uz * uz;
  const float uu15 = 1.5f * uu;
  const float wr0 = Wd(0) * rho, wr1 = Wd(1) * rho, wr2 = Wd(7) * rho;
  float eq[19];
  float pxx = 0.0f, pyy = 0.0f, pzz = 0.0f, pxy = 0.0f, pxz = 0.0f, pyz = 0.0f;
  // Pi^neq accumulated as each equilibrium is formed, directions in order 0..18
  // (every sum keeps the reference's order), so each incoming population dies
  // as soon as its term is taken.
  auto acc = [&](auto I) {
    constexpr int i = I;
    constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
    const float ne = g[i] - eq[i];
    if constexpr (cx != 0) pxx = pxx + ne;
    if constexpr (cy != 0) pyy = pyy + ne;
    if constexpr (cz != 0) pzz = pzz + ne;
    if constexpr (cx * cy > 0) pxy = pxy + ne;
    if constexpr (cx * cy < 0) pxy = pxy - ne;
    if constexpr (cx * cz > 0) pxz = pxz + ne;
    if constexpr (cx * cz < 0) pxz = pxz - ne;
    if constexpr (cy * cz > 0) pyz = pyz + ne;
    if constexpr (cy * cz < 0) pyz = pyz - ne;
  };
  // Opposite directions share 3 c.u (exact negation) and 4.5 (c.u)^2 (identical bits).
  eq[0] = wr0 * (1.0f + 3.0f * 0.0f + 4.5f * 0.0f * 0.0f - uu15);
  acc(std::integral_constant<int, 0>{});
  sfor<9>([&](auto P) {
    constexpr int i = 2 * P + 1;  // odd member of the pair (i, i + 1)
    const float cu = cdot<i>(ux, uy, uz);
    const float t3 = 3.0f * cu;
    const float t45 = 4.5f * cu * cu;
    const float wr = (i < 7 ? wr1 : wr2);
    eq[i] = wr * (1.0f + t3 + t45 - uu15);
    eq[i + 1] = wr * (1.0f - t3 + t45 - uu15);
    acc(std::integral_constant<int, i>{});
    acc(std::integral_constant<int, i + 1>{});
  });
  const float q = __fsqrt_rn(pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz));
  // ks2 q / rho with rho in [0.3, 3] (or 1 after the guard) and rcp = RN(1/rho):
  // IEEE-exact for ks2 q >= 2^-60; below that the quotient (< 2^-58) vanishes in
  // tau0^2 + quotient (tau0 >= 2^-10 is enforced by the API), as the exact one does.
  const float tau = 0.5f * (tau0 + __fsqrt_rn(tau0 * tau0 + div_rcp(ks2 * q, rho, rcp)));
  const float omega = __frcp_rn(tau);  // correctly rounded 1/tau, the same bits as 1.0f / tau
  const float c1 = (1.0f - omega) * 4.5f;
  const float k0 = c1 * Wd(0), k1 = c1 * Wd(1), k2 = c1 * Wd(7);
  // (c_a c_a - 1/3) with the reference's f32 third: 1 - third rounds to 0x1.555554p-1
  constexpr float third = 0x1.555556p-2f;
  const float a_xx = (1.0f - third) * pxx, b_xx = (0.0f - third) * pxx;
  const float a_yy = (1.0f - third) * pyy, b_yy = (0.0f - third) * pyy;
  const float a_zz = (1.0f - third) * pzz, b_zz = (0.0f - third) * pzz;
  const float pxy2 = 2.0f * pxy, pxz2 = 2.0f * pxz, pyz2 = 2.0f * pyz;
  fo[0] = eq[0] + k0 * ((b_xx + b_yy) + b_zz);
  sfor<9>([&](auto P) {  // (c_a c_b - delta/3) is the same for i and opp(i)
    constexpr int i = 2 * P + 1;
    constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
    float qp = ((cx != 0) ? a_xx : b_xx) + ((cy != 0) ? a_yy : b_yy);
    qp = qp + ((cz != 0) ? a_zz : b_zz);
    if constexpr (cx * cy > 0) qp = qp + pxy2;
    if constexpr (cx * cy < 0) qp = qp - pxy2;
    if constexpr (cx * cz > 0) qp = qp + pxz2;
    if constexpr (cx * cz < 0) qp = qp - pxz2;
    if constexpr (cy * cz > 0) qp = qp + pyz2;
    if constexpr (cy * cz < 0) qp = qp - pyz2;
    const float kq = (i < 7 ? k1 : k2) * qp;
    fo[i] = eq[i] + kq;
    fo[i + 1] = eq[i + 1] + kq;
  });
  o.ux = ux; o.uy = uy; o.uz = uz; o.rho = rho; o.guard = guard;
  return o;
}

template <class St>
__device__ __forceinline__ float ldp(const void* pop, int dir, uint32_t np, uint32_t cell) {
  return St::ld(reinterpret_cast<const typename St::T*>(pop) + (size_t)dir * np + cell, Wd(dir));
}
template <class St>
__device__ __forceinline__ void stp(void* pop, int dir, uint32_t np, uint32_t cell, float v, int wdir) {
  St::st(reinterpret_cast<typename St::T*>(pop) + (size_t)dir * np + cell, v, Wd(wdir));
}

// Regularized + Smagorinsky collision (wgsl.ts:231-272) on scaled deviations
// d_i = S (f_i - w_i), the step's working form for f16 / bf16 storage: the same
// model written out on moments, in FP32 with fused multiply-adds and the
// hardware's approximate reciprocal and square root.  It does not keep the
// reference's operation order (the f32 path's collide() does, bit for bit); its
// accuracy is judged against the FP64 oracle by the precision tests.
//   rho = 1 + dr, dr = sum d / S;  j = sum c d / S;  u = j / rho
//   Pi^neq_ab = sum c_a c_b d / S - rho u_a u_b - dr delta_ab / 3
//     (sum_i w_i c_ia c_ib = delta_ab / 3; the equilibrium's second moment is
//      rho u_a u_b + rho delta_ab / 3)
//   f_i' - w_i = w_i (dr - 1.5 rho u.u + rho (3 c.u + 4.5 (c.u)^2)) + 4.5 (1 - 1/tau) w_i (c_i c_i - I/3):Pi^neq
// Directions pair as (i, opp i) for odd i: sums s and differences m of each pair
// give the moments; pairs 0 x, 1 y, 2 z, 3 (+x+y), 4 (+x-y), 5 (+x+z), 6 (+x-z),
// 7 (+y+z), 8 (+y-z), named by their odd member.
template <class St>
__device__ __forceinline__ CellOut collide_dev(const float (&d)[19], float (&fo)[19], float tau0, float u_in, float ks2,
                                               bool duct, float guard_uu) {
  constexpr float S = St::S, iS = 1.0f / St::S;
  CellOut o;
  float s[9], m[9];
  sfor<9>([&](auto P) {
    constexpr int i = 2 * P + 1;
    s[P] = d[i] + d[i + 1];
    m[P] = d[i] - d[i + 1];
  });
  const float sd = ((d[0] + s[0]) + (s[1] + s[2])) + (((s[3] + s[4]) + (s[5] + s[6])) + (s[7] + s[8]));
  const float jx = ((m[0] + m[3]) + (m[4] + m[5])) + m[6];
  const float jy = ((m[1] + m[3]) - m[4]) + (m[7] + m[8]);
  const float jz = ((m[2] + m[5]) - m[6]) + (m[7] - m[8]);
  float sxx = ((s[0] + s[3]) + (s[4] + s[5])) + s[6];
  float syy = ((s[1] + s[3]) + (s[4] + s[7])) + s[8];
  float szz = ((s[2] + s[5]) + (s[6] + s[7])) + s[8];
  float sxy = s[3] - s[4], sxz = s[5] - s[6], syz = s[7] - s[8];
  float dr = sd * iS;
  float rho = 1.0f + dr;
  float rr = __fdividef(1.0f, rho);
  const float q = rr * iS;
  float ux = jx * q, uy = jy * q, uz = jz * q;
  // divergence guard (wgsl.ts:238-243): non-finite, rho outside [0.3, 3] or |u| > 0.35
  const float uu0 = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
  const bool guard = !(rho >= 0.3f && rho <= 3.0f && uu0 <= guard_uu);
  if (guard) {  // f = feq(1, (u_in/2, 0, 0)): its deviation moments are u_a u_b (scaled)
    rho = 1.0f;
    dr = 0.0f;
    rr = 1.0f;
    ux = u_in * 0.5f;
    uy = 0.0f;
    uz = 0.0f;
    sxx = S * ux * ux;
    syy = szz = sxy = sxz = syz = 0.0f;
  }
  if (duct) {  // wgsl.ts:248
    const float t = 0.04f, tu = 1.0f - 0.04f;
    ux = ux * tu + (0.55f * u_in) * t;
    uy = uy * tu + uy * t;
    uz = uz * tu + uz * t;
  }
  const float uu = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
  const float rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
  const float dr3 = dr * (1.0f / 3.0f);
  const float pxx = fmaf(sxx, iS, -fmaf(rux, ux, dr3));
  const float pyy = fmaf(syy, iS, -fmaf(ruy, uy, dr3));
  const float pzz = fmaf(szz, iS, -fmaf(ruz, uz, dr3));
  const float pxy = fmaf(sxy, iS, -(rux * uy));
  const float pxz = fmaf(sxz, iS, -(rux * uz));
  const float pyz = fmaf(syz, iS, -(ruy * uz));
  const float q2 = fmaf(pxx, pxx, fmaf(pyy, pyy, pzz * pzz)) + 2.0f * fmaf(pxy, pxy, fmaf(pxz, pxz, pyz * pyz));
  const float qn = q2 * rsqrtf(fmaxf(q2, 1e-30f));  // sqrt(q2), 0 for q2 = 0
  const float arg = fmaf(tau0, tau0, ks2 * qn * rr);
  const float tau = 0.5f * (tau0 + arg * rsqrtf(arg));  // arg >= tau0^2 > 0
  const float k = fmaf(-4.5f, __fdividef(1.0f, tau), 4.5f);
  const float tr3 = ((pxx + pyy) + pzz) * (1.0f / 3.0f);
  const float a = fmaf(-1.5f * rho, uu, dr);
  const float r3 = 3.0f * rho, r45 = 4.5f * rho;
  const float qx = pxx - tr3, qy = pyy - tr3, qz = pzz - tr3;
  const float bxy = qx + pyy, bxz = qx + pzz, byz = qy + pzz;
  const float qd[9] = {qx, qy, qz, fmaf(2.0f, pxy, bxy), fmaf(-2.0f, pxy, bxy), fmaf(2.0f, pxz, bxz),
                       fmaf(-2.0f, pxz, bxz), fmaf(2.0f, pyz, byz), fmaf(-2.0f, pyz, byz)};
  fo[0] = (S * Wd(0)) * fmaf(-k, tr3, a);
  sfor<9>([&](auto P) {
    constexpr int i = 2 * P + 1;
    const float cu = cdot<i>(ux, uy, uz);
    const float e = fmaf(r45 * cu, cu, fmaf(k, qd[P], a));
    constexpr float W = S * Wd(i);
    const float ew = W * e;
    const float lin = r3 * cu;
    fo[i] = fmaf(W, lin, ew);
    fo[i + 1] = fmaf(-W, lin, ew);
  });
  o.ux = ux; o.uy = uy; o.uz = uz; o.rho = rho; o.guard = guard;
  return o;
}

// How the step holds a cell's populations in registers: absolute f_i for f32
// storage (with the reference's arithmetic in collide(), bit for bit), scaled
// deviations d_i = S (f_i - w_i) for f16 / bf16 storage (their stored form,
// collided by collide_dev).  Boundary values come in the same form.
// NC: populations are loaded through the read-only (non-coherent) path, valid
// when no block rewrites them during the launch; the persistent batch kernel,
// whose steps rewrite them, loads with NC = false (L2-coherent loads).
template <class St, bool NC = true>
struct Rep {
  typedef typename St::T T;
  static constexpr bool dev = false;
  __device__ __forceinline__ static float ld(const T* p, int dir) {
    if constexpr (NC) return St::ld(p, Wd(dir));
    else return St::ld_coh(p, Wd(dir));
  }
  __device__ __forceinline__ static void st(T* p, float v, int dir) { St::st(p, v, Wd(dir)); }
  __device__ __forceinline__ static float solid(int k) { return Wd(k); }  // wgsl.ts:183
  __device__ __forceinline__ static float feq_in(const StepArgs& a, int i) { return a.feq_in[i]; }
  __device__ __forceinline__ static float floor_k(const StepArgs& a, int i) { return a.floor_k[i]; }
  template <int i> __device__ __forceinline__ static float outlet(float ux, float uy, float uz) {
    return feq_rho1<i>(ux, uy, uz);
  }
  template <int i> __device__ __forceinline__ static float link_t(float v) { return 2.0f * (v - Wd(i)); }
};
template <class St, bool NC = true>
struct RepDev {
  typedef typename St::T T;
  static constexpr bool dev = true;
  __device__ __forceinline__ static float ld(const T* p, int) {
    if constexpr (NC) return St::ldd(p);
    else return St::ldd_coh(p);
  }
  __device__ __forceinline__ static void st(T* p, float v, int) { St::std_(p, v); }
  __device__ __forceinline__ static float solid(int) { return 0.0f; }
  __device__ __forceinline__ static float feq_in(const StepArgs& a, int i) { return a.dev_in[i]; }
  __device__ __forceinline__ static float floor_k(const StepArgs& a, int i) { return a.floor_kd[i]; }
  template <int i> __device__ __forceinline__ static float outlet(float ux, float uy, float uz) {
    return (feq_rho1<i>(ux, uy, uz) - Wd(i)) * St::S;
  }
  template <int i> __device__ __forceinline__ static float link_t(float v) { return v * (2.0f / St::S); }
};
template <bool NC> struct Rep<StoreF16, NC> : RepDev<StoreF16, NC> {};
template <bool NC> struct Rep<StoreBF16, NC> : RepDev<StoreBF16, NC> {};

// A population of direction dir at cell index `cell` in the step's form.
template <class St, bool NC = true>
__device__ __forceinline__ float ldr(const void* pop, int dir, uint32_t np, uint32_t cell) {
  return Rep<St, NC>::ld(reinterpret_cast<const typename St::T*>(pop) + (size_t)dir * np + cell, dir);
}
template <class St>
__device__ __forceinline__ void str(void* pop, int dir, uint32_t np, uint32_t cell, float v, int wdir) {
  Rep<St>::st(reinterpret_cast<typename St::T*>(pop) + (size_t)dir * np + cell, v, wdir);
}

// Momentum exchange of one force-carrying link (wgsl.ts:221-223): the bounced
// value v = f[i]; group from the source cell's solid flag.
template <int i, class R>
__device__ __forceinline__ void link_force(float v, uint32_t group, float (&gf)[9]) {
  const float t = R::template link_t<i>(v);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (group == (uint32_t)(k + 1)) {
      if constexpr (CXd(i) > 0) gf[3 * k] = gf[3 * k] - t;
      if constexpr (CXd(i) < 0) gf[3 * k] = gf[3 * k] + t;
      if constexpr (CYd(i) > 0) gf[3 * k + 1] = gf[3 * k + 1] - t;
      if constexpr (CYd(i) < 0) gf[3 * k + 1] = gf[3 * k + 1] + t;
      if constexpr (CZd(i) > 0) gf[3 * k + 2] = gf[3 * k + 2] - t;
      if constexpr (CZd(i) < 0) gf[3 * k + 2] = gf[3 * k + 2] + t;
    }
  }
}

// ---------------------------------------------------------------------------
// One thread per cell, blocks of 128 cells along x (grid nx/128 x ny x nz).
// All 19 population reads are issued before the collision.  Warps away from
// the lattice faces take a short path: in the gather step each direction reads
// either the neighbour's slot or, for a bounce-back link, the cell's own slot
// (one select, one load); faces take the full boundary precedence.
// (A TMA-staged persistent variant - 19 cp.async.bulk row windows per tile into
// a double-buffered shared-memory stage - was measured slower on this kernel:
// 19.9 vs 26 GLUPS on the 256x96x80 F1, so it is not used.)
// ---------------------------------------------------------------------------
constexpr uint32_t TILE = 128;

// Slot offsets of direction i relative to the cell index (mod 2^32): the
// single-lattice kernel reads the host-computed tables straight from its
// parameter block and takes the plain-neighbour path and the L2 prefetch; the
// batch kernel, whose arguments sit in global memory, computes own-slot
// addresses from np and keeps the two-way (interior / face) gather.  (Staging
// the batch arguments in shared memory to give it the plain path measured 8-10 %
// slower on the 33-lattice aero map; reading 57 table entries from global
// memory instead spills ~400 B per thread.)
struct OfsTable {
  static constexpr bool plain_path = true;
  const StepArgs& a;
  template <int i, class PT> __device__ __forceinline__ PT* own_at(PT* P, uint32_t idx) const {
    return P + (idx + a.own_ofs[i]);
  }
  template <int i> __device__ __forceinline__ uint32_t pull() const { return a.pull_ofs[i]; }
  template <int i> __device__ __forceinline__ uint32_t push() const { return a.push_ofs[i]; }
};
struct OfsCalc {
  static constexpr bool plain_path = false;
  uint32_t np;
  template <int i, class PT> __device__ __forceinline__ PT* own_at(PT* P, uint32_t idx) const {
    return P + (size_t)i * np + idx;
  }
  template <int i> __device__ __forceinline__ uint32_t pull() const { return 0u; }
  template <int i> __device__ __forceinline__ uint32_t push() const { return 0u; }
};

// L2 prefetch of the tile a.prefetch_ahead blocks further on (about one wave of
// resident blocks ahead, in launch order; REV: tiles run in reverse order): thread
// t < 19 * by issues one bulk prefetch of direction t % 19 over row t / 19 of
// that tile, so DRAM streams the next wave's own-cell rows while this wave
// computes.  The byte range is widened to 16-byte boundaries and clipped to the
// population allocation.
template <class T, bool REV>
__device__ __forceinline__ void prefetch_tile(const StepArgs& a, uint3 bid, uint3 gdim) {
  if (a.prefetch_ahead == 0) return;
  const uint32_t nb = gdim.x * gdim.y * gdim.z;
  const uint32_t lin = bid.x + gdim.x * (bid.y + gdim.y * bid.z);
  if (REV && lin < a.prefetch_ahead) return;
  const uint32_t tb = REV ? lin - a.prefetch_ahead : lin + a.prefetch_ahead;
  const uint32_t t = threadIdx.x + blockDim.x * threadIdx.y;
  if (tb >= nb || t >= 19u * blockDim.y) return;
  const uint32_t dir = t % 19u, row = t / 19u;
  const uint32_t tx = tb % gdim.x, ty = (tb / gdim.x) % gdim.y, tz = tb / (gdim.x * gdim.y);
  const uint32_t y = ty * blockDim.y + row, x0 = tx * blockDim.x;
  if (y >= a.ny || x0 >= a.nx) return;
  const uint32_t cells = min(blockDim.x, a.nx - x0);
  const uint64_t e0 = (uint64_t)dir * a.np + x0 + (uint64_t)a.nx * (y + (uint64_t)a.ny * tz);
  const uint64_t b0 = (e0 * sizeof(T)) & ~15ull;
  uint64_t b1 = ((e0 + cells) * sizeof(T) + 15ull) & ~15ull;
  if (b1 > a.pop_bytes) b1 = a.pop_bytes & ~15ull;
  if (b1 <= b0) return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<const char*>(a.pop) + b0),
               "r"((uint32_t)(b1 - b0))
               : "memory");
}

// One block's cells of one lattice.  bid/gdim are the block coordinates and grid
// of that lattice's tiling; slots is where this step's force records go.
// LOOP: the block goes on to another tile after this one (persistent batch
// kernel), so the shared force arrays are released with a barrier at the end.
template <class St, bool GATHER, bool FIELDS, class Ofs, bool REV = false, bool LOOP = false>
__device__ __forceinline__ void step_tile(const StepArgs& a, const Ofs& ofs, ForceSlot* slots, uint3 bid, uint3 gdim) {
  const uint8_t* __restrict__ solid_u8 = a.solid;
  const uint32_t nx = a.nx, ny = a.ny, nz = a.nz;
  const uint32_t x = bid.x * blockDim.x + threadIdx.x;
  const uint32_t y = bid.y * blockDim.y + threadIdx.y;
  const uint32_t z = bid.z;
  const bool in = (x < nx) && (y < ny);
  const uint32_t nxy = nx * ny;
  const uint32_t np = (uint32_t)a.np;
  if constexpr (Ofs::plain_path) prefetch_tile<typename St::T, REV>(a, bid, gdim);
  const uint32_t idx = in ? x + nx * y + nxy * z : 0u;
  const uint32_t cw = in ? __ldg(a.cellw + idx) : CW_SOLID;
  typedef typename St::T PT;
  typedef Rep<St, !LOOP> R;
  PT* __restrict__ P = reinterpret_cast<PT*>(a.pop);
  float gf[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float rho_cell = 0.0f;
  bool guard = false;
  // A warp is 32 consecutive x of one (y, z) row (block widths are multiples of
  // 32), so the y/z faces are warp-uniform: those rows take the full boundary
  // path.  The x faces (inlet x = 0, outlet x = nx - 1) stay in the interior
  // paths: their out-of-domain directions still load an in-bounds slot (the
  // row wraps into the previous / next row of the same direction array), the
  // value is then replaced by the inlet / outlet population, and their
  // discarded pushes land in slots the next step never reads (the outlet and
  // inlet directions of x = nx - 1 and x = 0 cells).  No warp diverges on them.
  const bool yzface = (y == 0) | (y == ny - 1) | (z == 0) | (z == nz - 1);
  // Warp-uniform plain test (all lanes converged here): no fluid lane of this
  // warp has a bounce-back link, so every population moves between plain
  // neighbour slots.
  const bool plain = Ofs::plain_path &&
      __all_sync(0xffffffffu, !in || (cw & CW_SOLID) || (!yzface && (cw & CW_LINKS) == 0u));

  if (in && (cw & CW_SOLID)) {
    if constexpr (!GATHER) {  // wgsl.ts:183: solid cells hold w_i
      if constexpr (Ofs::plain_path) sfor<19>([&](auto K) { R::st(ofs.template own_at<K>(P, idx), R::solid(K), K); });
      else sfor<19>([&](auto K) { str<St>(a.pop, K, np, idx, R::solid(K), K); });
    }
    if constexpr (FIELDS) a.fields[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
  } else if (in) {
    float f[19], fo[19];
    float4 pu = make_float4(0.f, 0.f, 0.f, 0.f);
    if (x == nx - 1) pu = a.outlet_u[y + ny * z];
    const float floor_u = (cw & CW_BELT) ? 0.0f : a.u_in;

    // ---------------------------------------------------------------- gather
    if (plain) {
      sfor<19>([&](auto I) {
        constexpr int i = I;
        if constexpr (GATHER) f[i] = R::ld(P + (idx + ofs.template pull<i>()), i);
        else f[i] = R::ld(ofs.template own_at<i>(P, idx), i);
      });
    } else if (!yzface) {
      sfor<19>([&](auto I) {
        constexpr int i = I;
        if constexpr (i == 0) {
          f[0] = ldr<St, !LOOP>(a.pop, 0, np, idx);
        } else if constexpr (GATHER) {
          constexpr int off_x = CXd(i), off_y = CYd(i), off_z = CZd(i);
          const int off = off_x + off_y * (int)nx + off_z * (int)nxy;
          const bool bb = (cw >> i) & 1u;
          const uint32_t slot = bb ? (uint32_t)i * np + idx : (uint32_t)OPPd(i) * np + (uint32_t)((int)idx - off);
          const int wdir = bb ? i : OPPd(i);
          f[i] = R::ld(reinterpret_cast<const typename St::T*>(a.pop) + slot, wdir);
        } else {
          f[i] = ldr<St, !LOOP>(a.pop, i, np, idx);
        }
      });
    } else {
      sfor<19>([&](auto I) {
        constexpr int i = I;
        constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
        if constexpr (i == 0) {
          f[0] = ldr<St, !LOOP>(a.pop, 0, np, idx);
        } else {
          float v;
          if (cx > 0 && x == 0) {
            v = R::feq_in(a, i);
          } else if (cx < 0 && x == nx - 1) {
            v = R::template outlet<i>(pu.x, pu.y, pu.z);
          } else if (cy > 0 && y == 0) {
            v = ldr<St, !LOOP>(a.pop, i, np, idx);
            if constexpr (cx != 0) v = v + R::floor_k(a, i) * floor_u;
          } else if ((cy < 0 && y == ny - 1) || (cz < 0 && z == nz - 1)) {
            v = R::feq_in(a, i);
          } else if (GATHER) {
            if ((cw >> i) & 1u) {
              v = ldr<St, !LOOP>(a.pop, i, np, idx);
            } else if (cz > 0 && z == 0) {
              v = ldr<St, !LOOP>(a.pop, OPPd(ZMIRd(i)), np, (uint32_t)((int)idx - cx - cy * (int)nx));
            } else {
              const int off = cx + cy * (int)nx + cz * (int)nxy;
              v = ldr<St, !LOOP>(a.pop, OPPd(i), np, (uint32_t)((int)idx - off));
            }
          } else {
            v = ldr<St, !LOOP>(a.pop, i, np, idx);
          }
          f[i] = v;
        }
      });
    }
    if (!yzface) {  // inlet / outlet directions of the x-face lanes (wgsl.ts:207-210)
      if (x == 0) {
        sfor<19>([&](auto I) {
          if constexpr (CXd(I) > 0) f[I] = R::feq_in(a, I);
        });
      }
      if ((x | 31u) >= nx - 1) {  // warp-uniform: this warp holds the outlet column
        sfor<19>([&](auto I) {
          constexpr int i = I;
          if constexpr (CXd(i) < 0) {
            const float e = R::template outlet<i>(pu.x, pu.y, pu.z);
            f[i] = (x == nx - 1) ? e : f[i];
          }
        });
      }
    }

    // ---------------------------------------------------------------- forces
    if (cw & CW_FORCE) {
      sfor<19>([&](auto I) {
        constexpr int i = I;
        if constexpr (i != 0) {
          constexpr int cx = CXd(i), cy = CYd(i), cz = CZd(i);
          const bool mirrored = (cz > 0) && (z == 0);
          if (((cw >> i) & 1u) && !mirrored) {
            const int off = cx + cy * (int)nx + cz * (int)nxy;
            const uint32_t grp = __ldg(solid_u8 + (uint32_t)((int)idx - off));
            link_force<i, R>(f[i], grp, gf);
          }
        }
      });
    }

    // ---------------------------------------------------------------- collide
    CellOut o;
    if constexpr (R::dev)
      o = collide_dev<St>(f, fo, __ldg(a.tau0_x + x), a.u_in, a.ks2, (cw & CW_DUCT) != 0, a.guard_uu);
    else
      o = collide(f, fo, __ldg(a.tau0_x + x), a.u_in, a.ks2, (cw & CW_DUCT) != 0, a.feq_guard, a.guard_uu);
    if (o.guard) {
#pragma unroll
      for (int k = 0; k < 9; k++) gf[k] = 0.0f;
    }
    guard = o.guard;
    rho_cell = o.rho;
    if (x == nx - 1) a.outlet_u[y + ny * z] = make_float4(o.ux, o.uy, o.uz, 0.0f);
    if constexpr (FIELDS) a.fields[idx] = make_float4(o.ux, o.uy, o.uz, o.rho);

    // ---------------------------------------------------------------- scatter
    if constexpr (!GATHER) {
      sfor<19>([&](auto J) {
        constexpr int j = J;
        if constexpr (Ofs::plain_path) R::st(ofs.template own_at<OPPd(j)>(P, idx), fo[j], j);
        else str<St>(a.pop, OPPd(j), np, idx, fo[j], j);
      });
    } else if (plain) {
      sfor<19>([&](auto J) {
        constexpr int j = J;
        R::st(P + (idx + ofs.template push<j>()), fo[j], j);
      });
    } else if (!yzface) {
      sfor<19>([&](auto J) {
        constexpr int j = J;
        if constexpr (j == 0) {
          str<St>(a.pop, 0, np, idx, fo[0], 0);
        } else {
          constexpr int i = OPPd(j);
          const int off = CXd(j) + CYd(j) * (int)nx + CZd(j) * (int)nxy;
          const bool bb = (cw >> i) & 1u;
          const uint32_t slot = bb ? (uint32_t)i * np + idx : (uint32_t)j * np + (uint32_t)((int)idx + off);
          R::st(reinterpret_cast<typename St::T*>(a.pop) + slot, fo[j], j);
        }
      });
    } else {
      sfor<19>([&](auto J) {
        constexpr int j = J;
        constexpr int cx = CXd(j), cy = CYd(j), cz = CZd(j);
        constexpr int i = OPPd(j);
        if constexpr (j == 0) {
          str<St>(a.pop, 0, np, idx, fo[0], 0);
        } else {
          if (cx < 0 && x == 0) {
            // inlet side: the reference never reads this value
          } else if (cx > 0 && x == nx - 1) {
            // outlet side: discarded
          } else if (cy < 0 && y == 0) {
            str<St>(a.pop, i, np, idx, fo[j], j);  // moving-floor bounce-back source
          } else if ((cy > 0 && y == ny - 1) || (cz > 0 && z == nz - 1)) {
            // far field: discarded
          } else if ((cw >> i) & 1u) {
            str<St>(a.pop, i, np, idx, fo[j], j);  // bounce-back source (mirror included)
          } else if (cz < 0 && z == 0) {
            str<St>(a.pop, ZMIRd(j), np, (uint32_t)((int)idx + cx + cy * (int)nx), fo[j], j);
          } else {
            const int off = cx + cy * (int)nx + cz * (int)nxy;
            str<St>(a.pop, j, np, (uint32_t)((int)idx + off), fo[j], j);
          }
        }
      });
    }
  }

  // -------------------------------------------------------------- reductions
  const uint32_t lane = threadIdx.x & 31u, warp = (threadIdx.x + blockDim.x * threadIdx.y) >> 5;
  const uint32_t nwarps = (blockDim.x * blockDim.y + 31) >> 5;
  const uint32_t blk = bid.x + gdim.x * (bid.y + gdim.y * bid.z);
  const unsigned gb = __ballot_sync(0xffffffffu, guard);
  if (gb && lane == 0) atomicAdd(a.guard_count, (unsigned)__popc(gb));
  if constexpr (FIELDS) {  // per-warp FP64 mass partial, reduced in a fixed order later
    double m = (in && !(cw & CW_SOLID)) ? (double)rho_cell : 0.0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) m += __shfl_down_sync(0xffffffffu, m, s);
    if (lane == 0) a.mass_partial[(size_t)blk * nwarps + warp] = m;
  }
  const int32_t slot = __ldg(a.block_slot + blk);
  if (slot < 0) return;  // no force-carrying link in this block: no barrier, no record
  __shared__ double s_f[9][8];
  __shared__ int32_t s_r[6][8];
  bool any_force = false;
#pragma unroll
  for (int q = 0; q < 9; q++) any_force |= (gf[q] != 0.0f);
  if (!__any_sync(0xffffffffu, any_force)) {  // no force in this warp: zero record, no FP64 shuffles
    if (lane < 9) s_f[lane][warp] = 0.0;
    if (lane < 6) s_r[lane][warp] = 0;
  } else {
    double d[9];
    int32_t r[6];
#pragma unroll
    for (int q = 0; q < 9; q++) d[q] = (double)gf[q];
#pragma unroll
    for (int g = 0; g < 3; g++) {
      r[2 * g] = (gf[3 * g] != 0.0f) ? __float2int_rn(gf[3 * g] * 10000.0f) : 0;
      r[2 * g + 1] = (gf[3 * g + 1] != 0.0f) ? __float2int_rn(gf[3 * g + 1] * 10000.0f) : 0;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
#pragma unroll
      for (int q = 0; q < 9; q++) d[q] += __shfl_down_sync(0xffffffffu, d[q], s);
#pragma unroll
      for (int q = 0; q < 6; q++) r[q] = (int32_t)((uint32_t)r[q] + (uint32_t)__shfl_down_sync(0xffffffffu, r[q], s));
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < 9; q++) s_f[q][warp] = d[q];
#pragma unroll
      for (int q = 0; q < 6; q++) s_r[q][warp] = r[q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    ForceSlot& out = slots[slot];
    for (int q = 0; q < 9; q++) {
      double tt = 0.0;
      for (uint32_t w = 0; w < nwarps; w++) tt += s_f[q][w];
      out.f[q] = tt;
    }
    for (int q = 0; q < 6; q++) {
      uint32_t tt = 0;
      for (uint32_t w = 0; w < nwarps; w++) tt += (uint32_t)s_r[q][w];
      out.raw[q] = (int32_t)tt;
    }
  }
  if constexpr (LOOP) __syncthreads();  // thread 0 has read s_f / s_r before the next tile writes them
}

// Consecutive collide-stream launches are chained by programmatic dependent
// launch: each grid lets the next one be scheduled as soon as all of its own
// blocks are resident (launch_dependents), and every grid waits for its
// predecessor to complete and flush (wait) before it touches memory, so the next
// step's blocks are already on the SMs when the previous step retires.
__device__ __forceinline__ void chain_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <class K, class... Args>
cudaError_t launch_chained(K kernel, dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <class St, bool GATHER, bool FIELDS>
__global__ void __maxnreg__(St::max_regs) step_kernel(StepArgs a) {
  chain_enter();
  // FP32 local steps take the tiles in reverse launch order: their first tiles
  // are the ones the preceding gather step ran last, whose lines are still in
  // the L2 (the FP32 lattice at 256x96x80, 157 MB of populations, is larger than
  // the L2): +2.7 % there, neutral at 512x192x160.  For f16/bf16 it measured 9 %
  // slower at 256x96x80 (whose populations fit the L2) and neutral at
  // 512x192x160, so they keep the launch order.  Force and mass records are
  // keyed by tile coordinates, not by launch order, so the results do not change.
  const uint3 gdim = make_uint3(gridDim.x, gridDim.y, gridDim.z);
  if constexpr (GATHER || St::id != WT_STORE_F32) {
    step_tile<St, GATHER, FIELDS, OfsTable, false>(a, OfsTable{a}, a.slots, blockIdx, gdim);
  } else {
    const uint3 bid = make_uint3(gdim.x - 1 - blockIdx.x, gdim.y - 1 - blockIdx.y, gdim.z - 1 - blockIdx.z);
    step_tile<St, GATHER, FIELDS, OfsTable, true>(a, OfsTable{a}, a.slots, bid, gdim);
  }
}

// Many lattices in one launch: block b belongs to the lattice L with
// tile_base[L] <= b < tile_base[L+1]; its coordinates follow that lattice's grid.
template <class St, bool GATHER, bool FIELDS>
__global__ void __maxnreg__(St::max_regs) batch_step_kernel(const StepArgs* __restrict__ args,
                                                            const BatchTiles* __restrict__ tiles, uint32_t count,
                                                            uint32_t pending) {
  chain_enter();
  const uint32_t b = blockIdx.x;
  uint32_t lo = 0, hi = count;  // binary search: largest L with base[L] <= b
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&tiles[mid].base) <= b) lo = mid;
    else hi = mid;
  }
  const BatchTiles tl = tiles[lo];
  const uint32_t t = b - tl.base;
  const uint3 gdim = make_uint3(tl.gx, tl.gy, tl.gz);
  const uint3 bid = make_uint3(t % tl.gx, (t / tl.gx) % tl.gy, t / (tl.gx * tl.gy));
  const StepArgs& a = args[lo];
  const OfsCalc ofs{(uint32_t)a.np};
  step_tile<St, GATHER, FIELDS>(a, ofs, a.slots + (size_t)pending * a.nslots, bid, gdim);
}

// Persistent batch: ONE cooperative launch advances every lattice of the batch
// by nsteps LBM steps (at most the pending force-record capacity).  Each step
// walks all tiles of all lattices grid-stride in launch order, with the
// per-tile arithmetic and records of batch_step_kernel, so the results are the
// same bits; a grid barrier separates the steps.  The barrier's wait is bounded:
// on expiry the block raises sync[1] and leaves the kernel (the host reports
// the flag), so a failure ends the launch instead of hanging it.  The launch is
// cooperative, so all blocks are resident and every barrier can be met.
constexpr uint32_t BARRIER_POLLS = 1u << 22;  // x ~100 ns: ~0.4 s against ~2 ms steps

__device__ __forceinline__ uint32_t ld_acquire_u32(const unsigned int* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned int* sync, uint32_t target) {
  __shared__ uint32_t s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    atomicAdd(sync, 1u);
    uint32_t ok = 0;
    for (uint32_t i = 0; i < BARRIER_POLLS; i++) {
      if (ld_acquire_u32(sync) >= target) {
        ok = 1;
        break;
      }
      __nanosleep(100);
    }
    if (!ok) atomicExch(sync + 1, 1u);
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// (FP32: 8 registers above the step kernel's cap, 112 B of spills instead of 296)
template <class St>
__global__ void __maxnreg__(St::max_regs + (St::id == WT_STORE_F32 ? 8 : 0))
    batch_persist_kernel(const StepArgs* __restrict__ args, const BatchTiles* __restrict__ tiles, uint32_t count,
                         uint32_t total, uint32_t k0, uint32_t nsteps, uint32_t pending0, uint32_t fields_last,
                         unsigned int* sync) {
  for (uint32_t k = 0; k < nsteps; k++) {
    const bool gather = ((k0 + k) & 1u) == 0u;
    const bool fields = fields_last && k + 1 == nsteps;
    for (uint32_t b = blockIdx.x; b < total; b += gridDim.x) {
      uint32_t lo = 0, hi = count;  // largest L with base[L] <= b
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&tiles[mid].base) <= b) lo = mid;
        else hi = mid;
      }
      const BatchTiles tl = tiles[lo];
      const uint32_t t = b - tl.base;
      const uint3 gdim = make_uint3(tl.gx, tl.gy, tl.gz);
      const uint3 bid = make_uint3(t % tl.gx, (t / tl.gx) % tl.gy, t / (tl.gx * tl.gy));
      const StepArgs& a = args[lo];
      const OfsCalc ofs{(uint32_t)a.np};
      ForceSlot* slots = a.slots + (size_t)(pending0 + k) * a.nslots;
      if (gather) step_tile<St, true, false, OfsCalc, false, true>(a, ofs, slots, bid, gdim);
      else if (fields) step_tile<St, false, true, OfsCalc, false, true>(a, ofs, slots, bid, gdim);
      else step_tile<St, false, false, OfsCalc, false, true>(a, ofs, slots, bid, gdim);
    }
    if (k + 1 < nsteps && !grid_barrier(sync, (k + 1) * gridDim.x)) return;
  }
}

// Canonical initial state (LBM_INIT, wgsl.ts:147-155): f*_j = feq_j(1, (u_in,0,0))
// stored at pop[opp(j)][x] for every cell, fields (u_in,0,0,1).
struct Feq19 {
  float v[19];
};

template <class St>
__global__ void init_kernel(void* pop, float4* fields, float4* outlet_u, uint32_t n, uint32_t ny, uint32_t nz,
                            uint32_t np, float u_in, Feq19 feq_in) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) {
    sfor<19>([&](auto J) { stp<St>(pop, OPPd(J), np, idx, feq_in.v[J], J); });
    fields[idx] = make_float4(u_in, 0.0f, 0.0f, 1.0f);
  }
  if (idx < ny * nz) outlet_u[idx] = make_float4(u_in, 0.0f, 0.0f, 0.0f);
}

template <class St>
__global__ void read_pop_kernel(const void* pop, float* out, uint32_t n, uint32_t np) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  sfor<19>([&](auto J) { out[(size_t)J * n + idx] = ldp<St>(pop, OPPd(J), np, idx) ; });
}

template <class St>
__global__ void write_pop_kernel(const float* in, void* pop, uint32_t n, uint32_t np) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  sfor<19>([&](auto J) { stp<St>(pop, OPPd(J), np, idx, in[(size_t)J * n + idx], J); });
}

// Warm start: trilinear resample of a coarse (ux,uy,uz,rho) field onto the
// lattice, populations set to feq(rho, u).
template <class St>
__global__ void resample_kernel(const float4* coarse, uint32_t cx, uint32_t cy, uint32_t cz, void* pop,
                                float4* fields, float4* outlet_u, uint32_t nx, uint32_t ny, uint32_t nz,
                                uint32_t np) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nx * ny * nz) return;
  const uint32_t x = idx % nx, y = (idx / nx) % ny, z = idx / (nx * ny);
  const float gx = ((float)x + 0.5f) * (float)cx / (float)nx - 0.5f;
  const float gy = ((float)y + 0.5f) * (float)cy / (float)ny - 0.5f;
  const float gz = ((float)z + 0.5f) * (float)cz / (float)nz - 0.5f;
  const float fx = fminf(fmaxf(gx, 0.0f), (float)(cx - 1)), fy = fminf(fmaxf(gy, 0.0f), (float)(cy - 1)),
              fz = fminf(fmaxf(gz, 0.0f), (float)(cz - 1));
  const uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy, z0 = (uint32_t)fz;
  const uint32_t x1 = min(x0 + 1, cx - 1), y1 = min(y0 + 1, cy - 1), z1 = min(z0 + 1, cz - 1);
  const float tx = fx - (float)x0, ty = fy - (float)y0, tz = fz - (float)z0;
  auto at = [&](uint32_t a, uint32_t b, uint32_t c) { return coarse[a + cx * (b + cy * c)]; };
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  const uint32_t xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
    const float w = (ox ? tx : 1.f - tx) * (oy ? ty : 1.f - ty) * (oz ? tz : 1.f - tz);
    const float4 v = at(xs[ox], ys[oy], zs[oz]);
    acc.x += w * v.x; acc.y += w * v.y; acc.z += w * v.z; acc.w += w * v.w;
  }
  const float rho = acc.w > 0.3f ? acc.w : 1.0f;
  const float uu = acc.x * acc.x + acc.y * acc.y + acc.z * acc.z;
  sfor<19>([&](auto J) {
    constexpr int j = J;
    const float cu = cdot<j>(acc.x, acc.y, acc.z);
    const float e = Wd(j) * rho * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
    stp<St>(pop, OPPd(j), np, idx, e, j);
  });
  fields[idx] = make_float4(acc.x, acc.y, acc.z, rho);
  if (x == nx - 1) outlet_u[y + ny * z] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}

// Coarse box average of the fluid cells (the inverse direction of resample_kernel).
__global__ void coarse_average_kernel(const float4* __restrict__ fields, const uint32_t* __restrict__ cellw,
                                      uint32_t nx, uint32_t ny, uint32_t nz, float4* __restrict__ coarse, uint32_t cx,
                                      uint32_t cy, uint32_t cz) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cx * cy * cz) return;
  const uint32_t a = i % cx, b = (i / cx) % cy, c = i / (cx * cy);
  const uint32_t x0 = (uint32_t)((uint64_t)a * nx / cx), x1 = (uint32_t)((uint64_t)(a + 1) * nx / cx);
  const uint32_t y0 = (uint32_t)((uint64_t)b * ny / cy), y1 = (uint32_t)((uint64_t)(b + 1) * ny / cy);
  const uint32_t z0 = (uint32_t)((uint64_t)c * nz / cz), z1 = (uint32_t)((uint64_t)(c + 1) * nz / cz);
  double sx = 0.0, sy = 0.0, sz = 0.0, sr = 0.0;
  uint32_t cnt = 0;
  for (uint32_t z = z0; z < z1; z++)
    for (uint32_t y = y0; y < y1; y++)
      for (uint32_t x = x0; x < x1; x++) {
        const uint32_t idx = x + nx * (y + ny * z);
        if (cellw[idx] & CW_SOLID) continue;
        const float4 f = fields[idx];
        sx += f.x; sy += f.y; sz += f.z; sr += f.w;
        cnt++;
      }
  coarse[i] = cnt ? make_float4((float)(sx / cnt), (float)(sy / cnt), (float)(sz / cnt), (float)(sr / cnt))
                  : make_float4(0.0f, 0.0f, 0.0f, 1.0f);
}

// Deterministic reduction of the pending steps' partial records: block s < nsteps
// sums step s's records (each thread a fixed strided subset with all 15
// components in registers, then a fixed shuffle tree and the warps in order)
// into the history ring; block nsteps sums the mass partials; the last block to
// finish folds the steps into the running totals in step order.
constexpr uint32_t RED_THREADS = 256;
constexpr uint32_t RED_FCHUNKS = WT_RED_FCHUNKS, RED_MCHUNKS = WT_RED_MCHUNKS;

__device__ __forceinline__ double block_sum_d(double v, double* sm) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (uint32_t w = 0; w < RED_THREADS / 32; w++) t += sm[w];
  __syncthreads();
  return t;
}

// Pending steps' per-block force records into per-step history records and the
// totals, and the per-warp mass partials into the mass.  Each step's records
// are split into RED_FCHUNKS fixed ranges and the mass partials into
// RED_MCHUNKS, one block each; the last block to finish combines the chunk sums
// in chunk order.  The order of every sum is fixed, so the result is the same
// on every run.
__global__ void __launch_bounds__(RED_THREADS) force_reduce_kernel(const ReduceArgs* __restrict__ all, uint32_t nsteps,
                                                                   uint32_t with_mass) {
  // chained like the step kernels: the next launch may be scheduled now; wait
  // for the steps whose records this reads
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ double sm[RED_THREADS / 32];
  __shared__ double smf[9][RED_THREADS / 32];
  __shared__ uint32_t smr[6][RED_THREADS / 32];
  __shared__ bool last;
  const ReduceArgs& ra = all[blockIdx.y];
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const uint64_t hist_base = *ra.hist_pos;
  const uint32_t nforce = nsteps * RED_FCHUNKS;
  double* const mpart = ra.part + (size_t)WT_PENDING_MAX * RED_FCHUNKS * 16;
  if (blockIdx.x < nforce) {
    const uint32_t step = blockIdx.x / RED_FCHUNKS, chunk = blockIdx.x % RED_FCHUNKS;
    const uint32_t per = (ra.nslots + RED_FCHUNKS - 1) / RED_FCHUNKS;
    const uint32_t s0 = chunk * per, s1 = min(s0 + per, ra.nslots);
    const ForceSlot* base = ra.slots + (size_t)step * ra.nslots;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t racc[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t s = s0 + t; s < s1; s += RED_THREADS) {
      const ForceSlot r = base[s];
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] += r.f[k];
#pragma unroll
      for (int k = 0; k < 6; k++) racc[k] += (uint32_t)r.raw[k];
    }
    double* out = ra.part + (size_t)blockIdx.x * 16;
    // the nine FP64 sums and six integer sums together: warp trees (as
    // block_sum_d forms them), one barrier, then the warps in order
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
#pragma unroll
      for (int k = 0; k < 9; k++) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], s);
#pragma unroll
      for (int k = 0; k < 6; k++) racc[k] += __shfl_down_sync(0xffffffffu, racc[k], s);
    }
    if (lane == 0) {
      for (int k = 0; k < 9; k++) smf[k][warp] = acc[k];
      for (int k = 0; k < 6; k++) smr[k][warp] = racc[k];
    }
    __syncthreads();
    if (t < 9) {
      double v = 0.0;
      for (uint32_t w = 0; w < RED_THREADS / 32; w++) v += smf[t][w];
      out[t] = v;
    } else if (t < 15) {
      uint32_t v = 0;
      for (uint32_t w = 0; w < RED_THREADS / 32; w++) v += smr[t - 9][w];
      out[t] = (double)v;  // exact: below 2^32
    }
  } else if (with_mass) {
    const uint32_t chunk = blockIdx.x - nforce;
    const uint32_t per = (ra.nmass + RED_MCHUNKS - 1) / RED_MCHUNKS;
    const uint32_t s0 = chunk * per, s1 = min(s0 + per, ra.nmass);
    double acc = 0.0;
    for (uint32_t s = s0 + t; s < s1; s += RED_THREADS) acc += ra.mass_partial[s];
    const double v = block_sum_d(acc, sm);
    if (t == 0) mpart[chunk] = v;
  }
  __threadfence();
  if (t == 0) last = (atomicAdd(ra.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (uint32_t i = t; i < nsteps * 16; i += RED_THREADS) {  // per-step records, chunks in order
    const uint32_t step = i / 16, k = i % 16;
    if (k >= 15) continue;
    const double* in = ra.part + (size_t)step * RED_FCHUNKS * 16 + k;
    double* rec = ra.hist + ((hist_base + step) % ra.hist_cap) * 16;
    if (k < 9) {
      double v = 0.0;
      for (uint32_t c = 0; c < RED_FCHUNKS; c++) v += in[(size_t)c * 16];
      rec[k] = v;
    } else {
      uint32_t v = 0;
      for (uint32_t c = 0; c < RED_FCHUNKS; c++) v += (uint32_t)in[(size_t)c * 16];
      rec[k] = (double)(int32_t)v;
    }
  }
  if (with_mass && t == 0) {
    double v = 0.0;
    for (uint32_t c = 0; c < RED_MCHUNKS; c++) v += mpart[c];
    *ra.mass_out = v;
  }
  __syncthreads();
  // the totals: one thread per component, the steps in order
  if (t < 9) {
    double v = ra.totals[t];
    for (uint32_t s = 0; s < nsteps; s++) v += ra.hist[((hist_base + s) % ra.hist_cap) * 16 + t];
    ra.totals[t] = v;
  } else if (t < 15) {
    const uint32_t g = (t - 9) / 2, comp = (t - 9) % 2;  // raw x / y of group g
    uint32_t v = (uint32_t)ra.raw_totals[3 * g + comp];
    for (uint32_t s = 0; s < nsteps; s++)
      v += (uint32_t)(int32_t)ra.hist[((hist_base + s) % ra.hist_cap) * 16 + 9 + 2 * g + comp];
    ra.raw_totals[3 * g + comp] = (int32_t)v;
  }
  if (t == 0) {
    *ra.hist_pos = hist_base + nsteps;
    *ra.counter = 0u;
  }
}

template <class St>
cudaError_t launch_step_t(bool gather, bool fields, const StepGeom& g, const StepArgs& a, cudaStream_t s) {
  if (gather) {
    if (fields) return launch_chained(step_kernel<St, true, true>, g.grid, g.block, s, a);
    return launch_chained(step_kernel<St, true, false>, g.grid, g.block, s, a);
  }
  if (fields) return launch_chained(step_kernel<St, false, true>, g.grid, g.block, s, a);
  return launch_chained(step_kernel<St, false, false>, g.grid, g.block, s, a);
}

template <class St>
cudaError_t launch_batch_t(bool gather, bool fields, dim3 block, uint32_t total_blocks, const StepArgs* args,
                           const BatchTiles* tiles, uint32_t count, uint32_t pending, cudaStream_t s) {
  const dim3 grid(total_blocks);
  if (gather) {
    if (fields) return launch_chained(batch_step_kernel<St, true, true>, grid, block, s, args, tiles, count, pending);
    return launch_chained(batch_step_kernel<St, true, false>, grid, block, s, args, tiles, count, pending);
  }
  if (fields) return launch_chained(batch_step_kernel<St, false, true>, grid, block, s, args, tiles, count, pending);
  return launch_chained(batch_step_kernel<St, false, false>, grid, block, s, args, tiles, count, pending);
}

template <class St>
cudaError_t launch_batch_persist_t(dim3 block, uint32_t grid, uint32_t total, const StepArgs* args,
                                   const BatchTiles* tiles, uint32_t count, uint32_t k0, uint32_t nsteps,
                                   uint32_t pending0, bool fields_last, unsigned int* sync, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, batch_persist_kernel<St>, args, tiles, count, total, k0, nsteps, pending0,
                            fields_last ? 1u : 0u, sync);
}

// Host copy of feq(i, 1, (u, 0, 0)) with the reference's operation order
// (wgsl.ts:135-138); host float arithmetic without contraction gives the same
// bits as the device.
Feq19 feq_inlet(float u) {
  Feq19 r;
  for (int i = 0; i < 19; i++) {
    const float cu = (float)CXd(i) * u + (float)CYd(i) * 0.0f + (float)CZd(i) * 0.0f;
    const float uu = u * u + 0.0f * 0.0f + 0.0f * 0.0f;
    r.v[i] = Wd(i) * 1.0f * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
  }
  return r;
}

template <class F>
cudaError_t by_storage(uint32_t storage, F&& f) {
  switch (storage) {
    case WT_STORE_F32: return f(StoreF32());
    case WT_STORE_F16: return f(StoreF16());
    case WT_STORE_BF16: return f(StoreBF16());
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// Prefetch distance of the collide-stream kernel: one wave of resident blocks for
// f32 storage whose populations exceed twice the L2; 0 (off) otherwise.  f16/bf16
// measured slower with it (34.3 -> 30.4 GLUPS on the 256x96x80 F1); f32 gained at
// 512x192x160 (77.5 -> 79.8 % of the HBM roofline, 1.2 GB of populations) but at
// 256x96x80 (150 MB, with the alternating sweep order reusing the L2) it evicts
// lines the next step reads: kernel 32.8 GLUPS with it, 35.0 without.
uint32_t step_resident_blocks(uint32_t storage, const StepGeom& g, uint32_t sm_count, uint64_t pop_bytes,
                              uint64_t l2_bytes) {
  if (storage != WT_STORE_F32 || pop_bytes <= 2 * l2_bytes) return 0;
  int per_sm = 0;
  const int threads = (int)(g.block.x * g.block.y);
  cudaError_t e = by_storage(storage, [&](auto st) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_kernel<decltype(st), true, false>, threads, 0);
  });
  if (e != cudaSuccess || per_sm <= 0) return 0;
  return (uint32_t)per_sm * sm_count;
}

void fill_slot_offsets(StepArgs& a) {
  const uint32_t np = (uint32_t)a.np, nx = a.nx, nxy = a.nx * a.ny;
  for (int i = 0; i < 19; i++) {
    const uint32_t off = (uint32_t)CXd(i) + (uint32_t)CYd(i) * nx + (uint32_t)CZd(i) * nxy;  // mod 2^32
    a.own_ofs[i] = (uint32_t)i * np;
    a.pull_ofs[i] = (uint32_t)OPPd(i) * np - off;
    a.push_ofs[i] = (uint32_t)i * np + off;
  }
}

// Block shape (bx cells along x) x (by rows along y); bx a multiple of 32 and
// bx * by <= 256 (the kernels' launch bounds).  The autotuner picks the shape.
StepGeom step_geometry(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t bx, uint32_t by) {
  if (bx == 0 || bx % 32 != 0 || bx > 256) bx = TILE;
  if (by == 0 || bx * by > 256) by = 1;
  StepGeom g;
  g.block = dim3(bx, by, 1);
  g.grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
  g.nblocks = g.grid.x * g.grid.y * g.grid.z;
  return g;
}


cudaError_t launch_init(uint32_t storage, void* pop, float4* fields, float4* outlet_u, uint32_t nx, uint32_t ny,
                        uint32_t nz, uint64_t np, float u_in, cudaStream_t s) {
  const uint32_t n = nx * ny * nz;
  const uint32_t cover = n > ny * nz ? n : ny * nz;
  const Feq19 fe = feq_inlet(u_in);
  return by_storage(storage, [&](auto st) {
    using St = decltype(st);
    init_kernel<St><<<(cover + 255) / 256, 256, 0, s>>>(pop, fields, outlet_u, n, ny, nz, (uint32_t)np, u_in, fe);
    return cudaGetLastError();
  });
}

cudaError_t launch_step(uint32_t storage, bool gather, bool write_fields, const StepGeom& g, const StepArgs& a,
                        cudaStream_t s) {
  return by_storage(storage, [&](auto st) { return launch_step_t<decltype(st)>(gather, write_fields, g, a, s); });
}

cudaError_t launch_batch_step(uint32_t storage, bool gather, bool write_fields, dim3 block, uint32_t total_blocks,
                              const StepArgs* args, const BatchTiles* tiles, uint32_t count, uint32_t pending,
                              cudaStream_t s) {
  return by_storage(storage, [&](auto st) {
    return launch_batch_t<decltype(st)>(gather, write_fields, block, total_blocks, args, tiles, count, pending, s);
  });
}

uint32_t batch_persist_blocks(uint32_t storage, dim3 block, uint32_t sm_count) {
  int per_sm = 0;
  const int threads = (int)(block.x * block.y);
  cudaError_t e = by_storage(storage, [&](auto st) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persist_kernel<decltype(st)>, threads, 0);
  });
  if (e != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    return 0;
  }
  return (uint32_t)per_sm * sm_count;
}

cudaError_t launch_batch_persist(uint32_t storage, dim3 block, uint32_t grid, uint32_t total_blocks,
                                 const StepArgs* args, const BatchTiles* tiles, uint32_t count, uint32_t k0,
                                 uint32_t nsteps, uint32_t pending0, bool fields_last, unsigned int* sync,
                                 cudaStream_t s) {
  return by_storage(storage, [&](auto st) {
    return launch_batch_persist_t<decltype(st)>(block, grid, total_blocks, args, tiles, count, k0, nsteps, pending0,
                                                fields_last, sync, s);
  });
}

cudaError_t launch_force_reduce(const ReduceArgs* args, uint32_t count, uint32_t nsteps, bool with_mass,
                                cudaStream_t s) {
  if ((nsteps == 0 && !with_mass) || count == 0) return cudaSuccess;
  return launch_chained(force_reduce_kernel, dim3(nsteps * RED_FCHUNKS + (with_mass ? RED_MCHUNKS : 0u), count),
                        dim3(RED_THREADS), s, args, nsteps, with_mass ? 1u : 0u);
}

// The force readout in one launch: the accumulators into a wt_forces record
// (host-mapped memory, so no copy follows) and, with reset, their zeroing.
// One warp; each lane reads its words before it clears them.
__global__ void force_readback_kernel(double* totals, int32_t* raw, unsigned int* counters, wt_forces* out,
                                      uint64_t steps, int reset) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t t = threadIdx.x;
  if (t < 9) {
    out->sum[t] = totals[t];
    if (reset) totals[t] = 0.0;
  }
  if (t == 9) out->mass = totals[9];
  if (t < 12) {
    out->raw[t] = raw[t];
    if (reset) raw[t] = 0;
  }
  if (t == 12) {
    out->guarded = counters[0];
    out->steps = steps;
    if (reset) counters[0] = 0u;
  }
}

cudaError_t launch_force_readback(double* totals, int32_t* raw, unsigned int* counters, wt_forces* out,
                                  uint64_t steps, int reset, cudaStream_t s) {
  return launch_chained(force_readback_kernel, dim3(1), dim3(32), s, totals, raw, counters, out, steps, reset);
}

cudaError_t launch_read_pop(uint32_t storage, const void* pop, float* out, uint32_t n, uint64_t np, cudaStream_t s) {
  return by_storage(storage, [&](auto st) {
    read_pop_kernel<decltype(st)><<<(n + 255) / 256, 256, 0, s>>>(pop, out, n, (uint32_t)np);
    return cudaGetLastError();
  });
}

cudaError_t launch_write_pop(uint32_t storage, const float* in, void* pop, uint32_t n, uint64_t np, cudaStream_t s) {
  return by_storage(storage, [&](auto st) {
    write_pop_kernel<decltype(st)><<<(n + 255) / 256, 256, 0, s>>>(in, pop, n, (uint32_t)np);
    return cudaGetLastError();
  });
}

cudaError_t launch_coarse_average(const float4* fields, const uint32_t* cellw, uint32_t nx, uint32_t ny, uint32_t nz,
                                  float4* coarse, uint32_t cx, uint32_t cy, uint32_t cz, cudaStream_t s) {
  const uint32_t n = cx * cy * cz;
  coarse_average_kernel<<<(n + 127) / 128, 128, 0, s>>>(fields, cellw, nx, ny, nz, coarse, cx, cy, cz);
  return cudaGetLastError();
}

cudaError_t launch_resample_init(uint32_t storage, const float4* coarse, uint32_t cx, uint32_t cy, uint32_t cz,
                                 void* pop, float4* fields, float4* outlet_u, uint32_t nx, uint32_t ny, uint32_t nz,
                                 uint64_t np, cudaStream_t s) {
  const uint32_t n = nx * ny * nz;
  return by_storage(storage, [&](auto st) {
    resample_kernel<decltype(st)><<<(n + 255) / 256, 256, 0, s>>>(coarse, cx, cy, cz, pop, fields, outlet_u, nx, ny,
                                                                  nz, (uint32_t)np);
    return cudaGetLastError();
  });
}

}  // namespace wt
