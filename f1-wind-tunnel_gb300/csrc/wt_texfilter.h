// Sampling of the car mesh's albedo textures: the rgba8unorm-srgb textures
// with a full mip chain and the linear / linear / linear, repeat sampler that
// MeshCar creates (src/engine/mesh-car.ts:97-127), evaluated as this project
// defines it.  WebGPU leaves filtering precision, the level-of-detail formula
// and anisotropic filtering to the implementation; this definition is
// isotropic trilinear filtering (the sampler's maxAnisotropy 8 is not
// reproduced), shared by the device kernel and the CPU pipeline that checks
// it, so both give the same bits.
//
//   texels    sRGB bytes decoded to linear with the correctly rounded table
//             below ((c/255)/12.92 up to 0.04045, ((c/255 + 0.055)/1.055)^2.4
//             above), alpha c/255; filtering happens after decoding
//   levels    level m is max(1, w >> m) x max(1, h >> m), made by halveRgba
//             (mesh-car.ts:30-44) from level m - 1; floor(log2(max(w, h))) + 1
//             levels
//   lod       from the screen-space derivatives of uv (scaled to texels of
//             level 0): lambda = log2(max(|ddx|^2, |ddy|^2)) / 2, clamped to
//             [0, levels - 1] (a NaN gives 0)
//   level     bilinear: x = u * w - 0.5, i = floor(x), t = x - i, texel
//             indices wrapped into [0, w) (repeat), blended along x then y
//   trilinear floor(lambda) and the next level, mixed with lambda - floor(lambda)
// Built without floating-point contraction like the rest of the renderer.
#pragma once
#include <math.h>
#include <stdint.h>

#include "wt_fmath.h"

namespace wtx {

#if defined(__CUDACC__)
#define WTX_FN __device__ __forceinline__
__device__ __constant__
#else
#define WTX_FN static inline
#endif
static const float SRGB_TO_LINEAR[256] = {
    0x0p+0f, 0x1.3e4568p-12f, 0x1.3e4568p-11f, 0x1.dd681cp-11f,
    0x1.3e4568p-10f, 0x1.8dd6c2p-10f, 0x1.dd681cp-10f, 0x1.167cbap-9f,
    0x1.3e4568p-9f, 0x1.660e14p-9f, 0x1.8dd6c2p-9f, 0x1.b6a31cp-9f,
    0x1.e1e31ep-9f, 0x1.07c38cp-8f, 0x1.1fcc2cp-8f, 0x1.390ffap-8f,
    0x1.53936cp-8f, 0x1.6f5adep-8f, 0x1.8c6a94p-8f, 0x1.aac6cp-8f,
    0x1.ca7382p-8f, 0x1.eb74e2p-8f, 0x1.06e76cp-7f, 0x1.18c2a6p-7f,
    0x1.2b4e0ap-7f, 0x1.3e8b7cp-7f, 0x1.527cd6p-7f, 0x1.6723eep-7f,
    0x1.7c8292p-7f, 0x1.929a88p-7f, 0x1.a96d92p-7f, 0x1.c0fd68p-7f,
    0x1.d94bbep-7f, 0x1.f25a44p-7f, 0x1.061552p-6f, 0x1.135f3ep-6f,
    0x1.210bb8p-6f, 0x1.2f1b8cp-6f, 0x1.3d8f84p-6f, 0x1.4c6866p-6f,
    0x1.5ba6fap-6f, 0x1.6b4c04p-6f, 0x1.7b5842p-6f, 0x1.8bcc74p-6f,
    0x1.9ca958p-6f, 0x1.adefaap-6f, 0x1.bfa02p-6f, 0x1.d1bb74p-6f,
    0x1.e4425ap-6f, 0x1.f73586p-6f, 0x1.054ad4p-5f, 0x1.0f31bap-5f,
    0x1.194fccp-5f, 0x1.23a55ep-5f, 0x1.2e32c8p-5f, 0x1.38f86p-5f,
    0x1.43f678p-5f, 0x1.4f2d64p-5f, 0x1.5a9d76p-5f, 0x1.664702p-5f,
    0x1.722a56p-5f, 0x1.7e47c8p-5f, 0x1.8a9fa4p-5f, 0x1.97323ap-5f,
    0x1.a3ffd8p-5f, 0x1.b108dp-5f, 0x1.be4d6cp-5f, 0x1.cbcdfap-5f,
    0x1.d98ac6p-5f, 0x1.e7841cp-5f, 0x1.f5ba48p-5f, 0x1.0216cap-4f,
    0x1.096f26p-4f, 0x1.10e65cp-4f, 0x1.187c9p-4f, 0x1.2031e8p-4f,
    0x1.280688p-4f, 0x1.2ffa92p-4f, 0x1.380e2ap-4f, 0x1.404174p-4f,
    0x1.489494p-4f, 0x1.5107acp-4f, 0x1.599adep-4f, 0x1.624e4ep-4f,
    0x1.6b221ep-4f, 0x1.74167p-4f, 0x1.7d2b66p-4f, 0x1.86612p-4f,
    0x1.8fb7cp-4f, 0x1.992f68p-4f, 0x1.a2c83ap-4f, 0x1.ac8256p-4f,
    0x1.b65ddcp-4f, 0x1.c05aecp-4f, 0x1.ca79a8p-4f, 0x1.d4ba3p-4f,
    0x1.df1ca2p-4f, 0x1.e9a12p-4f, 0x1.f447cap-4f, 0x1.ff10bcp-4f,
    0x1.04fe0cp-3f, 0x1.0a84fep-3f, 0x1.101d44p-3f, 0x1.15c6eep-3f,
    0x1.1b8208p-3f, 0x1.214ea6p-3f, 0x1.272cd4p-3f, 0x1.2d1ca2p-3f,
    0x1.331e1ep-3f, 0x1.393158p-3f, 0x1.3f566p-3f, 0x1.458d42p-3f,
    0x1.4bd60ep-3f, 0x1.5230d4p-3f, 0x1.589dap-3f, 0x1.5f1c84p-3f,
    0x1.65ad8ap-3f, 0x1.6c50c4p-3f, 0x1.73063ep-3f, 0x1.79ce06p-3f,
    0x1.80a82ep-3f, 0x1.8794cp-3f, 0x1.8e93ccp-3f, 0x1.95a55ep-3f,
    0x1.9cc986p-3f, 0x1.a40052p-3f, 0x1.ab49cep-3f, 0x1.b2a60ap-3f,
    0x1.ba1512p-3f, 0x1.c196f4p-3f, 0x1.c92bbep-3f, 0x1.d0d37cp-3f,
    0x1.d88e3ep-3f, 0x1.e05c0ep-3f, 0x1.e83cfcp-3f, 0x1.f03116p-3f,
    0x1.f83866p-3f, 0x1.00297ep-2f, 0x1.044072p-2f, 0x1.086116p-2f,
    0x1.0c8b7p-2f, 0x1.10bf86p-2f, 0x1.14fd6p-2f, 0x1.194502p-2f,
    0x1.1d9676p-2f, 0x1.21f1bep-2f, 0x1.2656e4p-2f, 0x1.2ac5ecp-2f,
    0x1.2f3edep-2f, 0x1.33c1cp-2f, 0x1.384e98p-2f, 0x1.3ce56cp-2f,
    0x1.418642p-2f, 0x1.46312p-2f, 0x1.4ae60ep-2f, 0x1.4fa51p-2f,
    0x1.546e2cp-2f, 0x1.59416cp-2f, 0x1.5e1edp-2f, 0x1.630664p-2f,
    0x1.67f82ap-2f, 0x1.6cf428p-2f, 0x1.71fa68p-2f, 0x1.770aecp-2f,
    0x1.7c25bcp-2f, 0x1.814adcp-2f, 0x1.867a54p-2f, 0x1.8bb428p-2f,
    0x1.90f86p-2f, 0x1.9647p-2f, 0x1.9ba01p-2f, 0x1.a10394p-2f,
    0x1.a67192p-2f, 0x1.abea1p-2f, 0x1.b16d14p-2f, 0x1.b6faa4p-2f,
    0x1.bc92c6p-2f, 0x1.c2357ep-2f, 0x1.c7e2d2p-2f, 0x1.cd9acap-2f,
    0x1.d35d6ap-2f, 0x1.d92ab6p-2f, 0x1.df02b8p-2f, 0x1.e4e57p-2f,
    0x1.ead2e8p-2f, 0x1.f0cb26p-2f, 0x1.f6ce2cp-2f, 0x1.fcdcp-2f,
    0x1.017a56p-1f, 0x1.048c18p-1f, 0x1.07a34ap-1f, 0x1.0abfeep-1f,
    0x1.0de208p-1f, 0x1.11099ap-1f, 0x1.1436a8p-1f, 0x1.176932p-1f,
    0x1.1aa13ep-1f, 0x1.1ddecap-1f, 0x1.2121dep-1f, 0x1.246a7ap-1f,
    0x1.27b8ap-1f, 0x1.2b0c54p-1f, 0x1.2e6598p-1f, 0x1.31c46ep-1f,
    0x1.3528dcp-1f, 0x1.3892ep-1f, 0x1.3c028p-1f, 0x1.3f77bcp-1f,
    0x1.42f29ap-1f, 0x1.467318p-1f, 0x1.49f93ep-1f, 0x1.4d850ap-1f,
    0x1.511682p-1f, 0x1.54ada4p-1f, 0x1.584a78p-1f, 0x1.5becfep-1f,
    0x1.5f9538p-1f, 0x1.634328p-1f, 0x1.66f6d4p-1f, 0x1.6ab03ap-1f,
    0x1.6e6f6p-1f, 0x1.723448p-1f, 0x1.75fef4p-1f, 0x1.79cf64p-1f,
    0x1.7da59ep-1f, 0x1.8181a4p-1f, 0x1.856378p-1f, 0x1.894b1cp-1f,
    0x1.8d3892p-1f, 0x1.912bdep-1f, 0x1.9525p-1f, 0x1.9923fep-1f,
    0x1.9d28d8p-1f, 0x1.a13392p-1f, 0x1.a5442cp-1f, 0x1.a95aacp-1f,
    0x1.ad771p-1f, 0x1.b1995ep-1f, 0x1.b5c198p-1f, 0x1.b9efbep-1f,
    0x1.be23d4p-1f, 0x1.c25ddep-1f, 0x1.c69ddcp-1f, 0x1.cae3d2p-1f,
    0x1.cf2fcp-1f, 0x1.d381aap-1f, 0x1.d7d994p-1f, 0x1.dc377ep-1f,
    0x1.e09b6ap-1f, 0x1.e5055cp-1f, 0x1.e97556p-1f, 0x1.edeb5cp-1f,
    0x1.f2676cp-1f, 0x1.f6e98cp-1f, 0x1.fb71bcp-1f, 0x1p+0f,
};

struct Level {
  const uint8_t* rgba;  // w x h texels, 4 bytes each, rows from the top
  int w, h;
};
struct Rgba {
  float r, g, b, a;
};

WTX_FN int wrap(int i, int n) {
  const int m = i % n;
  return m < 0 ? m + n : m;
}
WTX_FN Rgba texel(const Level& l, int x, int y) {
  const uint8_t* t = l.rgba + ((size_t)y * (size_t)l.w + (size_t)x) * 4;
  return Rgba{SRGB_TO_LINEAR[t[0]], SRGB_TO_LINEAR[t[1]], SRGB_TO_LINEAR[t[2]], (float)t[3] / 255.0f};
}
WTX_FN Rgba lerp4(Rgba a, Rgba b, float t) {
  const float s = 1.0f - t;
  return Rgba{a.r * s + b.r * t, a.g * s + b.g * t, a.b * s + b.b * t, a.a * s + b.a * t};
}
WTX_FN Rgba bilinear(const Level& l, float u, float v) {
  const float x = u * (float)l.w - 0.5f, y = v * (float)l.h - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float tx = x - fx, ty = y - fy;
  // texel indices of far-off coordinates: wrap the float first so the int conversion is exact
  float wx = fx - floorf(fx / (float)l.w) * (float)l.w, wy = fy - floorf(fy / (float)l.h) * (float)l.h;
  if (!(wx >= 0.0f && wx < 16777216.0f)) wx = 0.0f;  // NaN or infinite coordinates
  if (!(wy >= 0.0f && wy < 16777216.0f)) wy = 0.0f;
  const int x0 = wrap((int)wx, l.w), y0 = wrap((int)wy, l.h);
  const int x1 = wrap(x0 + 1, l.w), y1 = wrap(y0 + 1, l.h);
  const Rgba top = lerp4(texel(l, x0, y0), texel(l, x1, y0), tx);
  const Rgba bot = lerp4(texel(l, x0, y1), texel(l, x1, y1), tx);
  return lerp4(top, bot, ty);
}
// levels[0..n) of one texture; (dux, dvx) and (duy, dvy) the uv derivatives
// along x and y of the fragment's 2 x 2 quad
WTX_FN Rgba sample(const Level* levels, int n, float u, float v, float dux, float dvx, float duy, float dvy) {
  const float w0 = (float)levels[0].w, h0 = (float)levels[0].h;
  const float ax = dux * w0, ay = dvx * h0, bx = duy * w0, by = dvy * h0;
  const float lx = ax * ax + ay * ay, ly = bx * bx + by * by;
  const float rho2 = lx > ly ? lx : ly;
  float lod = wtm::log2f(rho2) * 0.5f;
  const float top = (float)(n - 1);
  lod = lod > 0.0f ? (lod < top ? lod : top) : 0.0f;  // a NaN lands on 0
  const int l0 = (int)floorf(lod);
  const int l1 = l0 + 1 < n ? l0 + 1 : n - 1;
  const float f = lod - (float)l0;
  const Rgba c0 = bilinear(levels[l0], u, v);
  if (f == 0.0f) return c0;
  return lerp4(c0, bilinear(levels[l1], u, v), f);
}

}  // namespace wtx
