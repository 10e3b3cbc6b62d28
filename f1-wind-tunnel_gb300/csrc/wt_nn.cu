// Element-wise and reduction operators of the warm-start network (include/wt_net.h):
// weight re-layout for the data gradient, 2x2x2 average pooling and nearest 2x
// upsampling with their gradients, skip additions, ReLU masking of gradients,
// bias gradients, the masked mean-square loss and the Adam update.  All are
// HBM-bound one-pass kernels over channels-last tensors.
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>

#include "wt_internal.h"
#include "wt_net.h"

namespace wt {
namespace {

constexpr uint32_t TB = 256;

inline uint32_t blocks_for(uint64_t n) {
  uint64_t b = (n + TB - 1) / TB;
  return (uint32_t)(b < 65535ull * 64 ? b : 65535ull * 64);
}

__global__ void weight_transpose_kernel(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt,
                                        uint32_t cout, uint32_t taps, uint32_t cin) {
  const uint64_t n = (uint64_t)cout * taps * cin;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ci = i % cin, t = (i / cin) % taps, co = (uint32_t)(i / ((uint64_t)cin * taps));
    wt[((uint64_t)ci * taps + t) * cout + co] = w[i];
  }
}

// y[b][z][y][x][c] = mean of the 8 fine cells x[b][2z+i][2y+j][2x+k][c] (d, h, w fine).
__global__ void pool2_fwd_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, uint32_t batch,
                                 uint32_t d, uint32_t h, uint32_t w, uint32_t c) {
  const uint32_t dc = d / 2, hc = h / 2, wc = w / 2;
  const uint64_t n = (uint64_t)batch * dc * hc * wc * c;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ch = i % c;
    uint64_t v = i / c;
    const uint32_t xc = v % wc; v /= wc;
    const uint32_t yc = v % hc; v /= hc;
    const uint32_t zc = v % dc;
    const uint64_t b = v / dc;
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const uint64_t src = (((b * d + 2 * zc + (q >> 2)) * h + 2 * yc + ((q >> 1) & 1)) * w + 2 * xc + (q & 1)) * c + ch;
      s += __bfloat162float(x[src]);
    }
    y[i] = __float2bfloat16_rn(s * 0.125f);
  }
}

// dx[fine] = dy[parent] / 8 (d, h, w fine).
__global__ void pool2_bwd_kernel(const float* __restrict__ dy, float* __restrict__ dx, uint32_t batch, uint32_t d,
                                 uint32_t h, uint32_t w, uint32_t c) {
  const uint64_t n = (uint64_t)batch * d * h * w * c;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ch = i % c;
    uint64_t v = i / c;
    const uint32_t xx = v % w; v /= w;
    const uint32_t yy = v % h; v /= h;
    const uint32_t zz = v % d;
    const uint64_t b = v / d;
    const uint64_t src = (((b * (d / 2) + zz / 2) * (h / 2) + yy / 2) * (w / 2) + xx / 2) * c + ch;
    dx[i] = dy[src] * 0.125f;
  }
}

// y[fine] = x[parent] (d, h, w coarse).
__global__ void up2_fwd_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, uint32_t batch,
                               uint32_t d, uint32_t h, uint32_t w, uint32_t c) {
  const uint32_t df = 2 * d, hf = 2 * h, wf = 2 * w;
  const uint64_t n = (uint64_t)batch * df * hf * wf * c;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ch = i % c;
    uint64_t v = i / c;
    const uint32_t xx = v % wf; v /= wf;
    const uint32_t yy = v % hf; v /= hf;
    const uint32_t zz = v % df;
    const uint64_t b = v / df;
    y[i] = x[(((b * d + zz / 2) * h + yy / 2) * w + xx / 2) * c + ch];
  }
}

// dx[coarse] = sum of dy over its 8 fine children (d, h, w coarse).
__global__ void up2_bwd_kernel(const float* __restrict__ dy, float* __restrict__ dx, uint32_t batch, uint32_t d,
                               uint32_t h, uint32_t w, uint32_t c) {
  const uint64_t n = (uint64_t)batch * d * h * w * c;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t ch = i % c;
    uint64_t v = i / c;
    const uint32_t xc = v % w; v /= w;
    const uint32_t yc = v % h; v /= h;
    const uint32_t zc = v % d;
    const uint64_t b = v / d;
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const uint64_t src =
          (((b * 2 * d + 2 * zc + (q >> 2)) * 2 * h + 2 * yc + ((q >> 1) & 1)) * 2 * w + 2 * xc + (q & 1)) * c + ch;
      s += dy[src];
    }
    dx[i] = s;
  }
}

__global__ void add_kernel(const __nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b,
                           __nv_bfloat16* __restrict__ y, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

__global__ void grad_to_bf16_kernel(const float* __restrict__ g, const float* __restrict__ g2,
                                    const __nv_bfloat16* __restrict__ act, __nv_bfloat16* __restrict__ out,
                                    uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    float v = g[i];
    if (g2) v += g2[i];
    if (act && !(__bfloat162float(act[i]) > 0.0f)) v = 0.0f;
    out[i] = __float2bfloat16_rn(v);
  }
}

// Bias gradient in two passes with a fixed summation order: block b of the first
// pass sums rows [b * chunk, (b + 1) * chunk) of every channel (thread t owns
// channel t % c and every (TB / c)-th row of the chunk, then the block folds its
// row phases in order) into partial[b][c]; the second pass sums the blocks.
constexpr uint32_t BG_BLOCKS = 512;

__global__ void bias_grad_partial_kernel(const __nv_bfloat16* __restrict__ dy, float* __restrict__ partial,
                                         uint64_t rows, uint32_t c, uint64_t chunk) {
  __shared__ float red[TB];
  const uint32_t phases = TB / c;  // c divides TB (c in {8, 16, 32, 64, 128})
  const uint32_t ch = threadIdx.x % c, ph = threadIdx.x / c;
  const uint64_t r0 = (uint64_t)blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
  float acc = 0.0f;
  for (uint64_t r = r0 + ph; r < r1; r += phases) acc += __bfloat162float(dy[r * c + ch]);
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < c) {
    float t = 0.0f;
    for (uint32_t q = 0; q < phases; q++) t += red[q * c + threadIdx.x];
    partial[(size_t)blockIdx.x * c + threadIdx.x] = t;
  }
}

__global__ void bias_grad_final_kernel(const float* __restrict__ partial, float* __restrict__ db, uint32_t nblocks,
                                       uint32_t c) {
  const uint32_t ch = blockIdx.x * blockDim.x + threadIdx.x;
  if (ch >= c) return;
  float t = 0.0f;
  for (uint32_t b = 0; b < nblocks; b++) t += partial[(size_t)b * c + ch];
  db[ch] = t;
}

// Per-block partial loss in double (fixed order), gradient written per element.
__global__ void mse_kernel(const __nv_bfloat16* __restrict__ pred, uint32_t cp, const float* __restrict__ target,
                           const float* __restrict__ mask, uint64_t rows, float inv_norm,
                           __nv_bfloat16* __restrict__ dpred, double* __restrict__ partial) {
  __shared__ double red[TB];
  double acc = 0.0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
    const float mk = mask ? mask[r] : 1.0f;
    for (uint32_t k = 0; k < cp; k++) {
      float gk = 0.0f;
      if (k < 4) {
        const float e = __bfloat162float(pred[r * cp + k]) - target[r * 4 + k];
        acc += (double)(mk * e * e);
        gk = 2.0f * mk * e * inv_norm;
      }
      dpred[r * cp + k] = __float2bfloat16_rn(gk);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (uint32_t s = TB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void sum_partials_kernel(const double* __restrict__ partial, uint32_t n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (uint32_t i = 0; i < n; i++) s += partial[i];
    *out += s;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, __nv_bfloat16* __restrict__ pb, uint64_t n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    const float pi = p[i] - upd;
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

int done(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    net_error() = std::string(what) + ": " + cudaGetErrorString(e);
    return WT_ERR_CUDA;
  }
  return WT_OK;
}

int bad(const char* what) {
  net_error() = std::string(what) + ": invalid argument";
  return WT_ERR_ARG;
}

inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }
typedef __nv_bfloat16 bf;

}  // namespace
}  // namespace wt

using namespace wt;

extern "C" {

int wt_nn_weight_transpose(const void* w, void* wt, uint32_t cout, uint32_t taps, uint32_t cin, void* stream) {
  if (!w || !wt || !cout || !taps || !cin) return bad("wt_nn_weight_transpose");
  const uint64_t n = (uint64_t)cout * taps * cin;
  weight_transpose_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(static_cast<const bf*>(w), static_cast<bf*>(wt), cout,
                                                                taps, cin);
  return done("wt_nn_weight_transpose");
}

int wt_nn_pool2_forward(const void* x, void* y, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                        void* stream) {
  if (!x || !y || !c || (d | h | w) & 1u || !d || !h || !w) return bad("wt_nn_pool2_forward");
  const uint64_t n = (uint64_t)batch * (d / 2) * (h / 2) * (w / 2) * c;
  pool2_fwd_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(static_cast<const bf*>(x), static_cast<bf*>(y), batch, d, h,
                                                         w, c);
  return done("wt_nn_pool2_forward");
}

int wt_nn_pool2_backward(const float* dy, float* dx, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                         void* stream) {
  if (!dy || !dx || !c || (d | h | w) & 1u || !d || !h || !w) return bad("wt_nn_pool2_backward");
  const uint64_t n = (uint64_t)batch * d * h * w * c;
  pool2_bwd_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(dy, dx, batch, d, h, w, c);
  return done("wt_nn_pool2_backward");
}

int wt_nn_up2_forward(const void* x, void* y, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                      void* stream) {
  if (!x || !y || !c || !d || !h || !w) return bad("wt_nn_up2_forward");
  const uint64_t n = (uint64_t)batch * 8 * d * h * w * c;
  up2_fwd_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(static_cast<const bf*>(x), static_cast<bf*>(y), batch, d, h, w,
                                                       c);
  return done("wt_nn_up2_forward");
}

int wt_nn_up2_backward(const float* dy, float* dx, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                       void* stream) {
  if (!dy || !dx || !c || !d || !h || !w) return bad("wt_nn_up2_backward");
  const uint64_t n = (uint64_t)batch * d * h * w * c;
  up2_bwd_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(dy, dx, batch, d, h, w, c);
  return done("wt_nn_up2_backward");
}

int wt_nn_add(const void* a, const void* b, void* y, uint64_t n, void* stream) {
  if (!a || !b || !y) return bad("wt_nn_add");
  if (n == 0) return WT_OK;
  add_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(static_cast<const bf*>(a), static_cast<const bf*>(b),
                                                   static_cast<bf*>(y), n);
  return done("wt_nn_add");
}

int wt_nn_grad_to_bf16(const float* g, const float* g2, const void* act, void* out, uint64_t n, void* stream) {
  if (!g || !out) return bad("wt_nn_grad_to_bf16");
  if (n == 0) return WT_OK;
  grad_to_bf16_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(g, g2, static_cast<const bf*>(act), static_cast<bf*>(out), n);
  return done("wt_nn_grad_to_bf16");
}

int wt_nn_bias_grad(const void* dy, float* db, uint64_t rows, uint32_t c, void* stream) {
  if (!dy || !db || !c || c > TB || TB % c) return bad("wt_nn_bias_grad");
  static float* partial = nullptr;  // BG_BLOCKS x 256 floats, allocated once
  if (!partial && cudaMalloc(&partial, (size_t)BG_BLOCKS * TB * sizeof(float)) != cudaSuccess)
    return bad("wt_nn_bias_grad scratch");
  const uint64_t chunk = rows ? (rows + BG_BLOCKS - 1) / BG_BLOCKS : 1;
  const uint32_t nb = (uint32_t)(rows ? (rows + chunk - 1) / chunk : 1);
  bias_grad_partial_kernel<<<nb, TB, 0, S(stream)>>>(static_cast<const bf*>(dy), partial, rows, c, chunk);
  bias_grad_final_kernel<<<(c + 127) / 128, 128, 0, S(stream)>>>(partial, db, nb, c);
  return done("wt_nn_bias_grad");
}

int wt_nn_mse(const void* pred, uint32_t cp, const float* target, const float* mask, uint64_t rows, float norm,
              void* dpred, double* loss_sum, void* stream) {
  if (!pred || !target || !dpred || !loss_sum || cp < 4 || !(norm > 0.0f)) return bad("wt_nn_mse");
  // partial sums live in the tail of a small static buffer: at most 1024 blocks
  static double* partial = nullptr;
  if (!partial && cudaMalloc(&partial, 1024 * sizeof(double)) != cudaSuccess) return bad("wt_nn_mse scratch");
  const uint32_t nb = (uint32_t)((rows + TB - 1) / TB < 1024 ? (rows + TB - 1) / TB : 1024);
  const uint32_t grid = nb ? nb : 1;
  mse_kernel<<<grid, TB, 0, S(stream)>>>(static_cast<const bf*>(pred), cp, target, mask, rows, 1.0f / norm,
                                         static_cast<bf*>(dpred), partial);
  sum_partials_kernel<<<1, 32, 0, S(stream)>>>(partial, grid, loss_sum);
  return done("wt_nn_mse");
}

int wt_nn_adam(float* param, const float* grad, float* m, float* v, void* param_bf16, uint64_t n, float lr,
               float beta1, float beta2, float eps, uint32_t step, void* stream) {
  if (!param || !grad || !m || !v || step == 0) return bad("wt_nn_adam");
  if (n == 0) return WT_OK;
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(param, grad, m, v, static_cast<bf*>(param_bf16), n, lr, beta1,
                                                    beta2, eps, c1, c2);
  return done("wt_nn_adam");
}

int wt_nn_to_bf16(const float* x, void* y, uint64_t n, void* stream) {
  if (!x || !y) return bad("wt_nn_to_bf16");
  if (n == 0) return WT_OK;
  to_bf16_kernel<<<blocks_for(n), TB, 0, S(stream)>>>(x, static_cast<bf*>(y), n);
  return done("wt_nn_to_bf16");
}

}  // extern "C"
