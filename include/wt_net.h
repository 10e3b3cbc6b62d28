/* libwt surrogate operators: the learned warm start's 3-D convolution network
 * (BF16 activations and weights, FP32 accumulation) trained and evaluated on the
 * GPU by the library's own kernels.
 *
 * The reference has no learned component; these entry points serve the warm
 * start, whose output (ux, uy, uz, rho on a coarse grid) enters the simulation
 * through wt_reset_from (wt.h) in place of LBM_INIT's uniform state
 * (src/engine/wgsl.ts:141-155, engine.ts:371-381).
 *
 * Conventions.  All tensor arguments are DEVICE pointers owned by the caller;
 * the calls enqueue work on `stream` (a cudaStream_t, NULL = the default stream)
 * and return at once.  Activations are channels-last [batch][d][h][w][c] BF16;
 * convolution weights are [cout][taps][cin] with taps = 27 (3x3x3, zero padding
 * 1, stride 1; tap t = (dz, dy, dx) = (t/9 - 1, t/3%3 - 1, t%3 - 1)) or 1.
 * Channel counts must be multiples of 8 and at most 128.  Return 0 or a
 * negative WT_ERR_* code (wt.h); wt_net_last_error() describes the last failure
 * of the calling thread.
 */
#ifndef WT_NET_H
#define WT_NET_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wt_conv_shape {
  uint32_t batch, d, h, w; /* activation grid */
  uint32_t cin, cout;      /* multiples of 8, <= 128 */
  uint32_t taps;           /* 27 or 1 */
} wt_conv_shape;

/* y = act(conv(x, w) + bias); act = ReLU when relu != 0.  bias may be NULL. */
int wt_conv3d_forward(const wt_conv_shape* s, const void* x, const void* w, const float* bias, void* y, int relu,
                      void* stream);
/* dx[m][ci] = sum_{t,co} dy[m - off(t)][co] * w[co][t][ci]  (FP32 output).
 * wt is the weight re-laid out as [cin][taps][cout] (wt_nn_weight_transpose). */
int wt_conv3d_backward_data(const wt_conv_shape* s, const void* dy, const void* wt, float* dx, void* stream);
/* dw[co][t][ci] = sum_m x[m + off(t)][ci] * dy[m][co]  (FP32, overwritten).
 * workspace: wt_conv3d_workspace_bytes() bytes of device memory. */
int wt_conv3d_backward_weight(const wt_conv_shape* s, const void* x, const void* dy, float* dw, void* workspace,
                              void* stream);
size_t wt_conv3d_workspace_bytes(const wt_conv_shape* s);

/* Element-wise and reduction operators of the network (shapes as above; c = channels). */
int wt_nn_weight_transpose(const void* w, void* wt, uint32_t cout, uint32_t taps, uint32_t cin, void* stream);
/* 2x2x2 average pool / its gradient; d, h, w are the FINE grid and must be even. */
int wt_nn_pool2_forward(const void* x, void* y, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                        void* stream);
int wt_nn_pool2_backward(const float* dy, float* dx, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                         void* stream);
/* Nearest 2x upsampling / its gradient; d, h, w are the COARSE grid. */
int wt_nn_up2_forward(const void* x, void* y, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                      void* stream);
int wt_nn_up2_backward(const float* dy, float* dx, uint32_t batch, uint32_t d, uint32_t h, uint32_t w, uint32_t c,
                       void* stream);
/* y = a + b (BF16). */
int wt_nn_add(const void* a, const void* b, void* y, uint64_t n, void* stream);
/* out = bf16((g + g2) * (act > 0)); g2 and act may be NULL (no term / no mask). */
int wt_nn_grad_to_bf16(const float* g, const float* g2, const void* act, void* out, uint64_t n, void* stream);
/* db[c] = sum over rows of dy[rows][c] (FP32, overwritten, fixed summation
 * order); c must divide 256. */
int wt_nn_bias_grad(const void* dy, float* db, uint64_t rows, uint32_t c, void* stream);
/* Masked mean-square error of pred[m][0:4] (BF16, row stride cp) against
 * target[m][0:4] (FP32): loss_sum[0] += sum mask*(p-t)^2; dpred[m][k] =
 * bf16(2 mask (p - t) / norm) for k < 4, 0 for 4 <= k < cp. */
int wt_nn_mse(const void* pred, uint32_t cp, const float* target, const float* mask, uint64_t rows, float norm,
              void* dpred, double* loss_sum, void* stream);
/* One Adam step (Kingma & Ba 2015, bias-corrected) over n FP32 parameters; also
 * refreshes their BF16 copy. */
int wt_nn_adam(float* param, const float* grad, float* m, float* v, void* param_bf16, uint64_t n, float lr,
               float beta1, float beta2, float eps, uint32_t step, void* stream);
/* FP32 -> BF16 conversion of n values. */
int wt_nn_to_bf16(const float* x, void* y, uint64_t n, void* stream);

/* Nonzero if a convolution kernel gave up waiting on its tensor-core pipeline
 * since the last call (the wait limit expired; the result is then invalid);
 * reading clears the flag.  Synchronizes the device. */
int wt_net_check(void);
const char* wt_net_last_error(void);

/* Fault-path test hook: the number of polls each K-slice stage wait of the
 * convolution pipeline makes before it gives up (default 2^21), for the
 * launches that follow; returns the previous value.  0 makes every stage wait
 * give up at once, so a convolution with more than two K slices leaves its K
 * loop, reports the expiry through wt_net_check and writes no output.  The
 * wait for the issued MMAs before tensor memory is freed always keeps its full
 * limit.  Not for production use; restore the returned value afterwards. */
uint32_t wt_net_set_stage_wait_limit(uint32_t polls);

#ifdef __cplusplus
}
#endif

#endif /* WT_NET_H */
