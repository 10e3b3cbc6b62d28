"""Test infrastructure: float64 numpy restatement of the warm-start network's
operators (include/wt_net.h), the checker for the library's tensor-core
convolution kernels and their gradients.  Only tests import it.

Layouts follow the library: activations channels-last [batch, d, h, w, c],
weights [cout, taps, cin] with tap t = (dz, dy, dx) = (t//9 - 1, t//3 % 3 - 1,
t % 3 - 1) for 3x3x3 kernels (zero padding 1) or the single centre tap.
The reference application has no learned component; these definitions are the
project's own (textbook convolution, pooling and their adjoints)."""
import numpy as np


def tap_offsets(taps):
    if taps == 1:
        return [(0, 0, 0)]
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def shift(x, dz, dy, dx):
    """out[b, z, y, x] = x[b, z + dz, y + dy, x + dx] (zero outside)."""
    out = np.zeros_like(x)
    B, D, H, W, C = x.shape
    zs, ze = max(0, -dz), min(D, D - dz)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if zs < ze and ys < ye and xs < xe:
        out[:, zs:ze, ys:ye, xs:xe] = x[:, zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv3d(x, w, bias=None, relu=False):
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    cout, taps, cin = w.shape
    y = np.zeros(x.shape[:4] + (cout,))
    for t, (dz, dy, dx) in enumerate(tap_offsets(taps)):
        y += shift(x, dz, dy, dx) @ w[:, t, :].T
    if bias is not None:
        y += np.asarray(bias, np.float64)
    return np.maximum(y, 0.0) if relu else y


def conv3d_backward_data(dy, w):
    """dx[m, ci] = sum_{t, co} dy[m - off(t), co] w[co, t, ci]."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    cout, taps, cin = w.shape
    dx = np.zeros(dy.shape[:4] + (cin,))
    for t, (dz, dyy, dxx) in enumerate(tap_offsets(taps)):
        dx += shift(dy, -dz, -dyy, -dxx) @ w[:, t, :]
    return dx


def conv3d_backward_weight(x, dy, taps):
    """dw[co, t, ci] = sum_m x[m + off(t), ci] dy[m, co]."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    cin, cout = x.shape[-1], dy.shape[-1]
    dw = np.zeros((cout, taps, cin))
    dyf = dy.reshape(-1, cout)
    for t, (dz, dyy, dxx) in enumerate(tap_offsets(taps)):
        dw[:, t, :] = dyf.T @ shift(x, dz, dyy, dxx).reshape(-1, cin)
    return dw


def pool2(x):
    B, D, H, W, C = x.shape
    return np.asarray(x, np.float64).reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def pool2_backward(dy):
    return np.repeat(np.repeat(np.repeat(np.asarray(dy, np.float64), 2, 1), 2, 2), 2, 3) / 8.0


def up2(x):
    return np.repeat(np.repeat(np.repeat(np.asarray(x, np.float64), 2, 1), 2, 2), 2, 3)


def up2_backward(dy):
    B, D, H, W, C = dy.shape
    return np.asarray(dy, np.float64).reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def bf16_round(a):
    """Round float values to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)
