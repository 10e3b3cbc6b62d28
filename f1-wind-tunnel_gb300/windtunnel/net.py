"""The warm start's network operators (include/wt_net.h) over ctypes.

Tensors are torch tensors on the GPU used only as device memory; every
operation runs in libwt's own kernels (the convolutions on the tensor cores),
enqueued on torch's current stream so that allocation and compute stay ordered.
"""
import ctypes

from . import _abi


class ConvShape(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_uint32), ("d", ctypes.c_uint32), ("h", ctypes.c_uint32), ("w", ctypes.c_uint32),
                ("cin", ctypes.c_uint32), ("cout", ctypes.c_uint32), ("taps", ctypes.c_uint32)]


_vp, _u32, _u64, _f = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float
_CS = ctypes.POINTER(ConvShape)
PROTOS = {
    "wt_conv3d_forward": (ctypes.c_int, [_CS, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "wt_conv3d_backward_data": (ctypes.c_int, [_CS, _vp, _vp, _vp, _vp]),
    "wt_conv3d_backward_weight": (ctypes.c_int, [_CS, _vp, _vp, _vp, _vp, _vp]),
    "wt_conv3d_workspace_bytes": (ctypes.c_size_t, [_CS]),
    "wt_nn_weight_transpose": (ctypes.c_int, [_vp, _vp, _u32, _u32, _u32, _vp]),
    "wt_nn_pool2_forward": (ctypes.c_int, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp]),
    "wt_nn_pool2_backward": (ctypes.c_int, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp]),
    "wt_nn_up2_forward": (ctypes.c_int, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp]),
    "wt_nn_up2_backward": (ctypes.c_int, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp]),
    "wt_nn_add": (ctypes.c_int, [_vp, _vp, _vp, _u64, _vp]),
    "wt_nn_grad_to_bf16": (ctypes.c_int, [_vp, _vp, _vp, _vp, _u64, _vp]),
    "wt_nn_bias_grad": (ctypes.c_int, [_vp, _vp, _u64, _u32, _vp]),
    "wt_nn_mse": (ctypes.c_int, [_vp, _u32, _vp, _vp, _u64, _f, _vp, _vp, _vp]),
    "wt_nn_adam": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _u64, _f, _f, _f, _f, _u32, _vp]),
    "wt_nn_to_bf16": (ctypes.c_int, [_vp, _vp, _u64, _vp]),
    "wt_net_check": (ctypes.c_int, []),
    "wt_net_set_stage_wait_limit": (ctypes.c_uint32, [ctypes.c_uint32]),
    "wt_net_last_error": (ctypes.c_char_p, []),
}


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Ops:
    """Thin wrappers: tensors in, status checked, work on torch's current stream."""

    def __init__(self, lib=None):
        self.lib = lib or _abi.load()
        for name, (res, args) in PROTOS.items():
            fn = getattr(self.lib, name)
            fn.restype, fn.argtypes = res, args
        import torch
        self.torch = torch

    def _s(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _ok(self, rc, what):
        if rc != 0:
            raise _abi.WindTunnelError(rc, f"{what}: {self.lib.wt_net_last_error().decode()}")

    @staticmethod
    def shape(x_shape, cin, cout, taps):
        b, d, h, w = x_shape[:4]
        return ConvShape(b, d, h, w, cin, cout, taps)

    def conv_forward(self, x, w, bias, y, relu):
        cout, taps, cin = w.shape
        s = self.shape(x.shape, cin, cout, taps)
        self._ok(self.lib.wt_conv3d_forward(ctypes.byref(s), _p(x), _p(w), _p(bias), _p(y), int(relu), self._s()),
                 "conv forward")

    def conv_backward_data(self, dy, wt, dx, cin, cout, taps):
        s = self.shape(dy.shape, cin, cout, taps)
        self._ok(self.lib.wt_conv3d_backward_data(ctypes.byref(s), _p(dy), _p(wt), _p(dx), self._s()), "conv dgrad")

    def workspace_bytes(self, x_shape, cin, cout, taps):
        s = self.shape(x_shape, cin, cout, taps)
        return int(self.lib.wt_conv3d_workspace_bytes(ctypes.byref(s)))

    def conv_backward_weight(self, x, dy, dw, ws, taps):
        cin, cout = x.shape[-1], dy.shape[-1]
        s = self.shape(x.shape, cin, cout, taps)
        self._ok(self.lib.wt_conv3d_backward_weight(ctypes.byref(s), _p(x), _p(dy), _p(dw), _p(ws), self._s()),
                 "conv wgrad")

    def weight_transpose(self, w, wt):
        cout, taps, cin = w.shape
        self._ok(self.lib.wt_nn_weight_transpose(_p(w), _p(wt), cout, taps, cin, self._s()), "weight transpose")

    def pool2(self, x, y):
        b, d, h, w, c = x.shape
        self._ok(self.lib.wt_nn_pool2_forward(_p(x), _p(y), b, d, h, w, c, self._s()), "pool2")

    def pool2_backward(self, dy, dx):
        b, d, h, w, c = dx.shape
        self._ok(self.lib.wt_nn_pool2_backward(_p(dy), _p(dx), b, d, h, w, c, self._s()), "pool2 backward")

    def up2(self, x, y):
        b, d, h, w, c = x.shape
        self._ok(self.lib.wt_nn_up2_forward(_p(x), _p(y), b, d, h, w, c, self._s()), "up2")

    def up2_backward(self, dy, dx):
        b, d, h, w, c = dx.shape
        self._ok(self.lib.wt_nn_up2_backward(_p(dy), _p(dx), b, d, h, w, c, self._s()), "up2 backward")

    def add(self, a, b, y):
        self._ok(self.lib.wt_nn_add(_p(a), _p(b), _p(y), a.numel(), self._s()), "add")

    def grad_to_bf16(self, g, g2, act, out):
        self._ok(self.lib.wt_nn_grad_to_bf16(_p(g), _p(g2), _p(act), _p(out), g.numel(), self._s()), "grad to bf16")

    def bias_grad(self, dy, db):
        c = dy.shape[-1]
        self._ok(self.lib.wt_nn_bias_grad(_p(dy), _p(db), dy.numel() // c, c, self._s()), "bias grad")

    def mse(self, pred, target, mask, norm, dpred, loss_sum):
        cp = pred.shape[-1]
        rows = pred.numel() // cp
        self._ok(self.lib.wt_nn_mse(_p(pred), cp, _p(target), _p(mask), rows, float(norm), _p(dpred), _p(loss_sum),
                                    self._s()), "mse")

    def adam(self, p, g, m, v, pb, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        self._ok(self.lib.wt_nn_adam(_p(p), _p(g), _p(m), _p(v), _p(pb), p.numel(), float(lr), b1, b2, eps, int(step),
                                     self._s()), "adam")

    def to_bf16(self, x, y):
        self._ok(self.lib.wt_nn_to_bf16(_p(x), _p(y), x.numel(), self._s()), "to bf16")

    def check(self):
        """Raises if a convolution gave up waiting on its tensor-core pipeline."""
        flag = self.lib.wt_net_check()
        if flag < 0:
            raise _abi.WindTunnelError(flag, self.lib.wt_net_last_error().decode())
        if flag:
            raise _abi.WindTunnelError(-2, "a convolution kernel's pipeline wait expired; results are invalid")
