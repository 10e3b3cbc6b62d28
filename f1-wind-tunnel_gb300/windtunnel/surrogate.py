"""Learned warm start: a 3-D convolutional encoder-decoder that maps the car's
coarse signed distance field plus its ride heights and wing angles to a coarse
(ux, uy, uz, rho) flow field, which then replaces LBM_INIT's uniform state
(src/engine/wgsl.ts:141-155) through wt_reset_from.

Network (channels-last BF16 activations, FP32 accumulation; every operation a
libwt kernel, the 3x3x3 convolutions on the tensor cores):

    input 8 ch @ 64x24x24 ............................................ level 0
    conv 8->16, conv 16->16 = s0 ; pool 2
    conv 16->32, conv 32->32 = s1 ; pool 2 ........................... level 1
    conv 32->64, conv 64->64 = s2 ; pool 2 ........................... level 2
    conv 64->128, conv 128->128 = b .................................. level 3
    up 2, conv 128->64 (+ s2), conv 64->64
    up 2, conv 64->32  (+ s1), conv 32->32
    up 2, conv 32->16  (+ s0), conv 16->16
    head 1x1x1 conv 16->8 (outputs 0..3 used, linear)

All convolutions but the head are followed by ReLU.  Training minimises the
masked mean-square error against time-averaged fields of LBM runs, with Adam on
FP32 master weights; the backward pass is written out layer by layer below.
"""
import math

import numpy as np

from .net import Ops

COARSE = (64, 24, 20)      # x, y, z cells of the target field
PADDED_Z = 24              # z padded to a multiple of 8 for three 2x poolings
IN_CH, HEAD_CH = 8, 8


class Conv:
    def __init__(self, torch, cin, cout, taps, relu, rng, std=None, cin_real=None):
        self.cin, self.cout, self.taps, self.relu = cin, cout, taps, relu
        fan_in = taps * (cin_real or cin)
        std = math.sqrt(2.0 / fan_in) if std is None else std
        w = rng.standard_normal((cout, taps, cin)).astype(np.float32) * std
        if cin_real is not None:
            w[:, :, cin_real:] = 0.0
        dev = "cuda"
        self.w = torch.tensor(w, device=dev)
        self.b = torch.zeros(cout, dtype=torch.float32, device=dev)
        self.wb = torch.empty((cout, taps, cin), dtype=torch.bfloat16, device=dev)
        self.wt = torch.empty((cin, taps, cout), dtype=torch.bfloat16, device=dev)
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.mw, self.vw = torch.zeros_like(self.w), torch.zeros_like(self.w)
        self.mb, self.vb = torch.zeros_like(self.b), torch.zeros_like(self.b)

    def params(self):
        return [self.w, self.b]


class Surrogate:
    """The encoder-decoder with its forward, backward and Adam step."""

    LAYERS = [  # name, cin, cout, taps, relu
        ("e0a", IN_CH, 16, 27, True), ("e0b", 16, 16, 27, True),
        ("e1a", 16, 32, 27, True), ("e1b", 32, 32, 27, True),
        ("e2a", 32, 64, 27, True), ("e2b", 64, 64, 27, True),
        ("e3a", 64, 128, 27, True), ("e3b", 128, 128, 27, True),
        ("d2a", 128, 64, 27, True), ("d2b", 64, 64, 27, True),
        ("d1a", 64, 32, 27, True), ("d1b", 32, 32, 27, True),
        ("d0a", 32, 16, 27, True), ("d0b", 16, 16, 27, True),
        ("head", 16, HEAD_CH, 1, False),
    ]

    def __init__(self, seed=0, ops=None):
        import torch
        self.torch = torch
        self.ops = ops or Ops()
        rng = np.random.default_rng(seed)
        self.L = {}
        for name, cin, cout, taps, relu in self.LAYERS:
            kw = {}
            if name == "e0a":
                kw["cin_real"] = 7
            if name == "head":
                kw["std"] = 0.05
            self.L[name] = Conv(torch, cin, cout, taps, relu, rng, **kw)
        # head outputs 4..7 are padding: zero weights stay zero (their gradient is zero)
        self.L["head"].w[4:] = 0.0
        self.step_count = 0
        self._bufs = {}
        self.refresh_weights()

    # ------------------------------------------------------------------ utils
    def refresh_weights(self):
        for c in self.L.values():
            self.ops.to_bf16(c.w, c.wb)
            self.ops.weight_transpose(c.wb, c.wt)

    def _buf(self, key, shape, dtype):
        t = self._bufs.get(key)
        if t is None or tuple(t.shape) != tuple(shape) or t.dtype != dtype:
            t = self.torch.empty(shape, dtype=dtype, device="cuda")
            self._bufs[key] = t
        return t

    def _act(self, key, B, d, h, w, c):
        return self._buf(key, (B, d, h, w, c), self.torch.bfloat16)

    def _conv(self, name, x, out_key):
        c = self.L[name]
        y = self._act(out_key, *x.shape[:4], c.cout)
        self.ops.conv_forward(x, c.wb, c.b, y, c.relu)
        return y

    # ---------------------------------------------------------------- forward
    def forward(self, x):
        """x: [B, 24, 24, 64, 8] BF16 -> prediction [B, 24, 24, 64, 8] BF16 (channels 0..3)."""
        o, A = self.ops, {}
        B, d, h, w, _ = x.shape
        A["x"] = x
        A["e0a"] = self._conv("e0a", x, "e0a")
        A["s0"] = self._conv("e0b", A["e0a"], "s0")
        A["p0"] = self._act("p0", B, d // 2, h // 2, w // 2, 16); o.pool2(A["s0"], A["p0"])
        A["e1a"] = self._conv("e1a", A["p0"], "e1a")
        A["s1"] = self._conv("e1b", A["e1a"], "s1")
        A["p1"] = self._act("p1", B, d // 4, h // 4, w // 4, 32); o.pool2(A["s1"], A["p1"])
        A["e2a"] = self._conv("e2a", A["p1"], "e2a")
        A["s2"] = self._conv("e2b", A["e2a"], "s2")
        A["p2"] = self._act("p2", B, d // 8, h // 8, w // 8, 64); o.pool2(A["s2"], A["p2"])
        A["e3a"] = self._conv("e3a", A["p2"], "e3a")
        A["bt"] = self._conv("e3b", A["e3a"], "bt")
        A["u2"] = self._act("u2", B, d // 4, h // 4, w // 4, 128); o.up2(A["bt"], A["u2"])
        A["a2"] = self._conv("d2a", A["u2"], "a2")
        A["m2"] = self._act("m2", B, d // 4, h // 4, w // 4, 64); o.add(A["a2"], A["s2"], A["m2"])
        A["q2"] = self._conv("d2b", A["m2"], "q2")
        A["u1"] = self._act("u1", B, d // 2, h // 2, w // 2, 64); o.up2(A["q2"], A["u1"])
        A["a1"] = self._conv("d1a", A["u1"], "a1")
        A["m1"] = self._act("m1", B, d // 2, h // 2, w // 2, 32); o.add(A["a1"], A["s1"], A["m1"])
        A["q1"] = self._conv("d1b", A["m1"], "q1")
        A["u0"] = self._act("u0", B, d, h, w, 32); o.up2(A["q1"], A["u0"])
        A["a0"] = self._conv("d0a", A["u0"], "a0")
        A["m0"] = self._act("m0", B, d, h, w, 16); o.add(A["a0"], A["s0"], A["m0"])
        A["q0"] = self._conv("d0b", A["m0"], "q0")
        A["y"] = self._conv("head", A["q0"], "y")
        self.A = A
        return A["y"]

    # --------------------------------------------------------------- backward
    def _f32(self, key, like, c=None):
        shape = tuple(like.shape[:4]) + ((c if c is not None else like.shape[4]),)
        return self._buf(key, shape, self.torch.float32)

    def _layer_back(self, name, x, gy_bf16, need_dx=True):
        """Weight / bias gradients of layer `name` (input x, output gradient gy) and,
        if asked, the FP32 gradient of its input."""
        c, o = self.L[name], self.ops
        ws = self._buf("ws_" + name, (max(1, o.workspace_bytes(x.shape, c.cin, c.cout, c.taps) // 4),),
                       self.torch.float32)
        o.conv_backward_weight(x, gy_bf16, c.gw, ws, c.taps)
        o.bias_grad(gy_bf16, c.gb)
        if not need_dx:
            return None
        dx = self._f32("dx_" + name, x)
        o.conv_backward_data(gy_bf16, c.wt, dx, c.cin, c.cout, c.taps)
        return dx

    def _mask(self, key, g, g2, act):
        out = self._buf("gb_" + key, tuple(g.shape), self.torch.bfloat16)
        self.ops.grad_to_bf16(g, g2, act, out)
        return out

    def backward(self, dpred):
        A, o = self.A, self.ops
        g = self._layer_back("head", A["q0"], dpred)                       # d q0
        g = self._layer_back("d0b", A["m0"], self._mask("q0", g, None, A["q0"]))   # d m0
        g_m0 = g
        g = self._layer_back("d0a", A["u0"], self._mask("a0", g_m0, None, A["a0"]))  # d u0
        g_q1 = self._f32("g_q1", A["q1"]); o.up2_backward(g, g_q1)
        g = self._layer_back("d1b", A["m1"], self._mask("q1", g_q1, None, A["q1"]))
        g_m1 = g
        g = self._layer_back("d1a", A["u1"], self._mask("a1", g_m1, None, A["a1"]))
        g_q2 = self._f32("g_q2", A["q2"]); o.up2_backward(g, g_q2)
        g = self._layer_back("d2b", A["m2"], self._mask("q2", g_q2, None, A["q2"]))
        g_m2 = g
        g = self._layer_back("d2a", A["u2"], self._mask("a2", g_m2, None, A["a2"]))
        g_bt = self._f32("g_bt", A["bt"]); o.up2_backward(g, g_bt)
        g = self._layer_back("e3b", A["e3a"], self._mask("bt", g_bt, None, A["bt"]))
        g = self._layer_back("e3a", A["p2"], self._mask("e3a", g, None, A["e3a"]))
        g_s2 = self._f32("g_s2", A["s2"]); o.pool2_backward(g, g_s2)
        g = self._layer_back("e2b", A["e2a"], self._mask("s2", g_s2, g_m2, A["s2"]))
        g = self._layer_back("e2a", A["p1"], self._mask("e2a", g, None, A["e2a"]))
        g_s1 = self._f32("g_s1", A["s1"]); o.pool2_backward(g, g_s1)
        g = self._layer_back("e1b", A["e1a"], self._mask("s1", g_s1, g_m1, A["s1"]))
        g = self._layer_back("e1a", A["p0"], self._mask("e1a", g, None, A["e1a"]))
        g_s0 = self._f32("g_s0", A["s0"]); o.pool2_backward(g, g_s0)
        g = self._layer_back("e0b", A["e0a"], self._mask("s0", g_s0, g_m0, A["s0"]))
        self._layer_back("e0a", A["x"], self._mask("e0a", g, None, A["e0a"]), need_dx=False)

    def adam_step(self, lr):
        self.step_count += 1
        for c in self.L.values():
            self.ops.adam(c.w, c.gw, c.mw, c.vw, c.wb, lr, self.step_count)
            self.ops.adam(c.b, c.gb, c.mb, c.vb, None, lr, self.step_count)
            self.ops.weight_transpose(c.wb, c.wt)

    def loss_and_grad(self, target, mask):
        """Masked MSE of the current prediction; returns (loss tensor (device), dpred)."""
        y = self.A["y"]
        dpred = self._buf("dpred", tuple(y.shape), self.torch.bfloat16)
        loss = self.torch.zeros(1, dtype=self.torch.float64, device="cuda")
        norm = float(max(1.0, float(mask.sum())) * 4.0)
        self.ops.mse(y, target, mask, norm, dpred, loss)
        return loss, dpred, norm

    def train_step(self, x, target, mask, lr):
        self.forward(x)
        loss, dpred, norm = self.loss_and_grad(target, mask)
        self.backward(dpred)
        self.adam_step(lr)
        return loss, norm

    # ------------------------------------------------------------ persistence
    def state(self):
        return {f"{n}.{k}": getattr(self.L[n], k).detach().cpu().numpy() for n in self.L for k in ("w", "b")}

    def load_state(self, st):
        for n, c in self.L.items():
            c.w.copy_(self.torch.tensor(np.asarray(st[f"{n}.w"], np.float32), device="cuda"))
            c.b.copy_(self.torch.tensor(np.asarray(st[f"{n}.b"], np.float32), device="cuda"))
        self.refresh_weights()
