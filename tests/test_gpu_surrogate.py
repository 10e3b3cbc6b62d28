"""The warm-start network's backward pass end to end: every layer's weight and
bias gradient from the GPU (BF16 activations, tensor-core convolutions)
against a float64 restatement of the same network built from the oracle's
operators (oracle/conv_ref.py) with the same weights and input, rounding to
BF16 where the GPU stores BF16 (activations, the gradients fed to the
convolutions).  What remains is FP32 versus float64 accumulation, which flips
the odd BF16 rounding; the check is the relative error of each gradient (2 %)
and the cosine of the angle to the oracle's (0.9995)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def oracle_network(W, B, x, target, mask):
    from oracle import conv_ref as R
    relu = lambda a: np.maximum(a, 0.0)
    q = R.bf16_round
    A = {}

    def conv(name, inp, act=True):
        y = R.conv3d(inp, W[name], B[name])
        return q(relu(y) if act else y)

    A["x"] = x
    A["e0a"] = conv("e0a", x); A["s0"] = conv("e0b", A["e0a"]); A["p0"] = q(R.pool2(A["s0"]))
    A["e1a"] = conv("e1a", A["p0"]); A["s1"] = conv("e1b", A["e1a"]); A["p1"] = q(R.pool2(A["s1"]))
    A["e2a"] = conv("e2a", A["p1"]); A["s2"] = conv("e2b", A["e2a"]); A["p2"] = q(R.pool2(A["s2"]))
    A["e3a"] = conv("e3a", A["p2"]); A["bt"] = conv("e3b", A["e3a"])
    A["u2"] = R.up2(A["bt"]); A["a2"] = conv("d2a", A["u2"]); A["m2"] = q(A["a2"] + A["s2"]); A["q2"] = conv("d2b", A["m2"])
    A["u1"] = R.up2(A["q2"]); A["a1"] = conv("d1a", A["u1"]); A["m1"] = q(A["a1"] + A["s1"]); A["q1"] = conv("d1b", A["m1"])
    A["u0"] = R.up2(A["q1"]); A["a0"] = conv("d0a", A["u0"]); A["m0"] = q(A["a0"] + A["s0"]); A["q0"] = conv("d0b", A["m0"])
    y = conv("head", A["q0"], act=False)
    norm = max(1.0, mask.sum()) * 4.0
    dy = np.zeros_like(y)
    dy[..., :4] = q(2.0 * mask[..., None] * (y[..., :4] - target) / norm)
    G = {}

    def back(name, inp, out, g, act=True):
        gy = q(g * (out > 0)) if act else g
        G[name] = (R.conv3d_backward_weight(inp, gy, W[name].shape[1]), gy.reshape(-1, gy.shape[-1]).sum(0))
        return R.conv3d_backward_data(gy, W[name])

    g = back("head", A["q0"], y, dy, act=False)
    gm0 = back("d0b", A["m0"], A["q0"], g)
    g = back("d0a", A["u0"], A["a0"], gm0); g = R.up2_backward(g)
    gm1 = back("d1b", A["m1"], A["q1"], g)
    g = back("d1a", A["u1"], A["a1"], gm1); g = R.up2_backward(g)
    gm2 = back("d2b", A["m2"], A["q2"], g)
    g = back("d2a", A["u2"], A["a2"], gm2); g = R.up2_backward(g)
    g = back("e3b", A["e3a"], A["bt"], g)
    g = back("e3a", A["p2"], A["e3a"], g); g = R.pool2_backward(g) + gm2
    g = back("e2b", A["e2a"], A["s2"], g)
    g = back("e2a", A["p1"], A["e2a"], g); g = R.pool2_backward(g) + gm1
    g = back("e1b", A["e1a"], A["s1"], g)
    g = back("e1a", A["p0"], A["e1a"], g); g = R.pool2_backward(g) + gm0
    g = back("e0b", A["e0a"], A["s0"], g)
    back("e0a", A["x"], A["e0a"], g)
    return G


def test_network_gradients_match_oracle(wt_lib):
    from oracle.conv_ref import bf16_round
    from windtunnel.surrogate import Surrogate
    model = Surrogate(seed=3)
    rng = np.random.default_rng(0)
    for c in model.L.values():  # nonzero biases so every bias path is exercised
        c.b.copy_(torch.tensor(rng.standard_normal(c.cout).astype(np.float32) * 0.05, device="cuda"))
    model.refresh_weights()
    shape = (2, 8, 8, 16)
    x = bf16_round(rng.standard_normal(shape + (8,)) * 0.5)
    x[..., 7] = 0.0
    target = rng.standard_normal(shape + (4,)).astype(np.float32)
    mask = (rng.random(shape) > 0.2).astype(np.float32)
    xt = torch.tensor(x.astype(np.float32), device="cuda").to(torch.bfloat16)
    model.forward(xt)
    _, dpred, _ = model.loss_and_grad(torch.tensor(target, device="cuda"), torch.tensor(mask, device="cuda"))
    model.backward(dpred)
    model.ops.check()
    W = {n: bf16_round(c.w.cpu().numpy()) for n, c in model.L.items()}
    B = {n: c.b.cpu().numpy().astype(np.float64) for n, c in model.L.items()}
    G = oracle_network(W, B, x, target.astype(np.float64), mask.astype(np.float64))
    for name, c in model.L.items():
        gw, gb = c.gw.cpu().numpy().astype(np.float64), c.gb.cpu().numpy().astype(np.float64)
        rw, rb = G[name]
        if name == "e0a":
            gw, rw = gw[:, :, :7], rw[:, :, :7]  # channel 7 of the input is zero padding
        if name == "head":
            gw, rw, gb, rb = gw[:4], rw[:4], gb[:4], rb[:4]
        for got, want in ((gw, rw), (gb, rb)):
            nrm = np.linalg.norm(want)
            assert nrm > 0, name
            rel = np.linalg.norm(got - want) / nrm
            cos = float((got * want).sum() / (np.linalg.norm(got) * nrm))
            assert rel < 0.02 and cos > 0.9995, (name, rel, cos)
