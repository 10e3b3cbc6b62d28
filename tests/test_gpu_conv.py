"""The warm start network's operators on the GPU (tensor-core convolutions and
their data / weight gradients, pooling, upsampling, loss, Adam) against the
float64 oracle (oracle/conv_ref.py) on the same BF16-rounded inputs.

Tolerances: FP32 accumulation of BF16 products, so data and weight gradients
(FP32 outputs) agree to 1e-4 of the output's scale; the forward pass rounds its
output to BF16 (relative 2^-8)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ops(wt_lib):
    from windtunnel.net import Ops
    return Ops()


@pytest.fixture(scope="module")
def ref():
    from oracle import conv_ref
    return conv_ref


def bf16_tensor(a):
    return torch.tensor(np.asarray(a, np.float32), device="cuda").to(torch.bfloat16)


def rand(rng, shape, scale=1.0):
    from oracle.conv_ref import bf16_round
    return bf16_round(rng.standard_normal(shape) * scale)


CASES = [  # (batch, d, h, w, cin, cout, taps)
    (2, 6, 5, 7, 16, 24, 27),   # partial M tile, N not a multiple of 16
    (1, 4, 4, 4, 8, 8, 1),      # 1x1x1 head-like
    (1, 8, 8, 8, 128, 128, 27), # K = 3456: 54 K slices through both stages
    (4, 16, 12, 12, 16, 32, 27),  # 9216 voxels: split-K weight gradient
]


@pytest.mark.parametrize("case", CASES)
def test_conv_forward(ops, ref, case):
    b, d, h, w, cin, cout, taps = case
    rng = np.random.default_rng(1)
    x = rand(rng, (b, d, h, w, cin))
    wt = rand(rng, (cout, taps, cin), 1.0 / np.sqrt(taps * cin))
    bias = rng.standard_normal(cout).astype(np.float32) * 0.1
    for relu in (False, True):
        y = torch.empty((b, d, h, w, cout), dtype=torch.bfloat16, device="cuda")
        ops.conv_forward(bf16_tensor(x), bf16_tensor(wt), torch.tensor(bias, device="cuda"), y, relu)
        ops.check()
        got = y.float().cpu().numpy().astype(np.float64)
        want = ref.conv3d(x, wt, bias, relu)
        err = np.abs(got - want).max() / np.abs(want).max()
        assert np.all(np.abs(got - want) <= 2.0 ** -8 * np.abs(want) + 1e-4 * np.abs(want).max()), err


@pytest.mark.parametrize("case", CASES)
def test_conv_backward_data(ops, ref, case):
    b, d, h, w, cin, cout, taps = case
    rng = np.random.default_rng(2)
    dy = rand(rng, (b, d, h, w, cout))
    wt = rand(rng, (cout, taps, cin), 1.0 / np.sqrt(taps * cin))
    w_t = torch.empty((cin, taps, cout), dtype=torch.bfloat16, device="cuda")
    ops.weight_transpose(bf16_tensor(wt), w_t)
    dx = torch.empty((b, d, h, w, cin), dtype=torch.float32, device="cuda")
    ops.conv_backward_data(bf16_tensor(dy), w_t, dx, cin, cout, taps)
    ops.check()
    want = ref.conv3d_backward_data(dy, wt)
    got = dx.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()


@pytest.mark.parametrize("case", CASES)
def test_conv_backward_weight(ops, ref, case):
    b, d, h, w, cin, cout, taps = case
    rng = np.random.default_rng(3)
    x = rand(rng, (b, d, h, w, cin))
    dy = rand(rng, (b, d, h, w, cout))
    dw = torch.empty((cout, taps, cin), dtype=torch.float32, device="cuda")
    ws = torch.empty(ops.workspace_bytes(x.shape, cin, cout, taps) // 4, dtype=torch.float32, device="cuda")
    ops.conv_backward_weight(bf16_tensor(x), bf16_tensor(dy), dw, ws, taps)
    ops.check()
    want = ref.conv3d_backward_weight(x, dy, taps)
    got = dw.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()


def test_adjoint_identity(ops, ref):
    """<conv(x), dy> = <x, dgrad(dy)> through the GPU kernels (FP32 outputs of the
    linear maps, no bias, no activation)."""
    b, d, h, w, cin, cout, taps = 1, 6, 6, 6, 16, 16, 27
    rng = np.random.default_rng(4)
    x, dy = rand(rng, (b, d, h, w, cin)), rand(rng, (b, d, h, w, cout))
    wt = rand(rng, (cout, taps, cin), 0.1)
    w_t = torch.empty((cin, taps, cout), dtype=torch.bfloat16, device="cuda")
    ops.weight_transpose(bf16_tensor(wt), w_t)
    dx = torch.empty((b, d, h, w, cin), dtype=torch.float32, device="cuda")
    ops.conv_backward_data(bf16_tensor(dy), w_t, dx, cin, cout, taps)
    lhs = float((ref.conv3d(x, wt) * dy).sum())
    rhs = float((x * dx.cpu().numpy()).sum())
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + 1.0)


def test_elementwise_operators(ops, ref):
    rng = np.random.default_rng(5)
    x = rand(rng, (2, 4, 6, 8, 16))
    xt = bf16_tensor(x)
    y = torch.empty((2, 2, 3, 4, 16), dtype=torch.bfloat16, device="cuda")
    ops.pool2(xt, y)
    assert np.allclose(y.float().cpu().numpy(), ref.pool2(x), rtol=2 ** -8, atol=1e-6)
    g = rng.standard_normal((2, 2, 3, 4, 16)).astype(np.float32)
    dx = torch.empty(x.shape, dtype=torch.float32, device="cuda")
    ops.pool2_backward(torch.tensor(g, device="cuda"), dx)
    assert np.allclose(dx.cpu().numpy(), ref.pool2_backward(g), rtol=1e-6)
    up = torch.empty((2, 8, 12, 16, 16), dtype=torch.bfloat16, device="cuda")
    ops.up2(xt, up)
    assert np.array_equal(up.float().cpu().numpy(), ref.up2(x))
    gu = rng.standard_normal((2, 8, 12, 16, 16)).astype(np.float32)
    du = torch.empty(x.shape, dtype=torch.float32, device="cuda")
    ops.up2_backward(torch.tensor(gu, device="cuda"), du)
    assert np.allclose(du.cpu().numpy(), ref.up2_backward(gu), rtol=1e-5, atol=1e-5)
    s = torch.empty_like(xt)
    ops.add(xt, xt, s)
    assert np.array_equal(s.float().cpu().numpy(), 2 * x)
    g1 = rng.standard_normal(x.shape).astype(np.float32)
    g2 = rng.standard_normal(x.shape).astype(np.float32)
    out = torch.empty_like(xt)
    ops.grad_to_bf16(torch.tensor(g1, device="cuda"), torch.tensor(g2, device="cuda"), xt, out)
    assert np.allclose(out.float().cpu().numpy(), ref.bf16_round((g1 + g2) * (x > 0)), rtol=0, atol=0)
    db = torch.empty(16, dtype=torch.float32, device="cuda")
    ops.bias_grad(xt, db)
    assert np.allclose(db.cpu().numpy(), x.reshape(-1, 16).sum(0), rtol=1e-5, atol=1e-4)


def test_mse_and_adam(ops, ref):
    rng = np.random.default_rng(6)
    rows = 1000
    pred = rand(rng, (rows, 8))
    target = rng.standard_normal((rows, 4)).astype(np.float32)
    mask = (rng.random(rows) > 0.3).astype(np.float32)
    dpred = torch.empty((rows, 8), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    ops.mse(bf16_tensor(pred), torch.tensor(target, device="cuda"), torch.tensor(mask, device="cuda"), 123.0, dpred,
            loss)
    e = pred[:, :4] - target
    assert np.isclose(float(loss.cpu()), float((mask[:, None] * e * e).sum()), rtol=1e-5)
    want = np.zeros((rows, 8))
    want[:, :4] = 2 * mask[:, None] * e / 123.0
    assert np.allclose(dpred.float().cpu().numpy(), ref.bf16_round(want), rtol=2 ** -7, atol=1e-7)
    # Adam, two steps against the textbook update in float64
    n = 257
    p0 = rng.standard_normal(n)
    gs = [rng.standard_normal(n), rng.standard_normal(n)]
    p = torch.tensor(p0, dtype=torch.float32, device="cuda")
    m = torch.zeros(n, device="cuda")
    v = torch.zeros(n, device="cuda")
    pb = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    pw, mw, vw = p0.astype(np.float32).astype(np.float64), np.zeros(n), np.zeros(n)
    for k, g in enumerate(gs, start=1):
        ops.adam(p, torch.tensor(g, dtype=torch.float32, device="cuda"), m, v, pb, 1e-2, k)
        g32 = g.astype(np.float32).astype(np.float64)
        mw = 0.9 * mw + 0.1 * g32
        vw = 0.999 * vw + 0.001 * g32 * g32
        pw = pw - 1e-2 * (mw / (1 - 0.9 ** k)) / (np.sqrt(vw / (1 - 0.999 ** k)) + 1e-8)
    assert np.allclose(p.cpu().numpy(), pw, rtol=1e-5, atol=1e-6)
    assert np.array_equal(pb.float().cpu().numpy(), ref.bf16_round(p.cpu().numpy()))


def test_stage_wait_expiry_is_reported(ops, ref):
    """The pipeline's bounded stage wait made to run out (a poll budget of 0):
    every block leaves its K loop at the third slice, waits with the full limit
    for the MMAs it issued, frees its tensor memory and raises the flag that
    wt_net_check reports; the output is left unwritten.  The next launch with the
    normal budget succeeds and matches the oracle."""
    from windtunnel import WindTunnelError
    rng = np.random.default_rng(5)
    b, d, h, w, cin, cout, taps = 1, 6, 6, 8, 16, 32, 27  # K = 432: 7 K slices
    x = rand(rng, (b, d, h, w, cin))
    wt = rand(rng, (cout, taps, cin), 1.0 / np.sqrt(taps * cin))
    xs, ws = bf16_tensor(x), bf16_tensor(wt)
    y = torch.full((b, d, h, w, cout), 7.0, dtype=torch.bfloat16, device="cuda")
    ops.check()
    prev = ops.lib.wt_net_set_stage_wait_limit(0)
    try:
        ops.conv_forward(xs, ws, None, y, False)
        with pytest.raises(WindTunnelError, match="wait expired"):
            ops.check()
    finally:
        ops.lib.wt_net_set_stage_wait_limit(prev)
    assert bool((y.float() == 7.0).all())  # no block wrote a partial result
    ops.conv_forward(xs, ws, None, y, False)
    ops.check()
    want = ref.conv3d(x, wt)
    got = y.float().cpu().numpy().astype(np.float64)
    assert np.all(np.abs(got - want) <= 2.0 ** -8 * np.abs(want) + 1e-4 * np.abs(want).max())
