"""The network oracle (oracle/conv_ref.py) pinned by properties on the CPU: its
data and weight gradients are the exact adjoints / derivatives of its forward
convolution, pooling and upsampling are adjoint pairs, and its BF16 rounding
matches torch's."""
import numpy as np
import pytest

from oracle import conv_ref as R


@pytest.mark.parametrize("taps", [27, 1])
def test_gradients_are_adjoints(taps):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, 4, 3, 5, 8))
    dy = rng.standard_normal((2, 4, 3, 5, 16))
    w = rng.standard_normal((16, taps, 8))
    lhs = (R.conv3d(x, w) * dy).sum()
    assert np.isclose(lhs, (x * R.conv3d_backward_data(dy, w)).sum(), rtol=1e-12)
    assert np.isclose(lhs, (w * R.conv3d_backward_weight(x, dy, taps)).sum(), rtol=1e-12)


def test_weight_gradient_finite_difference():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((1, 3, 3, 3, 8))
    w = rng.standard_normal((8, 27, 8))
    dy = rng.standard_normal((1, 3, 3, 3, 8))
    g = R.conv3d_backward_weight(x, dy, 27)
    e = np.zeros_like(w)
    e[3, 13, 5] = 1e-6
    fd = ((R.conv3d(x, w + e) - R.conv3d(x, w - e)) * dy).sum() / 2e-6
    assert np.isclose(fd, g[3, 13, 5], rtol=1e-6, atol=1e-8)


def test_pool_and_upsample_adjoints():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((1, 4, 6, 8, 3))
    y = rng.standard_normal((1, 2, 3, 4, 3))
    assert np.isclose((R.pool2(x) * y).sum(), (x * R.pool2_backward(y)).sum(), rtol=1e-12)
    assert np.isclose((R.up2(y) * x).sum(), (y * R.up2_backward(x)).sum(), rtol=1e-12)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a = (rng.standard_normal(10000) * np.exp(rng.uniform(-20, 20, 10000))).astype(np.float32)
    want = torch.tensor(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(R.bf16_round(a).astype(np.float32), want)
