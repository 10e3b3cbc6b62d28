"""The project's sin/cos/atan (wt_fmath.h) against double-precision references:
a few ulp over the argument ranges the scenes use, and exact symmetries."""
import ctypes

import numpy as np


def run(oracle_mod, which, x):
    L = oracle_mod.oracle_lib()
    L.wto_fmath.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x)
    L.wto_fmath(which, x.ctypes.data, y.ctypes.data, x.size)
    return y


def ulps(got, want):
    want32 = want.astype(np.float32)
    spacing = np.spacing(np.abs(want32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - want) / spacing


def test_sin_cos_accuracy(oracle_mod):
    x = np.linspace(-8.0, 8.0, 400001, dtype=np.float32)
    xs = x.astype(np.float64)
    s, c = run(oracle_mod, 0, x), run(oracle_mod, 1, x)
    mask = np.abs(np.sin(xs)) > 1e-3
    assert ulps(s[mask], np.sin(xs[mask])).max() <= 2.0
    mask = np.abs(np.cos(xs)) > 1e-3
    assert ulps(c[mask], np.cos(xs[mask])).max() <= 2.0
    assert np.abs(s.astype(np.float64) - np.sin(xs)).max() < 2e-7
    np.testing.assert_array_equal(run(oracle_mod, 0, -x), -s)
    np.testing.assert_array_equal(run(oracle_mod, 1, -x), c)


def test_atan_accuracy(oracle_mod):
    x = np.concatenate([np.linspace(-60, 60, 400001), np.geomspace(1e-6, 1e6, 20001)]).astype(np.float32)
    a = run(oracle_mod, 2, x)
    assert ulps(a, np.arctan(x.astype(np.float64))).max() <= 3.0
    np.testing.assert_array_equal(run(oracle_mod, 2, -x), -a)
    assert run(oracle_mod, 2, np.array([np.inf], np.float32))[0] == np.float32(np.pi / 2)


def run2(oracle_mod, which, x, y):
    L = oracle_mod.oracle_lib()
    L.wto_fmath2.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(x)
    L.wto_fmath2(which, x.ctypes.data, y.ctypes.data, out.ctypes.data, x.size)
    return out


def test_exp_exp2_log2_accuracy(oracle_mod):
    x = np.concatenate([np.linspace(-80, 80, 400001), np.linspace(-1, 1, 100001)]).astype(np.float32)
    xs = x.astype(np.float64)
    assert ulps(run(oracle_mod, 3, x), np.exp(xs)).max() <= 2.0
    x2 = np.linspace(-120, 120, 400001).astype(np.float32)
    assert ulps(run(oracle_mod, 4, x2), np.exp2(x2.astype(np.float64))).max() <= 2.0
    pos = np.concatenate([np.geomspace(1e-30, 1e30, 400001), np.linspace(0.5, 2.0, 100001),
                          np.array([1.4e-45, 1e-40, 3.4e38])]).astype(np.float32)
    lg = run(oracle_mod, 5, pos)
    want = np.log2(pos.astype(np.float64))
    far = np.abs(want) > 1.0
    assert ulps(lg[far], want[far]).max() <= 3.0
    assert np.abs(lg[~far] - want[~far]).max() < 2.0 ** -21  # the WGSL bound inside [0.5, 2]
    # exact points and limits
    assert run(oracle_mod, 4, np.array([0, 1, -1, 10, -149], np.float32)).tolist() == [1.0, 2.0, 0.5, 1024.0, 2.0 ** -149]
    assert run(oracle_mod, 5, np.array([1, 2, 0.5, 1024], np.float32)).tolist() == [0.0, 1.0, -1.0, 10.0]
    sp = run(oracle_mod, 3, np.array([np.inf, -np.inf, 100, -200, np.nan], np.float32))
    assert sp[0] == np.inf and sp[1] == 0 and sp[2] == np.inf and sp[3] == 0 and np.isnan(sp[4])
    sl = run(oracle_mod, 5, np.array([0, -1, np.inf, np.nan], np.float32))
    assert sl[0] == -np.inf and np.isnan(sl[1]) and sl[2] == np.inf and np.isnan(sl[3])


def test_pow_atan2(oracle_mod):
    rng = np.random.default_rng(3)
    # pow over the shading ranges: bases in [0, 1] (colours, cosines), exponents 1/2.2 ... 900
    b = rng.uniform(0.0, 1.0, 200000).astype(np.float32)
    e = np.exp(rng.uniform(np.log(0.3), np.log(900.0), b.size)).astype(np.float32)
    got = run2(oracle_mod, 0, b, e)
    want = np.power(b.astype(np.float64), e.astype(np.float64))
    ok = want > 1e-30
    # exp2(y log2 x): the error grows with |y log2 x| as the WGSL definition allows
    rel = np.abs(got[ok] - want[ok]) / want[ok]
    bound = 2.0 ** -22 * (4.0 + 2.0 * np.abs(e[ok] * np.log2(b[ok].astype(np.float64))))
    assert (rel <= bound).all()
    assert run2(oracle_mod, 0, np.array([0, 0, 1, 4], np.float32), np.array([14, 0.45, 7, 0.5], np.float32)).tolist() == [0.0, 0.0, 1.0, 2.0]
    y = rng.uniform(-3, 3, 200000).astype(np.float32)
    x = rng.uniform(-3, 3, 200000).astype(np.float32)
    a = run2(oracle_mod, 1, y, x)
    assert np.abs(a - np.arctan2(y.astype(np.float64), x.astype(np.float64))).max() < 1e-6
    q = run2(oracle_mod, 1, np.array([1, -1, 0, 1, -1], np.float32), np.array([0, 0, 0, -1, -1], np.float32))
    np.testing.assert_allclose(q, [np.pi / 2, -np.pi / 2, 0.0, 3 * np.pi / 4, -3 * np.pi / 4], rtol=1e-7)
