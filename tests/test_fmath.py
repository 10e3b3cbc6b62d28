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
