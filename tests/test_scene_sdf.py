"""The scene signed-distance field at arbitrary points, bit for bit, in its
three implementations: the device code (wt_scene.cuh, built for the host by
oracle/shade_host_model.cpp), the oracle's restatement (oracle/wt_oracle.hpp)
and the reference's own SDF chunk translated to C++ (render module).  Rays and
shadow probes sample the field everywhere (both sides of the symmetry plane,
below the ground, inside bodies), not only at cell centres where the
voxelizer's thresholded flags are checked.  Also the whole RENDER fragment
shader of the device code against the render fixture."""
import ctypes
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from helpers import golden_shapes, same_half, shade_host_model

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


@pytest.fixture(scope="module")
def hm():
    L = shade_host_model()
    if L is None:
        pytest.skip("the CUDA headers are missing")
    return L


def points(seed, n=150000):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-1.5, 7.0, n), rng.uniform(-0.4, 2.4, n), rng.uniform(-1.6, 1.6, n)],
                    axis=1).astype(np.float32)


def device_sdf(L, shape, pts):
    out = np.zeros((len(pts), 2), np.float32)
    L.wthm_scene_sdf(ctypes.addressof(shape), pts.ctypes.data, len(pts), out.ctypes.data)
    return out


def oracle_sdf(oracle_mod, shape, pts):
    L = oracle_mod.oracle_lib()
    L.wto_scene_sdf.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    out = np.zeros((len(pts), 2), np.float32)
    L.wto_scene_sdf(ctypes.addressof(shape), pts.ctypes.data, len(pts), out.ctypes.data)
    return out


def test_sdf_bitexact_against_reference(hm, oracle_mod, golden):
    if oracle_mod.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    _, man = golden
    for k, (name, shape) in enumerate(sorted(golden_shapes(man).items())):
        pts = points(k)
        ref = oracle_mod.ref_scene_sdf(shape, pts)
        for impl, got in (("device", device_sdf(hm, shape, pts)), ("oracle", oracle_sdf(oracle_mod, shape, pts))):
            bad = np.nonzero(np.any(got.view(np.uint32) != ref.view(np.uint32), axis=1))[0]
            assert len(bad) == 0, f"{name} {impl}: {len(bad)} points differ, e.g. {pts[bad[:3]].tolist()}"


def test_device_and_oracle_sdf_agree(hm, oracle_mod, golden):
    """Where the reference is absent: the device code and the oracle agree."""
    _, man = golden
    for k, (name, shape) in enumerate(sorted(golden_shapes(man).items())):
        pts = points(100 + k, 50000)
        assert np.array_equal(device_sdf(hm, shape, pts).view(np.uint32), oracle_sdf(oracle_mod, shape, pts).view(np.uint32)), name


def test_device_render_pixel_matches_fixture(hm):
    import make_consumers as mc
    import make_render as mr
    from windtunnel import render as R
    c = {k: v for k, v in np.load(os.path.join(ROOT, "tests", "golden", "consumers.npz")).items()}
    z = np.load(os.path.join(ROOT, "tests", "golden", "render.npz"))
    shape, seqs = mr.sequences(c)
    view = mc.view()
    dims = np.array(mc.DIMS, np.uint32)
    org = np.array(mc.ORIGIN, np.float32)
    for name, frames in seqs:
        st = R.FrameState()
        for k, f in enumerate(frames):
            u = mr.frame_uniforms(st, f)
            from oracle import pyoracle
            pyoracle.shade_model_set_car(f.get("car"))
            w, h = mr.frame_size(f)
            out = pyoracle.shade_model_render(mr.frame_shape(shape, f), u.cam, f["look"], view, dims, org, mc.H,
                                              c["fields"], c["temps"], w, h, threads=4)
            ref = z[f"{name}_{k}_scene"]
            bad = np.argwhere(np.any(~same_half(out, ref), axis=-1))
            assert len(bad) == 0, f"{name}_{k}: {len(bad)} pixels differ, first {bad[:4].tolist()}"
