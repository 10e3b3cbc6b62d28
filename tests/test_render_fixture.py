"""The render fixture (tests/golden/render.npz) against the reference's own
render shaders: where the translated reference is built (the build
container), rerunning the frames reproduces every target bit for bit;
everywhere, the fixture is self-consistent.  Also the host-side camera and
jitter helpers against camera.ts / engine.ts semantics."""
import math
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from helpers import same_half

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))

TARGETS = ("scene", "hist", "glow", "bloom", "out")


def fixture():
    return np.load(os.path.join(GOLDEN, "render.npz"))


def test_fixture_is_consistent():
    import make_render as mr
    z = fixture()
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    assert keys == ["cube_0", "empty_0", "hero_0", "hero_1", "slice-x_0", "slice-y_0", "slice-z_0", "sphere_0",
                    "surface_0", "tiny_0", "tiny_1", "w17_0", "wing_0"]
    for k in keys:
        sc, out = z[k + "_scene"].astype(np.float32), z[k + "_out"]
        w, h = (17, 9) if k.startswith("tiny") else (mr.W, mr.H)
        assert sc.shape == (h, w, 4) and out.shape == (h, w, 4) and out.dtype == np.uint8
        assert z[k + "_bloom"].shape == (h // 2, w // 2, 4)
        # colours are finite except where the reference's normal estimate degenerates (four equal
        # distance taps on a quantized texture give normalize(0): NaN, as in the shader itself)
        assert np.isfinite(sc[..., 3]).all() and (sc[..., 3] > 0).all() and (sc[..., 3] <= 6e4).all()
        assert (~np.isfinite(sc[..., :3])).any(axis=-1).mean() < 1e-3
        assert (out[..., 3] == 255).all()
        assert (z[k + "_glow"].astype(np.float32) >= 0).all()
    # the car is in view, the glow draws hit pixels, history reprojection changed the second frame
    assert (z["hero_0_scene"][..., 3].astype(np.float32) < 20).sum() > 1000
    assert (z["hero_0_glow"][..., 3] > 0).sum() > 500 and (z["slice-z_0_glow"][..., 3] > 0).sum() > 50
    assert not np.array_equal(z["hero_1_hist"], z["hero_1_scene"])


def test_reference_reproduces_fixture():
    from oracle import pyoracle
    if pyoracle.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    import make_consumers as mc
    import make_render as mr
    from windtunnel import render as R
    z = fixture()
    c = np.load(os.path.join(GOLDEN, "consumers.npz"))
    shape, seqs = mr.sequences(c)
    for name, frames in seqs:
        st = R.FrameState()
        w, h = mr.frame_size(frames[0])
        hw, hh = max(1, w // 2), max(1, h // 2)
        hist = [np.zeros((h, w, 4), np.float32) for _ in range(2)]
        for k, f in enumerate(frames):
            u = mr.frame_uniforms(st, f)
            pyoracle.ref_set_car(f.get("car"))
            scene = pyoracle.ref_render_scene(mc.DIMS, mc.ORIGIN, mc.H, c["fields"], c["temps"],
                                              mr.frame_shape(shape, f), u.cam, f["look"], mc.view(), w, h)
            hist[u.cur] = pyoracle.ref_taa(scene, hist[1 - u.cur], u.taa)
            glow = pyoracle.ref_glow(scene, f.get("parts"), u.pdraw, f.get("lines"), u.sdraw)
            bb = pyoracle.ref_blur(pyoracle.ref_blur(glow, (1.0, 0.0), 3.0, 1.0, hw, hh), (0.0, 1.0), 1.5, 1.0, hw, hh)
            out = pyoracle.ref_present(hist[u.cur], glow, bb, u.post)
            key = f"{name}_{k}"
            for t, v in zip(TARGETS, (scene, hist[u.cur], glow, bb)):
                assert same_half(v, z[f"{key}_{t}"]).all(), (key, t)
            assert np.array_equal(out, z[key + "_out"]), key


def test_orbit_camera_and_jitter():
    from windtunnel import render as R
    cam = R.orbit_camera((2.75, 0.42, 0.0), 2.3, 0.3, 7.6, 16 / 9)
    assert abs(math.dist(cam.pos, (2.75, 0.42, 0.0)) - 7.6) < 1e-12
    for v in (cam.fwd, cam.right, cam.up):
        assert abs(math.hypot(*v) - 1.0) < 1e-12
    assert abs(sum(a * b for a, b in zip(cam.fwd, cam.right))) < 1e-12
    # the orbit target projects to the centre of the view, in front of the camera
    m = cam.view_proj.reshape(4, 4).T.astype(np.float64)
    clip = m @ np.array([2.75, 0.42, 0.0, 1.0])
    assert clip[3] > 0 and abs(clip[0] / clip[3]) < 1e-5 and abs(clip[1] / clip[3]) < 1e-5
    assert 0.0 < clip[2] / clip[3] < 1.0
    assert [R.halton(i, 2) for i in (1, 2, 3, 4)] == [0.5, 0.25, 0.75, 0.125]
    assert abs(R.halton(1, 3) - 1 / 3) < 1e-15 and abs(R.halton(5, 3) - 7 / 9) < 1e-15
    st = R.FrameState()
    a = st.next(cam, (128, 72))
    b = st.next(cam, (128, 72))
    assert (a.cur, b.cur) == (1, 0) and a.taa.blend == 1.0 and abs(b.taa.blend - 0.1) < 1e-7
    assert abs(a.cam.jitter[0] - (R.halton(2, 2) - 0.5) * 2 / 128) < 1e-7


def _viewer_without_gpu(shape_params, kmh=250.0, flow_mode=None):
    """A Viewer's host-side state over a stand-in engine (no device calls)."""
    from types import SimpleNamespace
    from windtunnel.viewer import FlowMode, Viewer, ViewParams
    v = object.__new__(Viewer)
    v.engine = SimpleNamespace(shape_params=shape_params, h=10.4 / 232, u_lb=0.0925, dims=(232, 68, 52))
    v.view = ViewParams(kmh=kmh, flow_mode=FlowMode.Streamlines if flow_mode is None else flow_mode)
    v.flow_time = 0.25
    return v


def test_viewer_uniforms_follow_the_engine():
    from windtunnel.engine import ORIGIN_X, ShapeKind, ShapeParams
    from windtunnel.viewer import MAX_LINES, STREAM_STEPS, FlowMode
    f1 = ShapeParams(kind=ShapeKind.F1, rideH=0.10)
    v = _viewer_without_gpu(f1)
    s = v.stream_params()                                    # streamConfig (engine.ts:558-570)
    assert (s.lines, s.rows, s.cols, s.seed_mode, s.steps) == (90, 18, 5, 0, STREAM_STEPS)
    assert list(s.seed_min) == pytest.approx([-1.2, 0.05, 0.03]) and list(s.seed_max) == pytest.approx([0, 1.3, 0.95])
    assert abs(s.step_len - 0.03) < 1e-7 and abs(s.time - 0.25) < 1e-7
    vx = _viewer_without_gpu(f1, flow_mode=FlowMode.Vortices).stream_params()
    assert (vx.seed_mode, vx.emitters, vx.per_emitter, vx.lines) == (1, 4, MAX_LINES // 4, MAX_LINES // 4 * 4)
    yw, yr = 0.19 + 0.10 * 0.45, 0.10 + 0.8
    assert list(vx.emitter[0]) == pytest.approx([0.52, yw + 0.2, 0.926, 0.06])
    assert list(vx.emitter[2]) == pytest.approx([5.36, yr + 0.26, 0.494, 0.06])
    lo, hi, rows, cols = v.spawn_region()                    # spawnRegion (engine.ts:731-737)
    assert lo == pytest.approx((ORIGIN_X + 2 * 10.4 / 232, 0.04, 0.0)) and (rows, cols) == (12, 7)
    assert hi == pytest.approx((0.0, 0.10 + 1.34 + 0.25, 0.98 + 0.25))
    u = v.view_uniform()                                     # viewUniform (engine.ts:503-518)
    assert (u.t_min, u.t_max, u.cp_min) == pytest.approx((0.0, 220.0, -1.1))
    cold = _viewer_without_gpu(ShapeParams(kind=ShapeKind.F1, heatBrakes=False, heatEngine=False, heatRad=False))
    stag = 0.5 * (250 / 3.6) ** 2 / 1005
    assert (cold.view_uniform().t_min, cold.view_uniform().t_max) == pytest.approx((-stag * 1.4, stag * 1.05))
    assert _viewer_without_gpu(f1, kmh=500).visual_flow_rate() == 1.6
    assert _viewer_without_gpu(f1, kmh=50).visual_flow_rate() == 0.35


def test_write_png_roundtrip(tmp_path):
    import struct
    import zlib
    from windtunnel.viewer import write_png
    img = (np.arange(5 * 7 * 4) % 251).astype(np.uint8).reshape(5, 7, 4)
    p = tmp_path / "a.png"
    write_png(str(p), img)
    b = p.read_bytes()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", b[16:24])
    assert (w, h) == (7, 5)
    i = b.index(b"IDAT")
    n = struct.unpack(">I", b[i - 4:i])[0]
    raw = zlib.decompress(b[i + 4:i + 4 + n])
    rows = [raw[r * (7 * 4 + 1) + 1:(r + 1) * (7 * 4 + 1)] for r in range(5)]
    assert np.array_equal(np.frombuffer(b"".join(rows), np.uint8).reshape(5, 7, 4), img)
