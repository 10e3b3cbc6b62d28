"""The render passes on the GPU (wt_render_* through the C ABI) bit for bit
against the fixture generated from the reference's own render shaders
(tests/golden/render.npz, tests/golden/make_render.py): scene ray march,
TAA resolve, glow rasterization, bloom and present, frame by frame over the
consumer fixture's flow."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from helpers import same_half

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)


@pytest.fixture(scope="module")
def setup(wt_lib):
    import make_consumers as mc
    import make_render as mr
    from windtunnel import AeroEngine
    c = np.load(os.path.join(GOLDEN, "consumers.npz"))
    z = np.load(os.path.join(GOLDEN, "render.npz"))
    e = AeroEngine(dims=mc.DIMS, origin=mc.ORIGIN, h=mc.H)
    shape, seqs = mr.sequences(c)
    e.set_shape_raw(shape)
    e.write_state(fields=c["fields"], temps=c["temps"])
    yield mc, mr, z, e, seqs, shape, c
    e.close()


def test_render_frames_bitexact(setup):
    from windtunnel import render as R
    mc, mr, z, e, seqs, shape, c = setup
    view = mc.view()
    for name, frames in seqs:
        if "car" in frames[0]:
            e.set_car_model(frames[0]["car"])
        e.set_shape_raw(mr.frame_shape(shape, frames[0]))  # the renderer draws the context's shape
        e.write_state(fields=c["fields"], temps=c["temps"])
        r = R.Renderer(e, *mr.frame_size(frames[0]))
        try:
            check_sequence(r, name, frames, z, view)
        finally:
            r.close()


def check_sequence(r, name, frames, z, view):
    from windtunnel import render as R
    for k, f in enumerate(frames):
        u = r.frame(f["cam"], f["look"], view, parts=f.get("parts"), color_mode=f.get("color_mode", 0),
                    smoke=f.get("smoke", True), lines=f.get("lines"), flow_time=f.get("flow_time", 0.0),
                    vortices=f.get("vortices", False))
        key = f"{name}_{k}"
        got = {"scene": r.read(R.TARGET_SCENE), "hist": r.read(R.TARGET_HIST0 + u.cur),
               "glow": r.read(R.TARGET_GLOW), "bloom": r.read(R.TARGET_BLOOM_B)}
        for t, v in got.items():
            ref = z[f"{key}_{t}"]
            bad = np.argwhere(np.any(~same_half(v, ref), axis=-1))
            assert len(bad) == 0, f"{key} {t}: {len(bad)} texels differ, first {bad[:4].tolist()}"
        assert np.array_equal(r.read(R.TARGET_OUTPUT), z[key + "_out"]), key


def test_render_full_size_deterministic(setup):
    """1280x720 (the headless check's size): finite targets, identical on a rerun."""
    from windtunnel import render as R
    mc, mr, z, e, seqs, shape, c = setup
    e.set_shape_raw(shape)
    e.write_state(fields=c["fields"], temps=c["temps"])
    f = seqs[0][1][0]
    cam = R.orbit_camera((2.75, 0.42, 0.0), 2.3, 0.3, 7.6, 1280 / 720)
    outs = []
    for _ in range(2):
        r = R.Renderer(e, 1280, 720)
        r.frame(cam, f["look"], mc.view(), lines=f["lines"], flow_time=0.7)
        sc = r.read(R.TARGET_SCENE).astype(np.float32)
        assert np.isfinite(sc).all()
        outs.append((r.read(R.TARGET_OUTPUT), r.read(R.TARGET_GLOW)))
        r.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][0][..., :3].mean() > 10


def test_render_errors(setup):
    from windtunnel import WindTunnelError
    from windtunnel import render as R
    mc, mr, z, e, seqs, shape, c = setup
    r = R.Renderer(e, 16, 8)
    f = seqs[0][1][0]
    lk = f["look"]
    lk_mesh = type(lk).from_buffer_copy(lk)
    lk_mesh.mesh_mode = 1
    u = R.FrameState().next(f["cam"], (16, 8))
    # meshMode over the cleared G-buffer: no car texels, so only ground and backdrop
    r.scene(u.cam, lk_mesh, mc.view())
    assert (r.read(R.TARGET_GNORMAL) == 0).all()
    with pytest.raises(WindTunnelError, match="cur"):
        r.taa(u.taa, 2)
    with pytest.raises(WindTunnelError, match="unknown target"):
        e._check(e.lib.wt_render_read(r.r, 10, np.zeros(4).ctypes.data), "wt_render_read")
    with pytest.raises(WindTunnelError, match="mesh missing"):
        e._check(e.lib.wt_render_mesh(r.r, None, None, None, 0), "wt_render_mesh")
    r.scene(u.cam, lk, mc.view())  # the renderer stays usable
    r.close()


def test_renderer_outlives_its_context(wt_lib):
    """Destroying the context first releases the renderer's targets; the handle
    then only reports errors and can still be destroyed."""
    from windtunnel import AeroEngine, WindTunnelError
    from windtunnel import render as R
    e = AeroEngine(dims=(16, 8, 8), h=0.2)
    r = R.Renderer(e, 8, 4)
    e.close()
    rc = e.lib.wt_render_bloom(r.r)
    assert rc != 0
    r.close()
    e2 = AeroEngine(dims=(16, 8, 8), h=0.2)
    with pytest.raises(WindTunnelError, match="width and height"):
        R.Renderer(e2, 0, 4)
    e2.close()
