"""The car mesh G-buffer pass on the GPU (wt_mesh_*, wt_render_mesh through the C
ABI) bit for bit against the fixture made with the reference's own MESH_DRAW
shaders in the restated WebGPU pipeline (tests/golden/mesh.npz,
tests/golden/make_mesh.py), and the scene pass's G-buffer composite
(meshMode) against the reference's RENDER shader."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from helpers import same_half

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)


def fixture_mesh(z):
    """The stand-in mesh as stored (draw ranges and materials from the generator)."""
    import make_mesh as mm
    from windtunnel.mesh_car import MeshData, synthetic_mesh
    draws = synthetic_mesh(mm.DETAIL).draws
    texs = [(z[f"tex{t}"].shape[1], z[f"tex{t}"].shape[0], z[f"tex{t}"]) for t in range(3)]
    return MeshData(z["verts"], z["indices"], z["tags"], draws, texs)


@pytest.fixture(scope="module")
def setup(wt_lib):
    import make_consumers as mc
    from windtunnel import AeroEngine
    from windtunnel.mesh_car import MeshCar
    c = np.load(os.path.join(GOLDEN, "consumers.npz"))
    z = np.load(os.path.join(GOLDEN, "mesh.npz"))
    e = AeroEngine(dims=mc.DIMS, origin=mc.ORIGIN, h=mc.H)
    mesh = MeshCar(e, fixture_mesh(z))
    yield mc, z, e, mesh, c
    mesh.close()
    e.close()


def check_gbuffer(r, z, name):
    from windtunnel import render as R
    for t, key in ((R.TARGET_GALBEDO, "albedo"), (R.TARGET_GNORMAL, "normal")):
        got, ref = r.read(t), z[f"{name}_{key}"]
        bad = np.argwhere(np.any(~same_half(got, ref), axis=-1))
        assert len(bad) == 0, f"{name} {key}: {len(bad)} texels differ, first {bad[:4].tolist()}"
    got, ref = r.read(R.TARGET_GMATERIAL), z[f"{name}_material"]
    bad = np.argwhere(np.any(got != ref, axis=-1))
    assert len(bad) == 0, f"{name} material: {len(bad)} texels differ, first {bad[:4].tolist()}"


def test_gbuffer_bitexact(setup):
    import make_mesh as mm
    from windtunnel import render as R
    from windtunnel.mesh_car import mesh_cam
    mc, z, e, mesh, c = setup
    for name, p, fly, cam, size, k in mm.cases():
        r = R.Renderer(e, *size)
        try:
            r.mesh(mesh, mesh_cam(cam, size, mm.frame_halton(k), p), z[f"{name}_rig"], p.gurney)
            check_gbuffer(r, z, name)
            # the pass clears its targets: a second frame gives the same bits
            r.mesh(mesh, mesh_cam(cam, size, mm.frame_halton(k), p), z[f"{name}_rig"], p.gurney)
            check_gbuffer(r, z, name)
        finally:
            r.close()


def test_gbuffer_corner_cases(setup):
    """Near-plane clipping, a triangle behind the camera, a zero-area one, z-fighting
    coplanar quads, decal layers in one plane, a wall larger than the view, a
    ragged and an empty draw (tests/golden/make_mesh.py edge_mesh)."""
    import make_mesh as mm
    from windtunnel import render as R
    from windtunnel.mesh_car import MeshCar, MeshData, mesh_cam
    mc, z, e, mesh, c = setup
    em = mm.edge_mesh()
    data = MeshData(z["edge_verts"], z["edge_indices"], em.tags, em.draws, [(8, 8, z["edge_tex"])])
    m = MeshCar(e, data)
    r = R.Renderer(e, 80, 48)
    try:
        r.mesh(m, mesh_cam(mm.edge_camera(), (80, 48), (0.0, 0.0), mm.cases()[0][1]), z["hero_rig"])
        check_gbuffer(r, z, "edge")
    finally:
        r.close()
        m.close()


def test_composite_bitexact(setup):
    """Mesh pass, then the scene pass with meshMode over the consumer fixture's
    flow, as Renderer.frame runs them (engine.ts:679-716)."""
    import make_mesh as mm
    from windtunnel import render as R
    from windtunnel.car_model import synthetic_w17
    mc, z, e, mesh, c = setup
    for name, p, fly, cam, size, k in mm.cases():
        if name not in ("hero", "rig"):
            continue
        e.set_car_model(synthetic_w17(p, fly))
        e.set_shape(p)
        e.write_state(fields=c["fields"], temps=c["temps"])
        for cooling in (1, 2):
            r = R.Renderer(e, *size)
            try:
                r.state.frame_no = k - 1
                r.frame(cam, R.make_look(p, palette=1, cooling=cooling), mc.view(), mesh=mesh,
                        rig=z[f"{name}_rig"], params=p)
                check_gbuffer(r, z, name)
                got, ref = r.read(R.TARGET_SCENE), z[f"{name}_scene_c{cooling}"]
                bad = np.argwhere(np.any(~same_half(got, ref), axis=-1))
                assert len(bad) == 0, f"{name} cooling {cooling}: {len(bad)} texels differ, first {bad[:4].tolist()}"
            finally:
                r.close()


def test_mesh_errors(setup):
    from windtunnel.mesh_car import draw_struct, DrawSpec
    mc, z, e, mesh, c = setup
    import ctypes
    lib = e.lib
    bad = DrawSpec("x", (1, 1, 1, 1), 0, 0.5, 0.2, 0, 0, 1, first=int(z["indices"].size) - 3, count=6)
    assert lib.wt_mesh_add_draw(mesh.m, ctypes.byref(draw_struct(bad))) != 0      # beyond the index buffer
    notex = DrawSpec("x", (1, 1, 1, 1), 0, 0.5, 0.2, 0, 0, 1, first=0, count=3, texture=7)
    assert lib.wt_mesh_add_draw(mesh.m, ctypes.byref(draw_struct(notex))) != 0    # no such texture
    v = np.zeros((3, 8), np.float32)
    i = np.array([0, 1, 3], np.uint32)
    t = np.zeros(3, np.uint8)
    m = ctypes.c_void_p()
    assert lib.wt_mesh_create(e.ctx, v.ctypes.data, 3, i.ctypes.data, 3, t.ctypes.data, ctypes.byref(m)) != 0


def test_set_shape_rebuilds_the_rig(setup):
    """setShape hands the W17 rig of the new wing settings to the scene (engine.ts:450-462)."""
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import ShapeKind, ShapeParams
    mc, z, e, mesh, c = setup
    p0 = ShapeParams(kind=ShapeKind.W17)
    p1 = ShapeParams(kind=ShapeKind.W17, frontFlapDeg=9.0, rearWing=1, thinWings=True)
    e.set_car_model(synthetic_w17(p0))
    e.set_shape(p1)
    assert np.array_equal(e.car_model.rig, synthetic_w17(p1).rig)
    d1 = e.debug_read()["solid"].copy()
    e.set_car_model(synthetic_w17(p1))
    e.set_shape(p1)
    assert np.array_equal(e.debug_read()["solid"], d1)
