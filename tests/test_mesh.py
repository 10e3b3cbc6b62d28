"""The baked-mesh path of the renderer without a GPU: the scene pass's G-buffer
composite (render-wgsl.ts:300-323, louvres :160-178) of the device code, built
for the host, equals the reference's translated RENDER shader at every pixel."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from helpers import same_half

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)


def synthetic_gbuffer(scene_dist, seed):
    """A G-buffer over a w x h view: car texels where the scene's hit distance is
    short (so surface points lie on the model, louvre regions included), unit
    normals leaning up, random albedo / roughness and material bytes."""
    rng = np.random.default_rng(seed)
    h, w = scene_dist.shape
    car = (scene_dist < 9.0) & (rng.random((h, w)) < 0.85)
    n = rng.normal(size=(h, w, 3)) + np.array([0.0, 1.1, 0.0])
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    normal = np.zeros((h, w, 4), np.float16)
    normal[..., :3] = n
    normal[..., 3] = np.where(car, scene_dist, 0.0)
    normal[~car, :3] = 0
    albedo = np.zeros((h, w, 4), np.float16)
    albedo[..., :3] = rng.random((h, w, 3))
    albedo[..., 3] = rng.uniform(0.05, 1.0, (h, w))
    material = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    material[..., 3] = 255
    return albedo, normal, material


@pytest.fixture(scope="module")
def mesh_views():
    """The W17 stand-in seen from above the sidepods, with the flow fixture's fields."""
    from oracle import pyoracle
    if pyoracle.ref_lib() is None or pyoracle.shade_model_lib() is None:
        pytest.skip("needs the translated reference and the CUDA headers")
    import make_consumers as mc
    from windtunnel import render as R
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import ShapeKind, ShapeParams, pack_shape
    c = {k: v for k, v in np.load(os.path.join(GOLDEN, "consumers.npz")).items()}
    p = ShapeParams(kind=ShapeKind.W17, rideH=0.11, rearRideH=0.14, sidepods=0)
    car = synthetic_w17(p)
    w, h = 96, 54
    cam = R.orbit_camera((3.4, 0.5, 0.3), 2.0, 0.55, 4.2, w / h)
    st = R.FrameState()
    u = st.next(cam, (w, h))
    pyoracle.ref_set_car(car)
    pyoracle.shade_model_set_car(car)
    args = (mc.DIMS, mc.ORIGIN, mc.H, c["fields"], c["temps"], pack_shape(p))
    yield pyoracle, args, u, p, mc.view(), (w, h)
    pyoracle.ref_set_car(None)
    pyoracle.shade_model_set_car(None)
    pyoracle.ref_set_gbuffer(None, None, None)
    pyoracle.shade_model_set_gbuffer(None, None, None)


def test_device_composite_matches_reference(mesh_views):
    from windtunnel import render as R
    po, (dims, origin, hh, fields, temps, shape), u, p, view, (w, h) = mesh_views
    base = R.make_look(p, palette=1)
    plain = po.ref_render_scene(dims, origin, hh, fields, temps, shape, u.cam, base, view, w, h)
    gb = synthetic_gbuffer(plain[..., 3], 7)
    po.ref_set_gbuffer(*gb)
    po.shade_model_set_gbuffer(*gb)
    slotted = 0
    for cooling in (0, 1, 2):
        for surf in (False, True):
            look = R.make_look(p, palette=1, surface_field=surf, cooling=cooling)
            look.mesh_mode = 1
            ref = po.ref_render_scene(dims, origin, hh, fields, temps, shape, u.cam, look, view, w, h)
            got = po.shade_model_render(shape, u.cam, look, view, np.array(dims, np.uint32),
                                        np.array(origin, np.float32), hh, fields, temps, w, h, threads=4)
            bad = np.argwhere(np.any(~same_half(got, ref), axis=-1))
            assert len(bad) == 0, f"cooling {cooling} surf {surf}: {len(bad)} pixels differ, first {bad[:4].tolist()}"
            if cooling == 0 and not surf:
                closed = ref
            elif not surf:
                slotted += int(np.any(~same_half(ref, closed), axis=-1).sum())
    car = gb[1][..., 3].astype(np.float32) > 0
    # the mesh replaced the marched surfaces, and open louvres changed some car texels
    assert car.sum() > 500 and not np.array_equal(ref[car], plain[car])
    assert slotted > 20


# ---------------------------------------------------------------- the mesh pass's inputs and fixture
def test_synthetic_mesh_matches_fixture():
    import make_mesh as mm
    from windtunnel.mesh_car import synthetic_mesh
    z = np.load(os.path.join(GOLDEN, "mesh.npz"))
    m = synthetic_mesh(mm.DETAIL)
    assert np.array_equal(m.verts.view(np.uint32), z["verts"].view(np.uint32))
    assert np.array_equal(m.indices, z["indices"]) and np.array_equal(m.tags, z["tags"])
    for t, (w, h, rgba) in enumerate(m.textures):
        assert rgba.shape == (h, w, 4) and np.array_equal(rgba, z[f"tex{t}"])
    # opaque draws first, then the two decals, then the optional gurney (MeshCar's order)
    assert [d.blend for d in m.draws] == [False] * 7 + [True, True, False] and m.draws[-1].optional
    assert m.indices.max() < m.verts.shape[0]
    # the strip joining the front wing to the nose was split by detach_seams: no mixed triangles left
    asm = m.tags[m.indices.reshape(-1, 3)] >> 3
    assert (asm.min(axis=1) == asm.max(axis=1)).all()


def test_reference_reproduces_mesh_fixture():
    from oracle import pyoracle
    if pyoracle.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    import make_mesh as mm
    from windtunnel.mesh_car import mesh_cam, synthetic_mesh
    z = np.load(os.path.join(GOLDEN, "mesh.npz"))
    mesh = synthetic_mesh(mm.DETAIL)
    for name, p, fly, cam, size, k in mm.cases():
        a, n, m, _ = pyoracle.ref_mesh_gbuffer(mesh, mesh_cam(cam, size, mm.frame_halton(k), p), z[f"{name}_rig"],
                                               size[0], size[1], gurney=p.gurney)
        assert same_half(a, z[f"{name}_albedo"]).all() and same_half(n, z[f"{name}_normal"]).all(), name
        assert np.array_equal(m, z[f"{name}_material"]), name
    em = mm.edge_mesh()
    assert np.array_equal(em.verts, z["edge_verts"]) and np.array_equal(em.indices, z["edge_indices"])
    a, n, m, _ = pyoracle.ref_mesh_gbuffer(em, mesh_cam(mm.edge_camera(), (80, 48), (0.0, 0.0), mm.cases()[0][1]),
                                           z["hero_rig"], 80, 48)
    assert same_half(a, z["edge_albedo"]).all() and same_half(n, z["edge_normal"]).all()
    assert np.array_equal(m, z["edge_material"])


def test_mesh_fixture_covers_the_pipeline():
    """The fixture exercises what the pass does: decals blended over the paint,
    rig-moved flaps, a flying wing, near-plane clipping, the large floor."""
    z = np.load(os.path.join(GOLDEN, "mesh.npz"))
    for name in ("hero", "rig", "fly", "close", "under"):
        n = z[f"{name}_normal"].astype(np.float32)
        car = n[..., 3] > 0
        assert car.sum() > 300, name
        assert np.allclose(np.linalg.norm(n[car][:, :3], axis=1), 1.0, atol=2e-3), name
        m = z[f"{name}_material"]
        assert (m[car][:, 3] == 255).all() and (m[~car] == 0).all(), name
    # emissive light (1.5 -> 255) and paint coat (255) and carbon coat (153) all appear
    assert set(np.unique(z["hero_material"][..., 1]).tolist()) >= {153, 255}
    # the composite differs with the louvres opened
    assert not np.array_equal(z["hero_scene_c1"], z["hero_scene_c2"])


def test_detach_seams_small():
    from windtunnel.mesh_car import detach_seams
    verts = np.arange(5 * 8, dtype=np.float32).reshape(5, 8)
    tags = np.array([0, 0, 8, 9, 16], np.uint8)   # assemblies 0, 0, 1, 1, 2
    idx = np.array([0, 1, 2,    2, 3, 0,    0, 3, 4], np.uint32)
    v2, t2 = detach_seams(verts, idx, tags)
    # face 0: two body corners -> body owns it, vertex 2 duplicated as assembly 0 (part 0)
    # face 1: two front-wing corners -> front wing, vertex 0 duplicated as assembly 1
    # face 2: all different -> the largest assembly (2) owns it
    assert idx.tolist()[:3] == [0, 1, 5] and t2[5] == 0 and np.array_equal(v2[5], verts[2])
    assert idx.tolist()[3:6] == [2, 3, 6] and t2[6] == 8
    assert idx[8] == 4 and t2[idx[6]] >> 3 == 2 and t2[idx[7]] == (9 & 7) | (2 << 3)


def _png(rgba, filt):
    """Encode RGBA8 with one PNG filter type on every row (the test's own encoder)."""
    import struct
    import zlib
    h, w, _ = rgba.shape
    raw = rgba.reshape(h, w * 4).astype(np.int32)
    rows = []
    for y in range(h):
        cur, up = raw[y], raw[y - 1] if y else np.zeros(w * 4, np.int32)
        left = np.concatenate([np.zeros(4, np.int32), cur[:-4]])
        ul = np.concatenate([np.zeros(4, np.int32), up[:-4]])
        if filt == 0:
            f = cur
        elif filt == 1:
            f = cur - left
        elif filt == 2:
            f = cur - up
        elif filt == 3:
            f = cur - (left + up) // 2
        else:
            p = left + up - ul
            pa, pb, pc = np.abs(p - left), np.abs(p - up), np.abs(p - ul)
            f = cur - np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, up, ul))
        rows.append(bytes([filt]) + (f & 255).astype(np.uint8).tobytes())

    def chunk(k, b):
        return struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b) & 0xffffffff)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


def test_png_decode_every_filter(wt_lib):
    from windtunnel.mesh_car import decode_png
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (13, 17, 4), dtype=np.uint8)
    for filt in range(5):
        w, h, out = decode_png(_png(img, filt))
        assert (w, h) == (17, 13) and np.array_equal(out, img), filt


def test_w17_assets_build_the_mesh(wt_lib):
    assets = os.path.join(os.environ.get("WT_REFERENCE_ROOT", "/root/reference"), "public", "models")
    if not os.path.isdir(assets):
        pytest.skip("the reference's W17 assets are not on this machine")
    import json
    from windtunnel.mesh_car import build_mesh, parse_glb
    with open(os.path.join(assets, "w17.glb"), "rb") as f:
        scene = parse_glb(f.read())
    assert sum(p.indices.size for p in scene.primitives) // 3 == 267690
    assert sum(p.positions.shape[0] for p in scene.primitives) == 188831
    parts = np.fromfile(os.path.join(assets, "w17.rig.bin"), np.uint8)
    rig = json.load(open(os.path.join(assets, "w17.rig.json")))
    used = {scene.texture_image[m.base_color_texture] for m in scene.materials if m.base_color_texture is not None}
    small = [i for i in used if len(scene.images[i][1]) < 300000]
    data = build_mesh(scene, parts, decode=lambda b, mime: (1, 1, np.full((1, 1, 4), 255, np.uint8)),
                      gurney_edge=rig["wings"]["rear"][-1])
    assert data.indices.max() < data.verts.shape[0]
    assert [d.blend for d in data.draws].index(True) == sum(not d.blend for d in data.draws) - 1  # gurney last
    assert data.draws[-1].optional and sum(d.blend for d in data.draws) == 3
    # the car sits in the tunnel frame: nose near x = 0, rear past 4.4, on the ground
    x = data.verts[:, 0]
    assert -0.4 < x.min() < 0.3 and 4.6 < x.max() < 5.4 and data.verts[:, 1].min() > -0.05
    # a few of the real textures decode (palette, RGB and RGBA images among them)
    from windtunnel.mesh_car import decode_png
    for i in small[:6]:
        w, h, rgba = decode_png(scene.images[i][1])
        assert rgba.shape == (h, w, 4) and rgba.dtype == np.uint8


def test_wing_fly_away_animation():
    """animateWings (engine.ts:395-408) as the viewer runs it for the mesh rig."""
    from types import SimpleNamespace
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import ShapeKind, ShapeParams
    from windtunnel.viewer import Viewer
    p = ShapeParams(kind=ShapeKind.W17, frontWingOn=False)
    v = Viewer.__new__(Viewer)
    v.fly = [0.0, 0.0]
    v.engine = SimpleNamespace(shape_params=p, car_model=synthetic_w17(p))
    for _ in range(30):
        v.animate_wings(1 / 60)
    assert v.fly[0] == pytest.approx(30 / 60 * 0.75) and v.fly[1] == 0.0
    for _ in range(200):
        v.animate_wings(1 / 60)
    # it stops within 1e-4 of the target, as the engine's loop does
    assert v.fly[0] == pytest.approx(1.0, abs=1e-4) and v.fly[1] == 0.0 and v.engine.fly == tuple(v.fly)
    rig = v.mesh_rig()
    assert rig[74].tolist() == pytest.approx([1.0, 0.0, 0.0, 1.0], abs=1e-4)  # progress; front off, rear fitted
    v.engine.shape_params = ShapeParams(kind=ShapeKind.W17)   # refitted: back at 1.4 per second
    v.animate_wings(0.5)
    assert v.fly[0] == pytest.approx(0.3)
