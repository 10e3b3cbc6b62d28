"""The baked W17 scene (kind 5) without a GPU: the synthetic stand-in model is
the same bits everywhere, the host-side restatements of rigUniform and
partsAtlas read the reference's own asset files (where its checkout is
present), the device code's sdW17 (built for the host) equals the reference's
own SDF at arbitrary points for the stand-in and for the real W17 assets, the
voxel fixture is the reference's voxelization, and the oracle's collide-stream
step on duct cells equals the reference's."""
import ctypes
import hashlib
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
ASSETS = os.path.join(os.environ.get("WT_REFERENCE_ROOT", "/root/reference"), "public", "models")
SYNTH_SHA = {"A": "5390fb17dac47e42a20a694c765c5665eaca3c51bbf33918300e89d06c4a716f",
             "B": "7152e927ed4d76525904bd8385e188808f4cd0cf6bc06cd4231ee02202c18ae6"}


def model_sha(m):
    return hashlib.sha256(m.body_sdf.tobytes() + m.parts.tobytes() + m.rig.tobytes()).hexdigest()


def test_synthetic_model_is_deterministic():
    import make_w17
    from windtunnel.car_model import synthetic_w17
    for k, p in make_w17.settings().items():
        m = synthetic_w17(p)
        assert m.body_sdf.shape == (67, 84, 368) and m.rig.shape == (87, 4)
        assert model_sha(m) == SYNTH_SHA[k], k


def test_rig_uniform_and_atlas_of_the_reference_assets():
    if not os.path.isdir(ASSETS):
        pytest.skip("the reference's W17 assets are not on this machine")
    import json
    from windtunnel.car_model import load_w17, parts_atlas, rig_uniform
    from windtunnel.engine import ShapeKind, ShapeParams
    rig = json.load(open(os.path.join(ASSETS, "w17.rig.json")))
    data = np.fromfile(os.path.join(ASSETS, "w17.parts.bin"), np.uint16)
    atlas, dims = parts_atlas(rig, data)
    g = rig["partGrids"]
    assert dims == (max(x["dims"][0] for x in g), max(x["dims"][1] for x in g), sum(x["dims"][2] + 1 for x in g))
    # the second grid starts after the first grid's slices and one padding slice (car-model.ts:183-191)
    gx, gy, gz = g[1]["dims"]
    z0 = g[0]["dims"][2] + 1
    np.testing.assert_array_equal(atlas[z0, :gy, :gx], data[g[1]["offset"]:g[1]["offset"] + gx * gy].reshape(gy, gx))
    assert (atlas[z0 - 1] == 0x2400).all()
    u = rig_uniform(rig, [0.1, 0.2, 0.3, 0.4], 0.05, 0.72, 0.32, (0, 0, 1, 0))
    assert u[71].tolist() == pytest.approx([*rig["rearMainHinge"], *rig["rearFlapHinge"]])
    assert u[75 + 3].tolist() == pytest.approx([*g[1]["dims"], g[0]["dims"][2] + 1])  # dims + atlas z offset
    m = load_w17(ASSETS, ShapeParams(kind=ShapeKind.W17, thinWings=True, sidepods=1))
    assert m.rig[73].tolist() == pytest.approx([0.0, 0.72, 0.32, 0.0])


def _sdf_bitexact(oracle_mod, model, shape, n=200000, seed=0):
    L = oracle_mod.shade_model_lib()
    oracle_mod.ref_set_car(model)
    oracle_mod.shade_model_set_car(model)
    rng = np.random.default_rng(seed)
    pts = np.stack([rng.uniform(-0.8, 6.0, n), rng.uniform(-0.2, 1.6, n), rng.uniform(-1.3, 1.3, n)],
                   axis=1).astype(np.float32)
    ref = oracle_mod.ref_scene_sdf(shape, pts)
    out = np.zeros((n, 2), np.float32)
    L.wthm_scene_sdf(ctypes.addressof(shape), pts.ctypes.data, n, out.ctypes.data)
    oracle_mod.ref_set_car(None)
    oracle_mod.shade_model_set_car(None)
    bad = np.nonzero(np.any(out.view(np.uint32) != ref.view(np.uint32), axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} points differ, e.g. {pts[bad[:3]].tolist()}"
    assert set(np.unique(ref[:, 1]).tolist()) >= {2.0, 7.0, 8.0, 12.0}   # tyres, front / rear parts, body


def test_device_sdf_matches_reference_w17(oracle_mod):
    if oracle_mod.ref_lib() is None or oracle_mod.shade_model_lib() is None:
        pytest.skip("needs the translated reference and the CUDA headers")
    import make_w17
    from windtunnel.car_model import load_w17, synthetic_w17
    from windtunnel.engine import pack_shape
    for k, p in make_w17.settings().items():
        _sdf_bitexact(oracle_mod, synthetic_w17(p), pack_shape(p), seed=ord(k))
        if os.path.isdir(ASSETS):
            _sdf_bitexact(oracle_mod, load_w17(ASSETS, p), pack_shape(p), seed=10 + ord(k))


def test_reference_reproduces_w17_fixture(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    import make_w17
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import pack_shape
    z = np.load(os.path.join(GOLDEN, "w17.npz"))
    for k, p in make_w17.settings().items():
        oracle_mod.ref_set_car(synthetic_w17(p))
        r = oracle_mod.Reference(make_w17.DIMS, make_w17.ORIGIN, make_w17.H)
        r.voxelize(pack_shape(p))
        d = r.read()
        oracle_mod.ref_set_car(None)
        np.testing.assert_array_equal(d["solid"].astype(np.uint8), z[f"solid_{k}"])
        np.testing.assert_array_equal(d["emit"], z[f"emit_{k}"])
    assert (z["emit_B"] < 0).sum() > 100 and (z["emit_A"] < 0).sum() == 0


def test_oracle_duct_step_matches_reference(oracle_mod):
    """Duct cells (emit < 0): the velocity relaxation and the force exclusion of
    the reference's step (wgsl.ts:200-201, 221-223, 246-248)."""
    if oracle_mod.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    import make_w17
    from windtunnel.engine import make_sim
    z = np.load(os.path.join(GOLDEN, "w17.npz"))
    sim = make_sim(u_in=0.08, tau0=0.51, smag=0.12)  # the reference's 18-cell sponge
    o = oracle_mod.Oracle(make_w17.DIMS, make_w17.ORIGIN, make_w17.H, sim)
    r = oracle_mod.Reference(make_w17.DIMS, make_w17.ORIGIN, make_w17.H, sim)
    for m in (o, r):
        m.set_solid(z["solid_B"].astype(np.uint32), z["emit_B"])
        m.reset()
    for _ in range(3):
        for m in (o, r):
            m.frame(6)
        a, b = o.read(reset_forces=True), r.read(reset_forces=True)
        for k in ("fields", "f", "temps", "forces"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    duct = z["emit_B"] < 0
    assert np.abs(a["fields"][duct, 0]).max() > 0  # air moves through the ducts
