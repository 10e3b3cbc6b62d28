"""The baked W17 scene (kind 5) on the GPU through the C ABI: voxel flags and
emission bit for bit against the reference's own voxelizer (tests/golden/w17.npz,
made by tests/golden/make_w17.py from the synthetic stand-in model), and a run
on the geometry with cooling ducts (emit -1 cells: velocity relaxation, no
force) bit for bit against the oracle."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def fixture():
    return np.load(os.path.join(ROOT, "tests", "golden", "w17.npz"))


def test_w17_voxelize_bitexact(wt_lib):
    import make_w17
    from windtunnel import AeroEngine
    from windtunnel.car_model import synthetic_w17
    z = fixture()
    e = AeroEngine(dims=make_w17.DIMS, origin=make_w17.ORIGIN, h=make_w17.H)
    for k, p in make_w17.settings().items():
        e.set_car_model(synthetic_w17(p))
        e.set_shape(p)
        d = e.debug_read(emit=True)
        np.testing.assert_array_equal(d["solid"].astype(np.uint8), z[f"solid_{k}"], err_msg=k)
        np.testing.assert_array_equal(d["emit"], z[f"emit_{k}"], err_msg=k)
    e.close()


def test_w17_run_with_ducts_bitexact(wt_lib, oracle_mod):
    import make_w17
    from windtunnel import AeroEngine
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import make_sim
    z = fixture()
    p = make_w17.settings()["B"]
    sim = make_sim(u_in=0.08, tau0=0.51, smag=0.12)
    e = AeroEngine(dims=make_w17.DIMS, origin=make_w17.ORIGIN, h=make_w17.H, sim=sim)
    e.set_car_model(synthetic_w17(p))
    e.set_shape(p)
    e.reset()
    o = oracle_mod.Oracle(make_w17.DIMS, make_w17.ORIGIN, make_w17.H, sim)
    o.set_solid(z["solid_B"].astype(np.uint32), z["emit_B"])
    o.reset()
    for _ in range(3):
        e.frame(6)
        o.frame(6)
        d = e.debug_read()
        od = o.read(reset_forces=True)
        np.testing.assert_array_equal(d["fields"], od["fields"])
        np.testing.assert_array_equal(d["temps"], od["temps"])
        np.testing.assert_array_equal(e.read_populations(), od["f"])
        assert list(e.read_forces_raw().raw) == od["forces"].tolist()
    duct = z["emit_B"] < 0
    assert np.abs(d["fields"][duct, 0]).max() > 0
    e.close()


def test_w17_needs_a_car_model(wt_lib):
    from windtunnel import AeroEngine, WindTunnelError
    from windtunnel.engine import ShapeKind, ShapeParams
    e = AeroEngine(dims=(32, 12, 10), h=0.2)
    with pytest.raises(WindTunnelError, match="car model"):
        e.set_shape(ShapeParams(kind=ShapeKind.W17))
    e.close()
