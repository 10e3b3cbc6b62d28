"""Fresh random scenes and states: oracle vs the reference's own shaders, bit for
bit.  Needs oracle/_ref (built from the reference checkout); skipped elsewhere."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("translated reference (oracle/_ref) not available on this machine")
    return oracle_mod


def random_shape(seed):
    from windtunnel.engine import ShapeParams, pack_shape
    r = np.random.default_rng(seed)
    return pack_shape(ShapeParams(frontWing=int(r.integers(0, 4)), rearWing=int(r.integers(0, 3)),
                                  sidepod=int(r.integers(0, 4)), cover=int(r.integers(0, 3)), nose=int(r.integers(0, 3)),
                                  frontFlapDeg=float(r.uniform(-10, 12)), rearFlapDeg=float(r.uniform(-15, 10)),
                                  rideH=float(r.uniform(0.01, 0.12)), rearRideH=float(r.uniform(0.01, 0.14)),
                                  cooling=int(r.integers(0, 3)), heatBrakes=bool(r.integers(0, 2))))


@pytest.mark.parametrize("seed", range(6))
def test_random_scene_voxelize(ref, seed):
    dims, origin, h = (80, 30, 24), (-2.4, 0.0, 0.0), 0.105 + 0.004 * seed
    s = random_shape(seed)
    o = ref.Oracle(dims, origin, h)
    r = ref.Reference(dims, origin, h)
    o.voxelize(s)
    r.voxelize(s)
    a, b = o.read(), r.read()
    np.testing.assert_array_equal(a["solid"], b["solid"])
    np.testing.assert_array_equal(a["emit"], b["emit"])


@pytest.mark.parametrize("seed", range(3))
def test_random_run(ref, seed):
    from windtunnel.engine import make_sim
    dims, origin, h = (56, 22, 18), (-2.4, 0.0, 0.0), 0.16
    sim = make_sim(u_in=0.06 + 0.01 * seed, tau0=0.505 + 0.005 * seed, smag=0.1 + 0.05 * seed)
    o = ref.Oracle(dims, origin, h, sim)
    r = ref.Reference(dims, origin, h, sim)
    s = random_shape(100 + seed)
    for m in (o, r):
        m.voxelize(s)
        m.reset()
    for _ in range(3):
        for m in (o, r):
            m.frame(6)
        a, b = o.read(reset_forces=True), r.read(reset_forces=True)
        for k in ("fields", "f", "temps", "forces"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
