"""Host-side logic of the engine mirror, checked against the reference engine's
semantics (src/engine/engine.ts) with a fake C ABI (no GPU)."""
import ctypes
import math

import numpy as np
import pytest

from windtunnel import ShapeKind, ShapeParams, make_sim, pack_shape
from windtunnel import engine as E


def test_pack_shape_follows_setshape():
    p = ShapeParams(frontFlapDeg=3.0, rearFlapDeg=-5.0, rideH=0.07, rearRideH=0.09, aoaDeg=4, cooling=2,
                    heatBrakes=True, heatEngine=False, heatRad=True, frontWing=2, nose=1)
    s = pack_shape(p)
    f32 = lambda v: float(np.float32(v))
    assert s.kind == ShapeKind.F1 and s.pw == 256 and s.ph == 128
    assert s.front_flap == f32((3.0 + 14) * math.pi / 180)   # engine.ts:434
    assert s.rear_main == f32(9 * math.pi / 180)              # engine.ts:435
    assert s.rear_flap == f32((-5.0 + 32) * math.pi / 180)    # engine.ts:436
    assert s.ride_h == f32(0.07) and s.rear_ride == f32(0.09)
    assert s.heat_brakes == 520.0 and s.heat_engine == 0.0    # engine.ts:443-444
    assert s.heat_rad == f32(75 * 0.6)                        # COOLING_HEAT[2]
    assert s.duct == f32(1.3)                                 # COOLING_DUCT[2]
    assert s.front_wing == 2 and s.nose == 1


def test_make_sim_defaults_are_the_engine_constants():
    s = make_sim()
    assert (s.u_in, s.tau0, s.smag) == (np.float32(0.0925), np.float32(0.508), np.float32(0.17))  # engine.ts:110,249
    assert s.sponge_cells == 18 and s.inlet_cells == 10                                          # wgsl.ts:260
    assert (s.heat_cool, s.heat_diffuse) == (np.float32(0.004), np.float32(0.04))                # engine.ts:263


class FakeLib:
    """Records the C calls; returns canned forces."""

    def __init__(self):
        self.calls = []
        self.raw = [1000, -2000, 0, 300, -400, 0, 50, -60, 0, 0, 0, 0]
        self.steps = 0

    def wt_create(self, g, s, ctx):
        ctypes.cast(ctx, ctypes.POINTER(ctypes.c_void_p))[0] = 1234
        return 0

    def wt_step(self, ctx, n, heat, dt):
        self.calls.append(("step", n, heat, dt))
        if n < 2 or n % 2:
            return -1
        self.steps += n
        return 0

    def wt_read_forces(self, ctx, fptr, reset):
        f = fptr._obj
        for k in range(12):
            f.raw[k] = self.raw[k]
        f.steps = self.steps
        if reset:
            self.steps = 0
        return 0

    def wt_last_error(self, ctx):
        return b"fake"

    def wt_destroy(self, ctx):
        return 0


def test_frame_uses_even_steps_and_half_dt():
    lib = FakeLib()
    eng = E.AeroEngine(dims=(16, 8, 8), h=0.1, lib=lib)
    assert eng.frame(7) == 6 and lib.calls[-1] == ("step", 6, 2, 3.0)   # engine.ts:585,659
    assert eng.frame(1) == 2 and lib.calls[-1] == ("step", 2, 2, 1.0)
    assert eng.frame(12) == 12 and lib.calls[-1] == ("step", 12, 2, 6.0)


def test_force_scaling_matches_maybe_read_forces():
    lib = FakeLib()
    eng = E.AeroEngine(dims=(232, 68, 52), lib=lib)
    eng.frame(8)
    r = eng.read_forces(kmh=250.0)
    h = 10.4 / 232
    scale = (1 / 10000 / 8) * 1.225 * ((250 / 3.6) / 0.0925) ** 2 * h * h * 2   # engine.ts:752
    assert r.body.drag == pytest.approx(1000 * scale)
    assert r.body.down == pytest.approx(2000 * scale)
    assert r.frontWing.down == pytest.approx(400 * scale)
    assert r.dragN == pytest.approx((1000 + 300 + 50) * scale)
    assert r.downforceN == pytest.approx((2000 + 400 + 60) * scale)
    assert r.steps == 8
    r2 = eng.read_forces()
    assert r2.steps == 0 and r2.dragN == 0.0   # engine.ts:750 (no steps since the last read)


def test_step_error_surfaces():
    lib = FakeLib()
    eng = E.AeroEngine(dims=(16, 8, 8), h=0.1, lib=lib)
    with pytest.raises(E._abi.WindTunnelError):
        eng.step(3)
