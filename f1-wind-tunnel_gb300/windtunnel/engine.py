"""AeroEngine: the simulation half of the reference engine class
(src/engine/engine.ts:159-769), driving libwt through its C ABI.

Same names, argument meaning and error behaviour as the reference where the
reference has them:

    eng = AeroEngine("medium")            # new AeroEngine(V, gpu, quality, size)  engine.ts:226
    eng.set_shape(ShapeParams(...))       # setShape(p)                            engine.ts:426
    eng.reset()                           # reset()                                engine.ts:371
    eng.frame(steps=8)                    # frame(target, cam, steps, dt), compute pass only  engine.ts:574
    f = eng.read_forces(kmh=250)          # maybeReadForces + onForces payload     engine.ts:739-761
    d = eng.debug_read()                  # debugRead()                            engine.ts:763

Rendering, particles and streamlines of frame() are not part of this path.
"""
import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _abi

# engine.ts:14-23,110 and wgsl.ts:174
QUALITIES = {
    "low": (168, 50, 38),
    "medium": (232, 68, 52),
    "high": (296, 88, 66),
}
DOMAIN_LENGTH = 10.4
ORIGIN_X = -2.4
FORCE_SCALE = 10_000
AIR_DENSITY = 1.225
LATTICE_U = 0.0925
PROFILE_W, PROFILE_H = 256, 128
DEG = math.pi / 180.0
COOLING_HEAT = [1.55, 1.0, 0.6]  # engine.ts:114
COOLING_DUCT = [0.0, 1.0, 1.3]   # engine.ts:116


class ShapeKind:  # engine.ts:30
    F1 = 0
    Sphere = 1
    Cube = 2
    Wing = 3
    Custom = 4
    W17 = 5
    Empty = 6
    Box = 7  # build extension: axis-aligned box (no reference counterpart)


@dataclass
class ShapeParams:
    """engine.ts:36-65 ShapeParams, plus the box extension."""
    kind: int = ShapeKind.F1
    frontWing: int = 0
    rearWing: int = 0
    sidepod: int = 0
    cover: int = 0
    nose: int = 0
    rearRideH: float = 0.12
    rearMainDeg: float = 0.0
    gurney: bool = False
    frontWingOn: bool = True
    rearWingOn: bool = True
    rearShape: int = 0
    thinWings: bool = False
    sidepods: int = 0
    cooling: int = 1
    frontFlapDeg: float = 0.0
    rearFlapDeg: float = 0.0
    rideH: float = 0.10
    aoaDeg: float = 6.0
    customMode: int = 0
    customWidth: float = 0.5
    customAxisY: float = 1.0
    heatBrakes: bool = True
    heatEngine: bool = True
    heatRad: bool = True
    boxCenter: tuple = (0.0, 0.0, 0.0)
    boxHalf: tuple = (0.0, 0.0, 0.0)


def pack_shape(p: ShapeParams, p_scale: float = 0.02) -> _abi.Shape:
    """The Shape uniform that setShape builds (engine.ts:429-448)."""
    s = _abi.Shape()
    s.kind = int(p.kind)
    s.profile_mode = int(p.customMode)
    s.pw, s.ph = PROFILE_W, PROFILE_H
    s.front_flap = (p.frontFlapDeg + 14) * DEG
    s.rear_main = 9 * DEG
    s.rear_flap = (p.rearFlapDeg + 32) * DEG
    s.ride_h = p.rideH
    s.aoa = p.aoaDeg * DEG
    s.width = p.customWidth
    s.axis_y = p.customAxisY
    s.p_scale = p_scale
    s.p_origin[0] = 0.0
    s.p_origin[1] = 0.0
    cool = p.cooling if p.cooling is not None else 1
    s.heat_brakes = 520.0 if p.heatBrakes else 0.0
    s.heat_engine = 620.0 * COOLING_HEAT[cool] if p.heatEngine else 0.0
    s.heat_rad = 75.0 * COOLING_HEAT[cool] if p.heatRad else 0.0
    s.front_wing = p.frontWing
    s.rear_wing = p.rearWing
    s.sidepod = p.sidepod
    s.cover = p.cover
    s.nose = p.nose
    s.rear_ride = p.rearRideH
    s.duct = COOLING_DUCT[cool]
    for k in range(3):
        s.box_center[k] = p.boxCenter[k]
        s.box_half[k] = p.boxHalf[k]
    return s


def make_sim(u_in=LATTICE_U, tau0=0.508, smag=0.17, sponge_cells=18.0, storage="f32", **kw) -> _abi.Sim:
    """Sim uniform (engine.ts:249) plus the collision and heat constants of the shaders."""
    s = _abi.Sim()
    s.u_in, s.tau0, s.smag = u_in, tau0, smag
    s.sponge_cells = sponge_cells
    s.sponge_amp = kw.get("sponge_amp", 0.4)
    s.inlet_cells = kw.get("inlet_cells", 10.0)
    s.inlet_amp = kw.get("inlet_amp", 0.25)
    s.heat_cool = kw.get("heat_cool", 0.004)
    s.heat_diffuse = kw.get("heat_diffuse", 0.04)
    s.heat_src_mix = kw.get("heat_src_mix", 0.35)
    s.storage = _abi.STORAGE[storage] if isinstance(storage, str) else int(storage)
    s.reserved = 0
    return s


@dataclass
class ForcePair:
    drag: float
    down: float


@dataclass
class ForceReading:
    """onForces payload (engine.ts:100-107) plus the FP64 sums and counters."""
    dragN: float
    downforceN: float
    body: ForcePair
    frontWing: ForcePair
    rearWing: ForcePair
    raw: np.ndarray = field(repr=False)
    sum64: np.ndarray = field(repr=False)
    steps: int = 0
    guarded: int = 0
    mass: float = 0.0


class AeroEngine:
    def __init__(self, quality="medium", dims=None, h=None, origin=None, sim=None, lib=None, _ctx=None):
        nx, ny, nz = dims if dims is not None else QUALITIES[quality]
        self.dims = (int(nx), int(ny), int(nz))
        self.n = nx * ny * nz
        self.h = float(h) if h is not None else DOMAIN_LENGTH / nx
        self.origin = tuple(origin) if origin is not None else (ORIGIN_X, 0.0, 0.0)
        self.lib = lib or _abi.load()
        self.sim = sim or make_sim()
        self.u_lb = self.sim.u_in
        g = _abi.Grid()
        g.nx, g.ny, g.nz = self.dims
        for k in range(3):
            g.origin[k] = self.origin[k]
        g.h = self.h
        self._grid = g
        self._owned = _ctx is None
        if _ctx is not None:  # a lattice that belongs to a batch
            self.ctx = ctypes.c_void_p(_ctx)
        else:
            ctx = ctypes.c_void_p()
            rc = self.lib.wt_create(ctypes.byref(g), ctypes.byref(self.sim), ctypes.byref(ctx))
            if rc != _abi.WT_OK:
                raise _abi.WindTunnelError(rc, "wt_create: " + self.lib.wt_last_error(None).decode())
            self.ctx = ctx
        self.shape_params = None
        self.steps_since_read = 0

    # -- lifetime ---------------------------------------------------------------
    def close(self):
        if getattr(self, "ctx", None):
            if getattr(self, "_owned", True):
                self.lib.wt_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        _abi.check(self.lib, self.ctx, rc, what)

    # -- engine calls -----------------------------------------------------------
    def set_sim(self, sim):
        self._check(self.lib.wt_set_sim(self.ctx, ctypes.byref(sim)), "wt_set_sim")
        self.sim = sim

    def reset(self):
        self._check(self.lib.wt_reset(self.ctx), "wt_reset")

    def set_shape(self, p: ShapeParams):
        """setShape (engine.ts:426-470): for the W17 scene the Rig uniform follows
        the wing settings of p (engine.ts:450-462) when the car model carries
        its rig data; then voxelize."""
        self.shape_params = p
        model = getattr(self, "car_model", None)
        if p.kind == ShapeKind.W17 and model is not None and model.rig_data is not None:
            from dataclasses import replace
            from .car_model import w17_rig
            rig = w17_rig(model.rig_data, p, tuple(getattr(self, "fly", (0.0, 0.0))))
            if not np.array_equal(rig, model.rig):
                self.set_car_model(replace(model, rig=rig))
        self.set_shape_raw(pack_shape(p))

    def set_car_model(self, model):
        """setCarModel (engine.ts:410-421) with its rig: a car_model.CarModel
        (body SDF, parts atlas, Rig uniform) for scene kind ShapeKind.W17."""
        body = np.ascontiguousarray(model.body_sdf, np.uint16)
        parts = np.ascontiguousarray(model.parts, np.uint16)
        dims = np.array(model.parts_dims, np.uint32)
        rig = np.ascontiguousarray(model.rig, np.float32)
        assert body.size == 368 * 84 * 67 and parts.size == int(np.prod(dims)) and rig.shape == (87, 4)
        self._check(self.lib.wt_set_car_model(self.ctx, body.ctypes.data, parts.ctypes.data, dims.ctypes.data,
                                              rig.ctypes.data), "wt_set_car_model")
        self.car_model = model

    def set_shape_raw(self, shape: _abi.Shape):
        self._check(self.lib.wt_voxelize(self.ctx, ctypes.byref(shape)), "wt_voxelize")

    def set_solid(self, solid, emit):
        s = np.ascontiguousarray(solid, dtype=np.uint32).reshape(-1)
        e = np.ascontiguousarray(emit, dtype=np.float32).reshape(-1)
        if s.size != self.n or e.size != self.n:
            raise ValueError("solid/emit must have one entry per cell")
        self._check(self.lib.wt_set_solid(self.ctx, s.ctypes.data, e.ctypes.data), "wt_set_solid")

    def frame(self, steps=8, heat_passes=2):
        """The compute pass of frame(): evenSteps = max(2, steps - steps % 2)
        collide-stream steps, then two heat passes with dt = evenSteps / 2."""
        even = max(2, steps - steps % 2)
        self.step(even, heat_passes, even / 2.0)
        return even

    def step(self, n_lbm_steps, heat_passes=0, heat_dt=0.0):
        self._check(self.lib.wt_step(self.ctx, int(n_lbm_steps), int(heat_passes), float(heat_dt)), "wt_step")
        self.steps_since_read += n_lbm_steps

    def read_forces_raw(self, reset=True) -> _abi.Forces:
        f = _abi.Forces()
        self._check(self.lib.wt_read_forces(self.ctx, ctypes.byref(f), 1 if reset else 0), "wt_read_forces")
        if reset:
            self.steps_since_read = 0
        return f

    def read_forces_async(self, reset=True):
        """Queue a force readback without waiting (wt_read_forces_async): returns a
        ticket for collect_forces."""
        t = ctypes.c_uint64()
        self._check(self.lib.wt_read_forces_async(self.ctx, 1 if reset else 0, ctypes.byref(t)),
                    "wt_read_forces_async")
        if reset:
            self.steps_since_read = 0
        return t.value

    def collect_forces(self, ticket) -> _abi.Forces:
        """Wait for the readback of `ticket` and return its raw forces."""
        f = _abi.Forces()
        self._check(self.lib.wt_forces_collect(self.ctx, ticket, ctypes.byref(f)), "wt_forces_collect")
        return f

    def read_forces(self, kmh=250.0, reset=True):
        """maybeReadForces() scaling (engine.ts:750-759): Newtons, x2 for the mirrored half."""
        f = self.read_forces_raw(reset)
        steps = int(f.steps)
        raw = np.array(f.raw[:], dtype=np.int32)
        s64 = np.array(f.sum[:], dtype=np.float64)
        if steps == 0:
            zero = ForcePair(0.0, 0.0)
            return ForceReading(0.0, 0.0, zero, zero, zero, raw, s64, 0, int(f.guarded), f.mass)
        v_real = kmh / 3.6
        scale = (1.0 / FORCE_SCALE / steps) * AIR_DENSITY * (v_real / self.u_lb) ** 2 * self.h * self.h * 2
        pairs = [ForcePair(float(raw[3 * g]) * scale, float(-raw[3 * g + 1]) * scale) for g in range(3)]
        return ForceReading(
            dragN=sum(p.drag for p in pairs), downforceN=sum(p.down for p in pairs),
            body=pairs[0], frontWing=pairs[1], rearWing=pairs[2], raw=raw, sum64=s64,
            steps=steps, guarded=int(f.guarded), mass=f.mass)

    def force_history(self, count):
        out = np.zeros((count, 9), dtype=np.float64)
        self._check(self.lib.wt_read_force_history(self.ctx, out.ctypes.data, count), "wt_read_force_history")
        return out

    def debug_read(self, links=False, emit=False):
        """debugRead() (engine.ts:763-768): fields (n,4), solid (n,), temps (n,)."""
        n = self.n
        fields = np.zeros((n, 4), np.float32)
        solid = np.zeros(n, np.uint32)
        temps = np.zeros(n, np.float32)
        em = np.zeros(n, np.float32) if emit else None
        lk = np.zeros(n, np.uint32) if links else None
        self._check(self.lib.wt_read_fields(self.ctx, fields.ctypes.data, solid.ctypes.data, temps.ctypes.data,
                                            em.ctypes.data if emit else None, lk.ctypes.data if links else None),
                    "wt_read_fields")
        out = {"fields": fields, "solid": solid, "temps": temps}
        if emit:
            out["emit"] = em
        if links:
            out["links"] = lk
        return out

    def read_populations(self):
        f = np.zeros(19 * self.n, np.float32)
        self._check(self.lib.wt_read_populations(self.ctx, f.ctypes.data), "wt_read_populations")
        return f

    def write_state(self, f=None, fields=None, temps=None):
        def ptr(a, dt, size):
            if a is None:
                return None, None
            arr = np.ascontiguousarray(a, dtype=dt).reshape(-1)
            if arr.size != size:
                raise ValueError("wrong array size")
            return arr, arr.ctypes.data
        fa, fp = ptr(f, np.float32, 19 * self.n)
        ua, up = ptr(fields, np.float32, 4 * self.n)
        ta, tp = ptr(temps, np.float32, self.n)
        self._check(self.lib.wt_write_state(self.ctx, fp, up, tp), "wt_write_state")

    def save(self, path):
        """Checkpoint the whole simulation state to a file (wt_save)."""
        self._check(self.lib.wt_save(self.ctx, os.fsencode(path)), "wt_save")

    def load(self, path):
        """Resume from a checkpoint of a lattice of the same size and storage (wt_load)."""
        self._check(self.lib.wt_load(self.ctx, os.fsencode(path)), "wt_load")

    def reset_from(self, coarse_u_rho):
        c = np.ascontiguousarray(coarse_u_rho, dtype=np.float32)
        cz, cy, cx, four = c.shape
        assert four == 4
        self._check(self.lib.wt_reset_from(self.ctx, c.ctypes.data, cx, cy, cz), "wt_reset_from")

    # ---- aero-map sweep (src/ui/aeromap.ts:73-114) on this lattice
    def aeromap_sweep(self, base_shape, front, rear, settle_steps, measure_steps, read_every=64, kmh=250.0):
        """Serpentine ride-height sweep with re-voxelization into the running flow;
        returns an array [n_front, n_rear] of _abi.SweepCell."""
        fr = (ctypes.c_float * len(front))(*front)
        re = (ctypes.c_float * len(rear))(*rear)
        sw = _abi.Sweep(len(front), len(rear), fr, re, int(settle_steps), int(measure_steps), int(read_every),
                        float(kmh))
        cells = (_abi.SweepCell * (len(front) * len(rear)))()
        self._check(self.lib.wt_aeromap_sweep(self.ctx, ctypes.byref(base_shape), ctypes.byref(sw),
                                              ctypes.cast(cells, ctypes.c_void_p)), "wt_aeromap_sweep")
        return [[cells[i * len(rear) + j] for j in range(len(rear))] for i in range(len(front))]

    # ---- field consumers (wgsl.ts:324-366, 516-594; render-wgsl.ts:520-576)
    def sample_flow(self, points, vorticity=False):
        """sampleFlow at world points [n, 3]: returns [n, 6] (ux, uy, uz, rho, temp, fluid)
        and, if asked, vorticityAt [n]."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        n = pts.shape[0]
        out = np.zeros((n, 6), np.float32)
        vort = np.zeros(n, np.float32) if vorticity else None
        self._check(self.lib.wt_sample_flow(self.ctx, pts.ctypes.data, n, out.ctypes.data,
                                            None if vort is None else vort.ctypes.data), "wt_sample_flow")
        return (out, vort) if vorticity else out

    def particles_step(self, parts, psim, view):
        """One particle pass over parts [count, 8] float32 (updated in place, host)."""
        assert parts.dtype == np.float32 and parts.flags.c_contiguous and parts.shape == (psim.count, 8)
        self._check(self.lib.wt_particles_step(self.ctx, parts.ctypes.data, 0, ctypes.byref(psim),
                                               ctypes.byref(view)), "wt_particles_step")
        return parts

    def streamlines(self, params, view):
        """The streamline pass: [lines, steps, 4] points (x, y, z, colour or -1)."""
        out = np.zeros((params.lines, params.steps, 4), np.float32)
        self._check(self.lib.wt_streamlines(self.ctx, ctypes.byref(params), ctypes.byref(view), out.ctypes.data),
                    "wt_streamlines")
        return out

    def read_coarse(self, cx, cy, cz):
        """Fluid-cell box average of the last step call's (ux, uy, uz, rho): array [cz, cy, cx, 4]."""
        out = np.empty((cz, cy, cx, 4), np.float32)
        self._check(self.lib.wt_read_coarse(self.ctx, cx, cy, cz, out.ctypes.data), "wt_read_coarse")
        return out

    def tune(self):
        """Autotune the collide-stream block shape (state is preserved); returns (bx, by, ms/step)."""
        bx, by, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_float()
        self._check(self.lib.wt_tune(self.ctx, ctypes.byref(bx), ctypes.byref(by), ctypes.byref(ms)), "wt_tune")
        return bx.value, by.value, ms.value

    def info(self):
        i = _abi.Info()
        self._check(self.lib.wt_info_get(self.ctx, ctypes.byref(i)), "wt_info_get")
        return i

    def stream(self):
        return self.lib.wt_stream(self.ctx)

    def sync(self):
        self._check(self.lib.wt_sync(self.ctx), "wt_sync")


class AeroBatch:
    """Many lattices advanced together by one kernel launch per step, or by one
    persistent launch per up to 64 steps (the aero-map sweep of
    src/ui/aeromap.ts:73-114 run as concurrent cases).
    `lattices[i]` is an AeroEngine view of lattice i for voxelize/read calls."""

    def __init__(self, grids, sim=None, lib=None):
        """grids: list of (dims, origin, h)."""
        self.lib = lib or _abi.load()
        self.sim = sim or make_sim()
        arr = (_abi.Grid * len(grids))()
        for k, (dims, origin, h) in enumerate(grids):
            arr[k].nx, arr[k].ny, arr[k].nz = [int(d) for d in dims]
            for j in range(3):
                arr[k].origin[j] = origin[j]
            arr[k].h = h
        b = ctypes.c_void_p()
        rc = self.lib.wt_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(grids), ctypes.byref(self.sim),
                                      ctypes.byref(b))
        if rc != _abi.WT_OK:
            raise _abi.WindTunnelError(rc, "wt_batch_create: " + self.lib.wt_batch_last_error(None).decode())
        self.b = b
        self.lattices = [AeroEngine(dims=d, origin=o, h=h, sim=self.sim, lib=self.lib,
                                    _ctx=self.lib.wt_batch_lattice(b, k)) for k, (d, o, h) in enumerate(grids)]

    def _check(self, rc, what):
        if rc != _abi.WT_OK:
            raise _abi.WindTunnelError(rc, f"{what}: {self.lib.wt_batch_last_error(self.b).decode()}")

    def step(self, n_lbm_steps, heat_passes=0, heat_dt=0.0):
        self._check(self.lib.wt_batch_step(self.b, int(n_lbm_steps), int(heat_passes), float(heat_dt)),
                    "wt_batch_step")
        for e in self.lattices:
            e.steps_since_read += n_lbm_steps

    def tune(self):
        bx, by, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_float()
        self._check(self.lib.wt_batch_tune(self.b, ctypes.byref(bx), ctypes.byref(by), ctypes.byref(ms)),
                    "wt_batch_tune")
        return bx.value, by.value, ms.value

    def stream(self):
        return self.lib.wt_batch_stream(self.b)

    def persistent_grid(self):
        """Blocks of the persistent launch, or 0 when the batch launches once per step."""
        return self.lib.wt_batch_persistent_grid(self.b)

    def close(self):
        if getattr(self, "b", None):
            for e in self.lattices:
                e.ctx = None
            self.lib.wt_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
