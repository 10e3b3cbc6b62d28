"""The whole frame of the reference engine (src/engine/engine.ts:574-726):
simulation steps and heat passes, the particle or streamline pass, and the
render passes into a headless RGBA8 image, plus the headless check
(scripts/headless-check.ts) that writes its shots as PNG files.

    v = Viewer(AeroEngine("medium"), 1280, 720)
    v.set_view(ViewParams(flow_mode=FlowMode.Streamlines))
    v.engine.set_shape(ShapeParams(...)); v.engine.reset()
    for _ in range(240):
        v.frame(orbit_camera((2.75, 0.42, 0), 2.3, 0.3, 7.6, 16 / 9), steps=8)
    write_png("hero.png", v.image())

    python -m windtunnel.viewer --frames 240 --out shots/     # the headless check
    python -m windtunnel.viewer --w17 --out shots/            # the W17 car, mesh-drawn (stand-in assets)

Particles live in host memory and go through wt_particles_step each frame;
streamlines through wt_streamlines; everything else stays on the device.
"""
import argparse
import json
import math
import os
import struct
import time
import zlib
from dataclasses import dataclass, field, replace

import numpy as np

from . import _abi
from .engine import ORIGIN_X, QUALITIES, AeroEngine, ShapeKind, ShapeParams
from .render import TARGET_OUTPUT, Renderer, make_look, orbit_camera, shape_bounds

MAX_LINES = 160      # engine.ts:27
STREAM_STEPS = 360   # engine.ts:28
PARTICLES = {"low": 40_000, "medium": 80_000, "high": 140_000}  # engine.ts:14-18


class ColorField:  # engine.ts:33
    Speed, Pressure, Temperature, Vorticity, Wake = range(5)


class FlowMode:  # engine.ts:34
    None_, Streamlines, Smoke, Fog, Vortices = range(5)


@dataclass
class Livery:
    paint: tuple = (0.38, 0.4, 0.43)
    accent: tuple = (0.0, 0.82, 0.75)
    carbon: bool = True


@dataclass
class ViewParams:
    """ViewParams (engine.ts), defaults of the headless check's base view."""
    color_field: int = ColorField.Speed
    surface_field: bool = False
    slice_axis: int = 0
    slice_pos: float = 0.0
    flow_mode: int = FlowMode.Streamlines
    kmh: float = 250.0
    livery: Livery = field(default_factory=Livery)


def write_png(path, rgba):
    """An RGBA8 image [h, w, 4] as a PNG file (zlib, no filtering)."""
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w, _ = rgba.shape
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def f1_anchors(ride_h):
    """f1Anchors (engine.ts:120-131): front- and rear-wing heights."""
    return 0.19 + ride_h * 0.45, ride_h + 0.8


class Viewer:
    """An AeroEngine with its render targets and flow-visualisation state."""

    def __init__(self, engine: AeroEngine, width=1280, height=720, particles=None):
        self.engine = engine
        self.renderer = Renderer(engine, width, height)
        self.size = (width, height)
        n = particles if particles is not None else PARTICLES.get(self._quality(), 80_000)
        self.parts = np.zeros((n, 8), np.float32)
        self.scatter_frames = 2
        self.flow_time = 0.0
        self.view = ViewParams()
        self.mesh = None   # the car mesh the W17 scene draws into the G-buffer (engine.ts:679)
        self.fly = [0.0, 0.0]  # fly-away progress of the front and rear wing (engine.ts:192-193)

    def _quality(self):
        for q, d in QUALITIES.items():
            if tuple(d) == tuple(self.engine.dims):
                return q
        return "medium"

    def close(self):
        self.renderer.close()

    def set_view(self, v: ViewParams):
        self.view = v

    def set_mesh(self, mesh):
        """A mesh_car.MeshCar for the W17 scene (setCarModel's mesh, engine.ts:410-421)."""
        self.mesh = mesh

    def reset_particles(self):
        """reset() restarts the particles with two scatter frames (engine.ts:380)."""
        self.parts[:] = 0.0
        self.scatter_frames = 2

    # -- per-frame uniforms (engine.ts:391-393, 503-570) -------------------------
    def visual_flow_rate(self):
        return min(1.6, max(0.35, self.view.kmh / 250.0))

    def view_uniform(self):
        v, p = self.view, self.engine.shape_params
        v_real = v.kmh / 3.6
        stag = 0.5 * v_real * v_real / 1005
        race = p is not None and p.kind in (ShapeKind.F1, ShapeKind.W17)
        hot = race and (p.heatBrakes or p.heatEngine or p.heatRad)
        u = _abi.View()
        u.u_in, u.v_real, u.cp_min, u.cp_max = self.engine.u_lb, v_real, -1.1, 0.7
        u.t_min, u.t_max = (0.0, 220.0) if hot else (-stag * 1.4, stag * 1.05)
        u.speed_max, u.vort_max = 1.5, 0.6
        return u

    def spawn_region(self):
        p = self.engine.shape_params
        lo, hi = shape_bounds(p)
        race = p is not None and p.kind in (ShapeKind.F1, ShapeKind.W17)
        z_max = max(0.3, hi[2] + 0.25)
        y_max = max(0.5, hi[1] + 0.25)
        y_min = 0.04 if race else max(0.04, lo[1] - 0.25)
        return (ORIGIN_X + self.engine.h * 2, y_min, 0.0), (0.0, y_max, z_max), 12, 7

    def emitter_points(self):
        p = self.engine.shape_params
        if p is not None and p.kind == ShapeKind.F1:
            yw, yr = f1_anchors(p.rideH)
            pts = [(0.52, yw + 0.2, 0.926, 0.06), (0.52, yw + 0.07, 0.21, 0.05), (5.36, yr + 0.26, 0.494, 0.06),
                   (2.22, p.rideH + 0.06, 0.79, 0.05)]
        else:
            lo, hi = shape_bounds(p)
            pts = [(hi[0], hi[1] - 0.05, hi[2] - 0.05, 0.08), (hi[0], lo[1] + 0.05, hi[2] - 0.05, 0.08),
                   (hi[0], (lo[1] + hi[1]) / 2, 0.05, 0.1)]
        return pts

    def stream_params(self):
        """streamConfig (engine.ts:558-570) as the Stream uniform."""
        p = self.engine.shape_params
        s = _abi.StreamParams()
        em = self.emitter_points()
        for i, e in enumerate(em[:8]):
            s.emitter[i][:] = e
        if self.view.flow_mode == FlowMode.Vortices:
            per = MAX_LINES // len(em)
            s.lines, s.seed_mode, s.per_emitter, s.emitters, s.step_len, s.rows, s.cols = \
                per * len(em), 1, per, len(em), 0.022, 1, 1
        else:
            race = p is not None and p.kind in (ShapeKind.F1, ShapeKind.W17)
            lo, hi = shape_bounds(p)
            s.rows, s.cols = 18, 5
            s.lines, s.seed_mode, s.per_emitter, s.emitters, s.step_len = 90, 0, 1, 1, 0.03
            s.seed_min[:] = (-1.2, 0.05 if race else max(0.04, lo[1] - 0.2), 0.03)
            s.seed_max[:] = (0.0, 1.3 if race else hi[1] + 0.2, 0.95 if race else hi[2] + 0.2)
        s.steps = STREAM_STEPS
        s.color_mode = 0 if self.view.color_field == ColorField.Vorticity else self.view.color_field
        s.time = self.flow_time
        return s

    def animate_wings(self, dt):
        """animateWings (engine.ts:395-408): a detached wing flies off at 0.75 per
        second and a refitted one returns at 1.4 per second; the result only
        moves the mesh (the distance field keeps the rig of the last setShape)."""
        p = self.engine.shape_params
        target = (0.0 if p.frontWingOn else 1.0, 0.0 if p.rearWingOn else 1.0)
        for i in (0, 1):
            if abs(target[i] - self.fly[i]) < 1e-4:
                continue
            self.fly[i] = min(1.0, self.fly[i] + dt * 0.75) if target[i] > self.fly[i] else \
                max(0.0, self.fly[i] - dt * 1.4)
        self.engine.fly = tuple(self.fly)  # the progress the next setShape builds its rig with

    def mesh_rig(self):
        """The Rig uniform the mesh is drawn with: the model's, with the current fly-away progress."""
        rig = np.array(self.engine.car_model.rig, np.float32)
        rig[74, 0:2] = self.fly
        return rig

    # -- frame(target, cam, steps, dt) ----------------------------------------------
    def frame(self, cam, steps=8, dt=1.0 / 60):
        e, v = self.engine, self.view
        p = e.shape_params
        mesh_mode = (self.mesh is not None and p is not None and p.kind == ShapeKind.W17 and
                     getattr(e, "car_model", None) is not None)
        if mesh_mode:
            self.animate_wings(dt)
        self.flow_time += dt * self.visual_flow_rate()
        even = max(2, steps - steps % 2)
        color_mode = 0 if v.color_field == ColorField.Vorticity else v.color_field
        view = self.view_uniform()
        frame_no = self.renderer.state.frame_no + 1
        use_parts = v.flow_mode in (FlowMode.Smoke, FlowMode.Fog)
        use_lines = v.flow_mode in (FlowMode.Streamlines, FlowMode.Vortices)
        e.frame(even)  # the LBM steps and both heat passes (engine.ts:708-712)
        parts = lines = None
        if use_parts:
            lo, hi, rows, cols = self.spawn_region()
            ps = _abi.PSim()
            ps.count, ps.spawn_mode, ps.color_mode, ps.frame = len(self.parts), 0 if v.flow_mode == FlowMode.Fog else 1, \
                color_mode, frame_no
            ps.dt, ps.life, ps.scatter, ps.rake_rows, ps.rake_cols = even * self.visual_flow_rate(), 900, \
                1 if self.scatter_frames > 0 else 0, rows, cols
            ps.spawn_min[:] = lo
            ps.spawn_max[:] = hi
            if self.scatter_frames > 0:
                self.scatter_frames -= 1
            e.particles_step(self.parts, ps, view)
            parts = self.parts
        if use_lines:
            lines = e.streamlines(self.stream_params(), view)
        look = make_look(e.shape_params, palette=v.color_field, surface_field=v.surface_field,
                         slice_axis=v.slice_axis, slice_pos=v.slice_pos, paint=v.livery.paint,
                         accent=v.livery.accent, carbon=v.livery.carbon,
                         cooling=e.shape_params.cooling if e.shape_params is not None else 1)
        self.renderer.frame(cam, look, view, dt, v.kmh, parts, color_mode, v.flow_mode == FlowMode.Smoke, lines,
                            self.flow_time, v.flow_mode == FlowMode.Vortices, mesh=self.mesh if mesh_mode else None,
                            rig=self.mesh_rig() if mesh_mode else None, params=p)

    def image(self):
        return self.renderer.read(TARGET_OUTPUT)


# ---------------------------------------------------------------- headless check
HEADLESS_SHAPE = ShapeParams(kind=ShapeKind.F1, rearRideH=0.12, rideH=0.10, aoaDeg=6)   # headless-check.ts:21-24
SHOTS = [  # headless-check.ts:62-71: (name, view changes, orbit changes)
    ("hero", {}, {}),
    ("side-neon", {}, {"yaw": math.pi / 2, "pitch": 0.02, "distance": 7.2, "target": (2.75, 0.5, 0)}),
    ("front-pressure", {"color_field": ColorField.Pressure, "surface_field": True, "flow_mode": FlowMode.None_},
     {"yaw": math.pi + 0.001, "pitch": 0.12, "distance": 5.0, "target": (2.4, 0.5, 0)}),
    ("vortices", {"flow_mode": FlowMode.Vortices}, {"yaw": 2.55, "pitch": 0.25, "distance": 4.0, "target": (0.9, 0.3, 0.6)}),
    ("clean", {"flow_mode": FlowMode.None_}, {"yaw": 2.1, "pitch": 0.22, "distance": 6.6}),
    ("low-pressure", {"color_field": ColorField.Pressure, "surface_field": True, "flow_mode": FlowMode.None_},
     {"yaw": 2.0, "pitch": 0.04, "distance": 7.0, "target": (2.7, 0.35, 0)}),
    ("helmet", {"flow_mode": FlowMode.None_}, {"yaw": 2.5, "pitch": 0.3, "distance": 1.3, "target": (2.67, 0.83, 0)}),
    ("rear", {"flow_mode": FlowMode.Smoke}, {"yaw": 0.5, "pitch": 0.28, "distance": 5.5, "target": (4.6, 0.6, 0)}),
]


def orbit(o, aspect):
    d = {"target": (2.75, 0.42, 0.0), "yaw": 2.3, "pitch": 0.3, "distance": 7.6}
    d.update(o)
    return orbit_camera(d["target"], d["yaw"], d["pitch"], d["distance"], aspect)


W17_SHAPE = ShapeParams(kind=ShapeKind.W17, rideH=0.12, rearRideH=0.14)   # wing-sensitivity.ts's W17 setup


def headless_check(quality="medium", frames=240, out_dir=None, only=None, width=1280, height=720, w17=False,
                   assets=None):
    """scripts/headless-check.ts: run `frames` frames of 8 steps, print the
    summary line, then render the shots (6 frames of 2 steps each) to PNG.
    With w17 the car is the baked W17 model drawn from its mesh (the reference's
    assets from `assets`, else the stand-ins of car_model and mesh_car)."""
    engine = AeroEngine(quality)
    viewer = Viewer(engine, width, height)
    base = ViewParams()
    viewer.set_view(base)
    mesh = None
    if w17:
        from .car_model import load_w17, synthetic_w17
        from .mesh_car import MeshCar, load_w17_mesh, synthetic_mesh
        engine.set_car_model(load_w17(assets, W17_SHAPE) if assets else synthetic_w17(W17_SHAPE))
        mesh = MeshCar(engine, load_w17_mesh(assets) if assets else synthetic_mesh())
        viewer.set_mesh(mesh)
    engine.set_shape(W17_SHAPE if w17 else HEADLESS_SHAPE)
    engine.reset()
    viewer.reset_particles()
    aspect = width / height
    t0 = time.perf_counter()
    readings = []
    for i in range(frames):
        viewer.frame(orbit({}, aspect), 8, 1 / 60)
        if (i + 1) % 8 == 0:  # maybeReadForces every 8 frames (engine.ts:740)
            readings.append(engine.read_forces(base.kmh))
    engine.sync()
    t1 = time.perf_counter()
    d = engine.debug_read()
    fluid = d["solid"] == 0
    u = np.linalg.norm(d["fields"][fluid, :3], axis=1)
    bad = int((~np.isfinite(d["fields"][fluid])).any(axis=1).sum())
    last = readings[-1] if readings else None
    summary = {"quality": quality, "dims": list(engine.dims), "solidCount": int((~fluid).sum()), "bad": bad,
               "uMax": float(np.nanmax(u)) if u.size else 0.0, "msPerFrame": (t1 - t0) * 1e3 / max(1, frames),
               "forces": None if last is None else {"dragN": last.dragN, "downforceN": last.downforceN}}
    print(json.dumps(summary))
    written = []
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        for name, vchg, ochg in SHOTS:
            if only and only not in name:
                continue
            viewer.set_view(replace(base, **vchg))
            for _ in range(6):
                viewer.frame(orbit(ochg, aspect), 2, 1 / 60)
            path = os.path.join(out_dir, f"{name}.png")
            write_png(path, viewer.image())
            written.append(path)
    if mesh is not None:
        mesh.close()
    viewer.close()
    engine.close()
    return summary, written


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--quality", default="medium", choices=sorted(QUALITIES))
    ap.add_argument("--frames", type=int, default=240)
    ap.add_argument("--out", default=None, help="directory for the PNG shots")
    ap.add_argument("--only", default=None)
    ap.add_argument("--size", default="1280x720")
    ap.add_argument("--w17", action="store_true", help="the baked W17 car, drawn from its mesh")
    ap.add_argument("--assets", default=None, help="the reference's public/models directory (W17 assets)")
    a = ap.parse_args(argv)
    w, h = (int(x) for x in a.size.split("x"))
    headless_check(a.quality, a.frames, a.out, a.only, w, h, a.w17, a.assets)


if __name__ == "__main__":
    main()
