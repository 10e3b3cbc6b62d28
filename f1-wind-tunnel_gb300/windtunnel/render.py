"""The render half of the reference engine's frame() (src/engine/engine.ts:574-726)
over libwt's render passes (include/wt.h, wt_render_*), into headless targets.

    cam = orbit_camera((2.75, 0.42, 0.0), yaw=2.3, pitch=0.3, distance=7.6, aspect=16 / 9)
    r = Renderer(engine, 1280, 720)
    r.frame(cam, make_look(engine.shape_params), view, dt=1 / 60)
    rgba = r.read(TARGET_OUTPUT)            # [720, 1280, 4] uint8

Camera helpers restate src/engine/camera.ts (orbitCamera) in double precision,
as JavaScript evaluates it, with the matrices rounded to float32 where the
reference stores them in Float32Array.  The per-frame host state (frame
counter, Halton jitter, TAA history flag, previous view-projection, time) is
the engine's (engine.ts:575-584, 662-676).
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import (TARGET_BLOOM_A, TARGET_BLOOM_B, TARGET_GALBEDO, TARGET_GLOW, TARGET_GMATERIAL, TARGET_GNORMAL,
                   TARGET_HIST0, TARGET_HIST1, TARGET_OUTPUT, TARGET_SCENE, Cam, Look, PDraw, Post, SDraw, Taa)

__all__ = ["CameraState", "orbit_camera", "halton", "shape_bounds", "make_look", "FrameState", "FrameUniforms",
           "Renderer", "TARGET_SCENE",
           "TARGET_HIST0", "TARGET_HIST1", "TARGET_GLOW", "TARGET_BLOOM_A", "TARGET_BLOOM_B", "TARGET_OUTPUT",
           "TARGET_GALBEDO", "TARGET_GNORMAL", "TARGET_GMATERIAL"]

STREAM_STEPS = 360  # engine.ts:28


@dataclass
class CameraState:
    """CameraState (engine.ts): world vectors as float64, view_proj as float32 column-major."""
    pos: tuple
    fwd: tuple
    right: tuple
    up: tuple
    fov_y: float
    view_proj: np.ndarray


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _norm(a):
    n = math.hypot(a[0], a[1], a[2]) or 1.0
    return (a[0] / n, a[1] / n, a[2] / n)


def orbit_camera(target, yaw, pitch, distance, aspect, fov_y=40 * math.pi / 180):
    """orbitCamera (src/engine/camera.ts:20-58)."""
    cp = math.cos(pitch)
    pos = (target[0] + distance * cp * math.cos(yaw), target[1] + distance * math.sin(pitch),
           target[2] + distance * cp * math.sin(yaw))
    fwd = _norm(_sub(target, pos))
    right = _norm(_cross(fwd, (0.0, 1.0, 0.0)))
    up = _cross(right, fwd)
    near, far = 0.05, 200.0
    f = 1.0 / math.tan(fov_y / 2)
    view = np.array([right[0], up[0], -fwd[0], 0, right[1], up[1], -fwd[1], 0, right[2], up[2], -fwd[2], 0,
                     -_dot(right, pos), -_dot(up, pos), _dot(fwd, pos), 1], np.float32)
    proj = np.array([f / aspect, 0, 0, 0, 0, f, 0, 0, 0, 0, far / (near - far), -1, 0, 0, (near * far) / (near - far), 0],
                    np.float32)
    vp = np.zeros(16, np.float32)
    for c in range(4):
        for r in range(4):
            s = 0.0
            for k in range(4):
                s += float(proj[k * 4 + r]) * float(view[c * 4 + k])
            vp[c * 4 + r] = s
    return CameraState(pos, fwd, right, up, fov_y, vp)


def halton(i, base):
    """halton (engine.ts:771-779)."""
    f, r, n = 1.0, 0.0, i
    while n > 0:
        f /= base
        r += f * (n % base)
        n = n // base
    return r


def shape_bounds(params):
    """shapeBounds (engine.ts:474-488) for the analytic scene kinds."""
    from .engine import ShapeKind
    k = params.kind if params is not None else ShapeKind.Empty
    if k == ShapeKind.F1:
        return (-0.08, 0.0, -0.98), (5.46, params.rideH + 1.34, 0.98)
    if k == ShapeKind.W17:
        return (-0.3, 0.0, -0.98), (5.2, params.rideH + 1.16, 0.98)
    if k == ShapeKind.Sphere:
        return (1.95, 0.35, -0.65), (3.25, 1.65, 0.65)
    if k == ShapeKind.Cube:
        return (2.05, 0.45, -0.55), (3.15, 1.55, 0.55)
    if k == ShapeKind.Wing:
        return (1.3, 0.2, -1.3), (3.6, 2.2, 1.3)
    return (2.6, 0.5, -0.05), (2.7, 0.6, 0.05)


def make_look(params, palette=0, surface_field=False, slice_axis=0, slice_pos=0.0, paint=(0.38, 0.4, 0.43),
              accent=(0.0, 0.82, 0.75), carbon=True, cooling=1):
    """The Look uniform the engine fills (engine.ts:697-704); livery defaults of the headless check."""
    from .engine import ShapeKind
    lo, hi = shape_bounds(params)
    lk = Look()
    lk.bmin[:] = lo
    lk.bmax[:] = hi
    lk.surf_mode = 1 if surface_field else 0
    lk.palette = palette
    lk.paint[:] = paint
    lk.carbon_body = 1 if carbon else 0
    lk.accent[:] = accent
    lk.is_f1 = 1 if params is not None and params.kind == ShapeKind.F1 else 0
    lk.slice_axis, lk.slice_pos, lk.slice_alpha, lk.show_flow = slice_axis, slice_pos, 0.82, 1
    lk.mesh_mode, lk.cooling = 0, cooling
    return lk


def cam_uniform(cam, size, time, road_speed, jitter):
    c = Cam()
    c.pos[:] = cam.pos
    c.tan_half = math.tan(cam.fov_y / 2)
    c.fwd[:] = cam.fwd
    c.aspect = size[0] / size[1]
    c.right[:] = cam.right
    c.time = time
    c.up[:] = cam.up
    c.road_speed = road_speed
    c.jitter[:] = jitter
    return c


def taa_uniform(cam, size, prev_view_proj, blend):
    t = Taa()
    t.prev_view_proj[:] = [float(v) for v in prev_view_proj]
    t.cam_pos[:] = cam.pos
    t.tan_half = math.tan(cam.fov_y / 2)
    t.fwd[:] = cam.fwd
    t.aspect = size[0] / size[1]
    t.right[:] = cam.right
    t.blend = blend
    t.up[:] = cam.up
    return t


def pdraw_uniform(cam, out_size, count, palette, smoke=True):
    """PDraw as frame() fills it (engine.ts:612-625)."""
    p = PDraw()
    p.view_proj[:] = [float(v) for v in cam.view_proj]
    p.cam_pos[:] = cam.pos
    p.width = max(1.4, out_size[1] / 700) * (1.4 if smoke else 1.1)
    p.res[:] = out_size
    p.trail = 6 if smoke else 3
    p.alpha = 0.08 if smoke else 0.16
    p.count = count
    p.palette = palette
    p.fade_in = 8
    return p


def sdraw_uniform(cam, out_size, lines, palette, time, vortices=False, steps=STREAM_STEPS):
    """SDraw as frame() fills it (engine.ts:642-655)."""
    s = SDraw()
    s.view_proj[:] = [float(v) for v in cam.view_proj]
    s.cam_pos[:] = cam.pos
    s.width = max(1.4, out_size[1] / 760)
    s.res[:] = out_size
    s.time = time
    s.intensity = 1.0 if vortices else 0.5
    s.lines = lines
    s.steps = steps
    s.palette = palette
    s.pulse = 2.6
    return s


@dataclass
class FrameUniforms:
    cam: Cam
    taa: Taa
    cur: int
    pdraw: object
    sdraw: object
    post: Post
    halton: tuple = (0.0, 0.0)  # the frame's (jx, jy) before scaling to pixels


class FrameState:
    """The engine's per-frame render state (engine.ts:575-584, 660-676): time,
    frame counter, Halton(2, 3) jitter over 8 frames, TAA history flag and the
    previous view-projection."""

    def __init__(self):
        self.frame_no = 0
        self.time = 0.0
        self.prev_view_proj = None
        self.history_valid = False

    def next(self, cam, size, dt=1.0 / 60, kmh=250.0, parts=None, color_mode=0, smoke=True, lines=None,
             flow_time=0.0, vortices=False):
        self.time += dt
        self.frame_no += 1
        k = (self.frame_no % 8) + 1
        jx, jy = halton(k, 2) - 0.5, halton(k, 3) - 0.5
        cur = self.frame_no & 1
        view_proj = np.asarray(cam.view_proj, np.float32)
        prev = self.prev_view_proj if self.prev_view_proj is not None else view_proj
        taa = taa_uniform(cam, size, prev, 0.1 if self.history_valid else 1.0)
        self.prev_view_proj = view_proj
        self.history_valid = True
        c = cam_uniform(cam, size, self.time, kmh / 3.6 * 0.12, (jx * 2 / size[0], -jy * 2 / size[1]))
        pd = None if parts is None else pdraw_uniform(cam, size, parts.shape[0], color_mode, smoke)
        sd = None if lines is None else sdraw_uniform(cam, size, lines.shape[0], color_mode, flow_time, vortices,
                                                      lines.shape[1])
        post = Post()
        post.bloom, post.exposure = 0.75, 1.0  # engine.ts:324
        return FrameUniforms(c, taa, cur, pd, sd, post, (jx, jy))


class Renderer:
    """Render targets of one view over an AeroEngine's lattice (engine.ts:290-306)."""

    def __init__(self, engine, width, height):
        self.engine = engine
        self.lib = engine.lib
        self.size = (int(width), int(height))
        self.half = (max(1, width >> 1), max(1, height >> 1))
        r = ctypes.c_void_p()
        engine._check(self.lib.wt_render_create(engine.ctx, width, height, ctypes.byref(r)), "wt_render_create")
        self.r = r
        self.state = FrameState()

    def close(self):
        if getattr(self, "r", None):
            self.lib.wt_render_destroy(self.r)
            self.r = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        self.engine._check(rc, what)

    # -- single passes -------------------------------------------------------
    def scene(self, cam, look, view):
        self._check(self.lib.wt_render_scene(self.r, ctypes.byref(cam), ctypes.byref(look), ctypes.byref(view)),
                    "wt_render_scene")

    def taa(self, taa, cur):
        self._check(self.lib.wt_render_taa(self.r, ctypes.byref(taa), cur), "wt_render_taa")

    def glow(self, parts=None, pdraw=None, pts=None, sdraw=None):
        """parts: [count, 8] float32 (host); pts: [lines, steps, 4] float32 (host)."""
        pp = None if parts is None else np.ascontiguousarray(parts, np.float32)
        sp = None if pts is None else np.ascontiguousarray(pts, np.float32)
        self._check(self.lib.wt_render_glow(self.r, None if pp is None else pp.ctypes.data, 0,
                                            None if pdraw is None else ctypes.byref(pdraw),
                                            None if sp is None else sp.ctypes.data, 0,
                                            None if sdraw is None else ctypes.byref(sdraw)), "wt_render_glow")

    def bloom(self):
        self._check(self.lib.wt_render_bloom(self.r), "wt_render_bloom")

    def present(self, post, cur):
        self._check(self.lib.wt_render_present(self.r, ctypes.byref(post), cur), "wt_render_present")

    def _shape(self, target):
        w, h = self.half if target in (TARGET_BLOOM_A, TARGET_BLOOM_B) else self.size
        return (h, w, 4), (np.uint8 if target in (TARGET_OUTPUT, TARGET_GMATERIAL) else np.float16)

    def read(self, target):
        """A target as [h, w, 4]: float16 for the float targets, uint8 for the output
        and the G-buffer's material target."""
        shape, dt = self._shape(target)
        out = np.empty(shape, dt)
        self._check(self.lib.wt_render_read(self.r, target, out.ctypes.data), "wt_render_read")
        return out

    def write(self, target, data):
        shape, dt = self._shape(target)
        arr = np.ascontiguousarray(data, dt).reshape(shape)
        self._check(self.lib.wt_render_write(self.r, target, arr.ctypes.data), "wt_render_write")

    def mesh(self, mesh_car, cam, rig, gurney=False):
        """The car mesh G-buffer pass (engine.ts:716): mesh_car a mesh_car.MeshCar,
        cam its MeshCam uniform, rig the [87, 4] Rig uniform."""
        mesh_car.record(self, cam, rig, gurney)

    # -- the frame's render passes (engine.ts:575-584, 660-725) ----------------
    def frame(self, cam, look, view, dt=1.0 / 60, kmh=250.0, parts=None, color_mode=0, smoke=True, lines=None,
              flow_time=0.0, vortices=False, mesh=None, rig=None, params=None):
        """Scene, TAA resolve, glow (particles and/or streamlines), bloom and
        present; returns the FrameUniforms used (u.cur = the history resolved into).
        With a car mesh (mesh_car.MeshCar, its Rig uniform and the ShapeParams of
        the W17 scene) the G-buffer pass runs first and the scene pass takes the
        car's surfaces from it (meshMode, engine.ts:679-686, 703, 716)."""
        u = self.state.next(cam, self.size, dt, kmh, parts, color_mode, smoke, lines, flow_time, vortices)
        if mesh is not None:
            from .mesh_car import mesh_cam
            self.mesh(mesh, mesh_cam(cam, self.size, u.halton, params), rig, bool(getattr(params, "gurney", False)))
            look = Look.from_buffer_copy(look)
            look.mesh_mode = 1
        self.scene(u.cam, look, view)
        self.taa(u.taa, u.cur)
        self.glow(parts, u.pdraw, lines, u.sdraw)
        self.bloom()
        self.present(u.post, u.cur)
        return u
