"""TEST INFRASTRUCTURE ONLY - ctypes wrappers of the oracle (oracle/_build/liboracle.so)
and, where it was built, of the translated reference shaders (oracle/_ref/libwgslref.so).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libwgslref.so")
REF_SRC = os.path.join(HERE, "_ref", "wgsl_modules.inc")
# the reference checkout the translator reads (only where it is present)
REFERENCE_ROOT = os.environ.get("WT_REFERENCE_ROOT", "/root/reference")
_vp = ctypes.c_void_p
_F = ctypes.c_float


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE, "_build/liboracle.so"], check=True)
    return ORACLE_SO


def build_ref():
    """Compile the translated reference if its generated source is present."""
    if os.path.exists(REF_SRC) or os.path.isdir(REFERENCE_ROOT):
        r = subprocess.run(["make", "-s", "-C", HERE, "ref"], capture_output=True, text=True)
        return os.path.exists(REF_SO) and r.returncode == 0
    return False


def _load_oracle():
    if not os.path.exists(ORACLE_SO):
        build_oracle()
    L = ctypes.CDLL(ORACLE_SO)
    L.wto_new.restype = _vp
    L.wto_new.argtypes = [ctypes.c_int] * 3 + [_F] * 4 + [ctypes.c_int]
    L.wto_free.argtypes = [_vp]
    L.wto_set_params.argtypes = [_vp, _vp]
    L.wto_reset.argtypes = [_vp]
    L.wto_voxelize.argtypes = [_vp, _vp]
    L.wto_set_solid.argtypes = [_vp, _vp, _vp]
    L.wto_steps.argtypes = [_vp, ctypes.c_int]
    L.wto_heat.argtypes = [_vp, _F]
    L.wto_read.argtypes = [_vp] + [_vp] * 7 + [ctypes.c_int]
    L.wto_read64.argtypes = [_vp, _vp, _vp]
    L.wto_write_state.argtypes = [_vp, _vp, _vp, _vp]
    L.wto_link_mask.argtypes = [_vp, _vp]
    L.wto_guarded.restype = ctypes.c_uint64
    L.wto_guarded.argtypes = [_vp]
    L.wto_threads.restype = ctypes.c_int
    L.wto_set_threads.argtypes = [ctypes.c_int]
    return L


def _load_ref():
    if not os.path.exists(REF_SO) and not build_ref():
        return None
    L = ctypes.CDLL(REF_SO)
    L.wtr_new.restype = _vp
    L.wtr_new.argtypes = [ctypes.c_int] * 3 + [_F] * 4
    L.wtr_free.argtypes = [_vp]
    L.wtr_set_sim.argtypes = [_vp, _F, _F, _F]
    L.wtr_set_heat.argtypes = [_vp, _F, _F]
    L.wtr_reset.argtypes = [_vp]
    L.wtr_voxelize.argtypes = [_vp, _vp]
    L.wtr_set_solid.argtypes = [_vp, _vp, _vp]
    L.wtr_steps.argtypes = [_vp, ctypes.c_int]
    L.wtr_heat.argtypes = [_vp, _F]
    L.wtr_read.argtypes = [_vp] + [_vp] * 6 + [ctypes.c_int]
    L.wtr_write_state.argtypes = [_vp, _vp, _vp, _vp]
    L.wtr_threads.restype = ctypes.c_int
    L.wtr_sample_flow.argtypes = [_vp, _vp, _F, _vp, _vp, _vp, ctypes.c_uint32, _vp, _vp]
    L.wtr_particles.argtypes = [_vp, _vp, _F, _vp, _vp, _vp, _vp, _vp, _vp]
    L.wtr_streamlines.argtypes = [_vp, _vp, _F, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    _i = ctypes.c_int
    L.wtr_render_scene.argtypes = [_vp, _vp, _F, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp]
    L.wtr_taa.argtypes = [_vp, _vp, _i, _i, _vp, _vp]
    L.wtr_blur.argtypes = [_vp, _i, _i, _vp, _i, _i, _vp]
    L.wtr_present.argtypes = [_vp, _i, _i, _vp, _i, _i, _vp, _i, _i, _vp, _vp]
    L.wtr_glow.argtypes = [_vp, _i, _i, _vp, _vp, ctypes.c_uint32, _vp, _vp, ctypes.c_uint32, _vp]
    L.wtr_scene_sdf.argtypes = [_vp, _vp, ctypes.c_uint32, _vp]
    L.wtr_set_car.argtypes = [_vp, _vp, _vp, _vp]
    L.wtr_set_gbuffer.argtypes = [_i, _i, _vp, _vp, _vp]
    L.wtr_mesh_gbuffer.argtypes = [_i, _i, _vp, ctypes.c_uint32, _vp, ctypes.c_uint32, _vp, _vp, _i, _i, _vp, _vp,
                                   _vp, _vp, _vp, _vp, _vp, _vp]
    return L


SHADE_SO = os.path.join(HERE, "_build", "libshadehm.so")
_S = None


def shade_model_lib():
    """The renderer's device shading code built for the host (shade_host_model.cpp),
    or None where it cannot be built (no CUDA headers)."""
    global _S
    if _S is None:
        r = subprocess.run(["make", "-s", "-C", HERE, "_build/libshadehm.so"], capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(SHADE_SO):
            return None
        L = ctypes.CDLL(SHADE_SO)
        L.wthm_render.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _F, _vp, _vp] + [ctypes.c_uint32] * 4 + [_vp]
        L.wthm_scene_sdf.argtypes = [_vp, _vp, ctypes.c_uint32, _vp]
        L.wthm_set_car.argtypes = [_vp, _vp, _vp, _vp]
        L.wthm_set_gbuffer.argtypes = [_vp, _vp, _vp]
        _S = L
    return _S


_SCAR = None


def shade_model_set_car(car):
    """Bind a W17 model (windtunnel.car_model.CarModel) to the host-built shading code, or None."""
    global _SCAR
    L = shade_model_lib()
    if car is None:
        L.wthm_set_car(None, None, None, None)
        _SCAR = None
        return
    keep = (np.ascontiguousarray(car.body_sdf, np.uint16), np.ascontiguousarray(car.parts, np.uint16),
            np.array(car.parts_dims, np.uint32), np.ascontiguousarray(car.rig, np.float32))
    L.wthm_set_car(*(a.ctypes.data for a in keep))
    _SCAR = keep


_SGB = None


def shade_model_set_gbuffer(albedo, normal, material):
    """Bind the car G-buffer ([h, w, 4] float16, float16, uint8) to the host-built
    shading code, or unbind it with None."""
    global _SGB
    L = shade_model_lib()
    if albedo is None:
        L.wthm_set_gbuffer(None, None, None)
        _SGB = None
        return
    keep = (np.ascontiguousarray(albedo, np.float16).view(np.uint16), np.ascontiguousarray(normal, np.float16)
            .view(np.uint16), np.ascontiguousarray(material, np.uint8))
    L.wthm_set_gbuffer(*(a.ctypes.data for a in keep))
    _SGB = keep


def shade_model_render(shape, cam, look, view, dims, origin, h, fields, temps, width, height, threads=1, rows=None):
    """RENDER fs_main of the device code on the host: [height, width, 4] float32
    (colour, hit distance) for the given rows (default all), one row per task
    over `threads` host threads."""
    import concurrent.futures as cf
    L = shade_model_lib()
    d = np.ascontiguousarray(dims, np.uint32)
    o = np.ascontiguousarray(origin, np.float32)
    f = np.ascontiguousarray(fields, np.float32)
    t = np.ascontiguousarray(temps, np.float32)
    out = np.zeros((height, width, 4), np.float32)

    def run(y):
        L.wthm_render(ctypes.addressof(shape), ctypes.addressof(cam), ctypes.addressof(look), ctypes.addressof(view),
                      d.ctypes.data, o.ctypes.data, float(h), f.ctypes.data, t.ctypes.data, width, height,
                      int(y), int(y) + 1, out.ctypes.data)

    with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        list(ex.map(run, range(height) if rows is None else rows))
    return out


_O = None
_R = None


def oracle_lib():
    global _O
    if _O is None:
        _O = _load_oracle()
    return _O


def ref_lib():
    global _R
    if _R is None:
        _R = _load_ref()
    return _R


def _grid_args(dims, origin, h):
    return (np.ascontiguousarray(dims, np.uint32), np.ascontiguousarray(origin, np.float32), float(h))


def ref_sample_flow(dims, origin, h, fields, temps, points):
    """The reference's sampleFlow / vorticityAt at points [n, 3] over fields [n, 4], temps [n]."""
    L = ref_lib()
    d, o, hh = _grid_args(dims, origin, h)
    f = np.ascontiguousarray(fields, np.float32)
    t = np.ascontiguousarray(temps, np.float32)
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.zeros((p.shape[0], 6), np.float32)
    vort = np.zeros(p.shape[0], np.float32)
    L.wtr_sample_flow(d.ctypes.data, o.ctypes.data, ctypes.c_float(hh), f.ctypes.data, t.ctypes.data, p.ctypes.data,
                      p.shape[0], out.ctypes.data, vort.ctypes.data)
    return out, vort


def ref_particles(dims, origin, h, fields, temps, psim, view, parts):
    """One reference particle pass; parts [count, 8] float32 updated in place."""
    L = ref_lib()
    d, o, hh = _grid_args(dims, origin, h)
    ps = np.array([psim.count, psim.spawn_mode, psim.color_mode, psim.frame, psim.scatter, psim.rake_rows,
                   psim.rake_cols], np.uint32)
    pf = np.array([psim.dt, psim.life, *psim.spawn_min, *psim.spawn_max], np.float32)
    vw = np.array([getattr(view, k) for k, _ in view._fields_], np.float32)
    f = np.ascontiguousarray(fields, np.float32)
    t = np.ascontiguousarray(temps, np.float32)
    assert parts.dtype == np.float32 and parts.flags.c_contiguous
    L.wtr_particles(d.ctypes.data, o.ctypes.data, ctypes.c_float(hh), f.ctypes.data, t.ctypes.data, ps.ctypes.data,
                    pf.ctypes.data, vw.ctypes.data, parts.ctypes.data)
    return parts


def ref_streamlines(dims, origin, h, fields, temps, params, view):
    L = ref_lib()
    d, o, hh = _grid_args(dims, origin, h)
    ss = np.array([params.lines, params.steps, params.seed_mode, params.color_mode, params.rows, params.cols,
                   params.per_emitter, params.emitters], np.uint32)
    sf = np.array([*params.seed_min, *params.seed_max, params.step_len, params.time], np.float32)
    em = np.array([[params.emitter[e][k] for k in range(4)] for e in range(8)], np.float32)
    vw = np.array([getattr(view, k) for k, _ in view._fields_], np.float32)
    f = np.ascontiguousarray(fields, np.float32)
    t = np.ascontiguousarray(temps, np.float32)
    out = np.zeros((params.lines, params.steps, 4), np.float32)
    L.wtr_streamlines(d.ctypes.data, o.ctypes.data, ctypes.c_float(hh), f.ctypes.data, t.ctypes.data, ss.ctypes.data,
                      sf.ctypes.data, em.ctypes.data, vw.ctypes.data, out.ctypes.data)
    return out


# ---- render passes (src/engine/render-wgsl.ts) through the translated shaders.
# Uniform arguments are the ctypes structs of windtunnel._abi (Cam, Look, Taa,
# PDraw, SDraw, Post), whose layouts are the WGSL uniforms'.  Targets are float32
# arrays [h, w, 4] holding binary16-rounded values; the output is uint8.
def _addr(st):
    return ctypes.addressof(st)


def ref_render_scene(dims, origin, h, fields, temps, shape, cam, look, view, width, height):
    L = ref_lib()
    d, o, hh = _grid_args(dims, origin, h)
    f = np.ascontiguousarray(fields, np.float32)
    t = np.ascontiguousarray(temps, np.float32)
    w = shape_words(shape)[:24].copy()
    out = np.zeros((height, width, 4), np.float32)
    L.wtr_render_scene(d.ctypes.data, o.ctypes.data, ctypes.c_float(hh), f.ctypes.data, t.ctypes.data, w.ctypes.data,
                       _addr(cam), _addr(look), _addr(view), width, height, out.ctypes.data)
    return out


def ref_scene_sdf(shape, pts):
    """The reference's sceneSdf at points [n, 3]: [n, 2] (distance, material)."""
    L = ref_lib()
    w = shape_words(shape)[:24].copy()
    p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    out = np.zeros((p.shape[0], 2), np.float32)
    L.wtr_scene_sdf(w.ctypes.data, p.ctypes.data, p.shape[0], out.ctypes.data)
    return out


_GB = None


def ref_set_gbuffer(albedo, normal, material):
    """Bind the car G-buffer ([h, w, 4] float16, float16, uint8, as the render
    targets store them) to the translated RENDER shader, or unbind it with None."""
    global _GB
    L = ref_lib()
    if albedo is None:
        L.wtr_set_gbuffer(1, 1, None, None, None)
        _GB = None
        return
    h, w = albedo.shape[:2]
    keep = (np.ascontiguousarray(albedo, np.float16).astype(np.float32),
            np.ascontiguousarray(normal, np.float16).astype(np.float32),
            np.ascontiguousarray(material, np.uint8).astype(np.float32) / np.float32(255.0))
    L.wtr_set_gbuffer(w, h, *(a.ctypes.data for a in keep))
    _GB = keep


def ref_mesh_gbuffer(data, cam, rig, width, height, gurney=False):
    """The reference's MESH_DRAW shaders over a car mesh (windtunnel.mesh_car.MeshData)
    in the restated WebGPU pipeline: the cleared G-buffer after the draws, as
    (albedo [h, w, 4] float16, normal-distance float16, material uint8, depth float32)."""
    from windtunnel.mesh_car import draw_words
    L = ref_lib()
    v = np.ascontiguousarray(data.verts, np.float32)
    i = np.ascontiguousarray(data.indices, np.uint32)
    t = np.zeros((data.tags.size + 3) // 4 * 4, np.uint8)
    t[:data.tags.size] = data.tags
    words = np.ascontiguousarray(draw_words(data, gurney))
    texs = [np.ascontiguousarray(rgba, np.uint8) for (_, _, rgba) in data.textures]
    dims = np.array([[w, h] for (w, h, _) in data.textures] or [[0, 0]], np.uint32)
    ptrs = (ctypes.c_void_p * max(1, len(texs)))(*[a.ctypes.data for a in texs])
    cw = np.frombuffer(bytes(cam), np.float32).copy()
    r = np.ascontiguousarray(rig, np.float32)
    albedo = np.zeros((height, width, 4), np.float32)
    normal = np.zeros((height, width, 4), np.float32)
    material = np.zeros((height, width, 4), np.uint8)
    depth = np.ones((height, width), np.float32)
    L.wtr_mesh_gbuffer(width, height, v.ctypes.data, v.shape[0], i.ctypes.data, i.size, t.ctypes.data,
                       words.ctypes.data, words.shape[0], len(texs), dims.ctypes.data, ptrs, cw.ctypes.data,
                       r.ctypes.data, albedo.ctypes.data, normal.ctypes.data, material.ctypes.data, depth.ctypes.data)
    return albedo.astype(np.float16), normal.astype(np.float16), material, depth


_CAR = None


def ref_set_car(car):
    """Bind a W17 model (windtunnel.car_model.CarModel: body SDF, parts atlas, rig)
    to the translated reference, or unbind it with None."""
    global _CAR
    L = ref_lib()
    if car is None:
        L.wtr_set_car(None, None, None, None)
        _CAR = None
        return
    sdf = np.ascontiguousarray(car.body_sdf, np.uint16)
    parts = np.ascontiguousarray(car.parts, np.uint16)
    dims = np.array(car.parts_dims, np.uint32)
    rig = np.ascontiguousarray(car.rig, np.float32).reshape(87, 4)
    L.wtr_set_car(sdf.ctypes.data, parts.ctypes.data, dims.ctypes.data, rig.ctypes.data)
    _CAR = (sdf, parts, dims, rig)


def ref_taa(cur, hist, taa):
    L = ref_lib()
    cur = np.ascontiguousarray(cur, np.float32)
    hist = np.ascontiguousarray(hist, np.float32)
    hgt, w = cur.shape[:2]
    out = np.zeros_like(cur)
    L.wtr_taa(cur.ctypes.data, hist.ctypes.data, w, hgt, _addr(taa), out.ctypes.data)
    return out


def ref_blur(src, dir_xy, spacing, gain, dw, dh):
    L = ref_lib()
    src = np.ascontiguousarray(src, np.float32)
    b = np.array([dir_xy[0], dir_xy[1], spacing, gain], np.float32)
    out = np.zeros((dh, dw, 4), np.float32)
    L.wtr_blur(src.ctypes.data, src.shape[1], src.shape[0], b.ctypes.data, dw, dh, out.ctypes.data)
    return out


def ref_present(scene, glow, bloom, post):
    L = ref_lib()
    scene, glow, bloom = (np.ascontiguousarray(a, np.float32) for a in (scene, glow, bloom))
    out = np.zeros(scene.shape, np.uint8)
    L.wtr_present(scene.ctypes.data, scene.shape[1], scene.shape[0], glow.ctypes.data, glow.shape[1], glow.shape[0],
                  bloom.ctypes.data, bloom.shape[1], bloom.shape[0], _addr(post), out.ctypes.data)
    return out


def ref_glow(scene, parts=None, pdraw=None, pts=None, sdraw=None):
    """The glow pass: particle quads (2 * count instances) and streamline quads
    (lines * 2 * (steps - 1) instances) added into a cleared target."""
    L = ref_lib()
    scene = np.ascontiguousarray(scene, np.float32)
    hgt, w = scene.shape[:2]
    out = np.zeros_like(scene)
    pp = None if parts is None else np.ascontiguousarray(parts, np.float32)
    sp = None if pts is None else np.ascontiguousarray(pts, np.float32)
    n_p = 0 if pp is None else 2 * pdraw.count
    n_s = 0 if sp is None else sdraw.lines * 2 * (sdraw.steps - 1)
    L.wtr_glow(scene.ctypes.data, w, hgt, None if pp is None else pp.ctypes.data,
               None if pp is None else _addr(pdraw), n_p, None if sp is None else sp.ctypes.data,
               None if sp is None else _addr(sdraw), n_s, out.ctypes.data)
    return out


def shape_words(shape) -> np.ndarray:
    """The 30 32-bit words of a wt_shape (ctypes struct) as uint32."""
    return np.frombuffer(bytes(shape), dtype=np.uint32).copy()


class Oracle:
    """CPU restatement of the tunnel path (wt_oracle.hpp); fp64=True gives the FP64 model."""

    def __init__(self, dims, origin, h, sim=None, fp64=False):
        self.L = oracle_lib()
        self.dims = tuple(int(d) for d in dims)
        self.n = int(np.prod(self.dims))
        self.h = float(h)
        self.p = self.L.wto_new(*self.dims, float(origin[0]), float(origin[1]), float(origin[2]), float(h),
                                1 if fp64 else 0)
        if sim is not None:
            self.set_sim(sim)

    def set_sim(self, sim):
        prm = np.array([sim.u_in, sim.tau0, sim.smag, sim.sponge_cells, sim.sponge_amp, sim.inlet_cells,
                        sim.inlet_amp, sim.heat_cool, sim.heat_diffuse, sim.heat_src_mix], np.float32)
        self.L.wto_set_params(self.p, prm.ctypes.data)

    def reset(self):
        self.L.wto_reset(self.p)

    def voxelize(self, shape):
        w = shape_words(shape)
        self.L.wto_voxelize(self.p, w.ctypes.data)

    def set_solid(self, solid, emit):
        s = np.ascontiguousarray(solid, np.uint32)
        e = np.ascontiguousarray(emit, np.float32)
        self.L.wto_set_solid(self.p, s.ctypes.data, e.ctypes.data)

    def steps(self, n):
        self.L.wto_steps(self.p, int(n))

    def heat(self, dt):
        self.L.wto_heat(self.p, float(dt))

    def frame(self, steps=8, heat_passes=2):
        self.steps(steps)
        if heat_passes:
            assert heat_passes == 2
            self.heat(steps / 2.0)

    def read(self, reset_forces=False):
        n = self.n
        out = dict(fields=np.zeros((n, 4), np.float32), solid=np.zeros(n, np.uint32), emit=np.zeros(n, np.float32),
                   temps=np.zeros(n, np.float32), f=np.zeros(19 * n, np.float32), forces=np.zeros(12, np.int32),
                   forces64=np.zeros(9, np.float64))
        self.L.wto_read(self.p, out["fields"].ctypes.data, out["solid"].ctypes.data, out["emit"].ctypes.data,
                        out["temps"].ctypes.data, out["f"].ctypes.data, out["forces"].ctypes.data,
                        out["forces64"].ctypes.data, 1 if reset_forces else 0)
        return out

    def read64(self):
        fields = np.zeros((self.n, 4), np.float64)
        f = np.zeros(19 * self.n, np.float64)
        self.L.wto_read64(self.p, fields.ctypes.data, f.ctypes.data)
        return fields, f

    def write_state(self, f=None, fields=None, temps=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (f, fields, temps)]
        self.L.wto_write_state(self.p, *[None if a is None else a.ctypes.data for a in arrs])

    def link_mask(self):
        m = np.zeros(self.n, np.uint32)
        self.L.wto_link_mask(self.p, m.ctypes.data)
        return m

    def guarded(self):
        return int(self.L.wto_guarded(self.p))

    def __del__(self):
        try:
            self.L.wto_free(self.p)
        except Exception:
            pass


class Reference:
    """The reference's own WGSL shaders compiled as C++ (oracle/_ref), f32 only."""

    def __init__(self, dims, origin, h, sim=None):
        self.L = ref_lib()
        if self.L is None:
            raise RuntimeError("oracle/_ref was not built (needs the reference checkout)")
        self.dims = tuple(int(d) for d in dims)
        self.n = int(np.prod(self.dims))
        self.p = self.L.wtr_new(*self.dims, float(origin[0]), float(origin[1]), float(origin[2]), float(h))
        if sim is not None:
            self.L.wtr_set_sim(self.p, sim.u_in, sim.tau0, sim.smag)
            self.L.wtr_set_heat(self.p, sim.heat_cool, sim.heat_diffuse)

    def reset(self):
        self.L.wtr_reset(self.p)

    def voxelize(self, shape):
        w = shape_words(shape)[:24].copy()
        self.L.wtr_voxelize(self.p, w.ctypes.data)

    def set_solid(self, solid, emit):
        s = np.ascontiguousarray(solid, np.uint32)
        e = np.ascontiguousarray(emit, np.float32)
        self.L.wtr_set_solid(self.p, s.ctypes.data, e.ctypes.data)

    def steps(self, n):
        self.L.wtr_steps(self.p, int(n))

    def heat(self, dt):
        self.L.wtr_heat(self.p, float(dt))

    def frame(self, steps=8, heat_passes=2):
        self.steps(steps)
        if heat_passes:
            self.heat(steps / 2.0)

    def read(self, reset_forces=False):
        n = self.n
        out = dict(fields=np.zeros((n, 4), np.float32), solid=np.zeros(n, np.uint32), emit=np.zeros(n, np.float32),
                   temps=np.zeros(n, np.float32), f=np.zeros(19 * n, np.float32), forces=np.zeros(12, np.int32))
        self.L.wtr_read(self.p, out["fields"].ctypes.data, out["solid"].ctypes.data, out["emit"].ctypes.data,
                        out["temps"].ctypes.data, out["f"].ctypes.data, out["forces"].ctypes.data,
                        1 if reset_forces else 0)
        return out

    def write_state(self, f=None, fields=None, temps=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (f, fields, temps)]
        self.L.wtr_write_state(self.p, *[None if a is None else a.ctypes.data for a in arrs])

    def __del__(self):
        try:
            self.L.wtr_free(self.p)
        except Exception:
            pass
