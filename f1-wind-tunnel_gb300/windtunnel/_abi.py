"""ctypes view of libwt (include/wt.h).

The structures mirror the C header field for field; `load()` opens the
in-tree build (f1-wind-tunnel_gb300/_build/libwt.so).  There is no fallback:
if the library is missing or the device is not an sm_103a GPU, calls fail with
WindTunnelError.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libwt.so")

WT_OK = 0
ERRORS = {
    -1: "WT_ERR_ARG",
    -2: "WT_ERR_CUDA",
    -3: "WT_ERR_NOMEM",
    -4: "WT_ERR_UNSUPPORTED",
    -5: "WT_ERR_STATE",
    -6: "WT_ERR_DEVICE",
}
STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2
STORAGE = {"f32": STORE_F32, "f16": STORE_F16, "bf16": STORE_BF16}
KIND_F1, KIND_SPHERE, KIND_CUBE, KIND_WING, KIND_W17, KIND_EMPTY, KIND_BOX = 0, 1, 2, 3, 5, 6, 7


class WindTunnelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32),
                ("origin", ctypes.c_float * 3), ("h", ctypes.c_float)]


class Sim(ctypes.Structure):
    _fields_ = [("u_in", ctypes.c_float), ("tau0", ctypes.c_float), ("smag", ctypes.c_float),
                ("sponge_cells", ctypes.c_float), ("sponge_amp", ctypes.c_float),
                ("inlet_cells", ctypes.c_float), ("inlet_amp", ctypes.c_float),
                ("heat_cool", ctypes.c_float), ("heat_diffuse", ctypes.c_float), ("heat_src_mix", ctypes.c_float),
                ("storage", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Shape(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("profile_mode", ctypes.c_uint32), ("pw", ctypes.c_uint32),
                ("ph", ctypes.c_uint32),
                ("front_flap", ctypes.c_float), ("rear_main", ctypes.c_float), ("rear_flap", ctypes.c_float),
                ("ride_h", ctypes.c_float),
                ("aoa", ctypes.c_float), ("width", ctypes.c_float), ("axis_y", ctypes.c_float),
                ("p_scale", ctypes.c_float),
                ("p_origin", ctypes.c_float * 2), ("heat_brakes", ctypes.c_float), ("heat_engine", ctypes.c_float),
                ("heat_rad", ctypes.c_float), ("front_wing", ctypes.c_float), ("rear_wing", ctypes.c_float),
                ("sidepod", ctypes.c_float),
                ("cover", ctypes.c_float), ("nose", ctypes.c_float), ("rear_ride", ctypes.c_float),
                ("duct", ctypes.c_float),
                ("box_center", ctypes.c_float * 3), ("box_half", ctypes.c_float * 3)]


class Forces(ctypes.Structure):
    _fields_ = [("raw", ctypes.c_int32 * 12), ("sum", ctypes.c_double * 9), ("mass", ctypes.c_double),
                ("steps", ctypes.c_uint64), ("guarded", ctypes.c_uint64)]


class Info(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64), ("steps_total", ctypes.c_uint64),
                ("storage", ctypes.c_uint32), ("fluid_cells", ctypes.c_uint32), ("solid_cells", ctypes.c_uint32 * 3),
                ("boundary_blocks", ctypes.c_uint32), ("history_capacity", ctypes.c_uint32),
                ("sm_count", ctypes.c_uint32)]


class View(ctypes.Structure):
    """View uniform (src/engine/wgsl.ts:431-434)."""
    _fields_ = [(n, ctypes.c_float) for n in ("u_in", "v_real", "cp_min", "cp_max", "t_min", "t_max", "speed_max",
                                               "vort_max")]


class PSim(ctypes.Structure):
    """PSim uniform (wgsl.ts:517-521) as plain C fields."""
    _fields_ = [("count", ctypes.c_uint32), ("spawn_mode", ctypes.c_uint32), ("color_mode", ctypes.c_uint32),
                ("frame", ctypes.c_uint32), ("dt", ctypes.c_float), ("life", ctypes.c_float),
                ("scatter", ctypes.c_uint32), ("rake_rows", ctypes.c_uint32), ("rake_cols", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("spawn_min", ctypes.c_float * 3), ("spawn_max", ctypes.c_float * 3)]


class StreamParams(ctypes.Structure):
    """Stream uniform and emitters (src/engine/render-wgsl.ts:521-527)."""
    _fields_ = [("lines", ctypes.c_uint32), ("steps", ctypes.c_uint32), ("seed_mode", ctypes.c_uint32),
                ("color_mode", ctypes.c_uint32), ("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32),
                ("per_emitter", ctypes.c_uint32), ("emitters", ctypes.c_uint32), ("seed_min", ctypes.c_float * 3),
                ("seed_max", ctypes.c_float * 3), ("step_len", ctypes.c_float), ("time", ctypes.c_float),
                ("emitter", (ctypes.c_float * 4) * 8)]


class CoefEma(ctypes.Structure):
    _fields_ = [("cd", ctypes.c_double), ("cl", ctypes.c_double), ("n", ctypes.c_uint32)]


class Sweep(ctypes.Structure):
    _fields_ = [("n_front", ctypes.c_uint32), ("n_rear", ctypes.c_uint32), ("front", ctypes.POINTER(ctypes.c_float)),
                ("rear", ctypes.POINTER(ctypes.c_float)), ("settle_steps", ctypes.c_uint32),
                ("measure_steps", ctypes.c_uint32), ("read_every", ctypes.c_uint32), ("kmh", ctypes.c_float)]


class SweepCell(ctypes.Structure):
    _fields_ = [("down_kg", ctypes.c_double), ("drag_n", ctypes.c_double), ("efficiency", ctypes.c_double),
                ("group_down_n", ctypes.c_double * 3), ("group_drag_n", ctypes.c_double * 3),
                ("order", ctypes.c_uint32), ("readings", ctypes.c_uint32)]


_F = ctypes.c_float
_U = ctypes.c_uint32


class Cam(ctypes.Structure):
    """Cam uniform (src/engine/render-wgsl.ts:5-11)."""
    _fields_ = [("pos", _F * 3), ("tan_half", _F), ("fwd", _F * 3), ("aspect", _F), ("right", _F * 3), ("time", _F),
                ("up", _F * 3), ("road_speed", _F), ("jitter", _F * 2), ("pad0", _F), ("pad1", _F)]


class Look(ctypes.Structure):
    """Look uniform (render-wgsl.ts:12-19)."""
    _fields_ = [("bmin", _F * 3), ("surf_mode", _U), ("bmax", _F * 3), ("palette", _U), ("paint", _F * 3),
                ("carbon_body", _U), ("accent", _F * 3), ("is_f1", _U), ("slice_axis", _U), ("slice_pos", _F),
                ("slice_alpha", _F), ("show_flow", _U), ("mesh_mode", _U), ("cooling", _U), ("pad1", _U),
                ("pad2", _U)]


class Taa(ctypes.Structure):
    """Taa uniform (render-wgsl.ts:457-463)."""
    _fields_ = [("prev_view_proj", _F * 16), ("cam_pos", _F * 3), ("tan_half", _F), ("fwd", _F * 3),
                ("aspect", _F), ("right", _F * 3), ("blend", _F), ("up", _F * 3), ("pad", _F)]


class PDraw(ctypes.Structure):
    """PDraw uniform (src/engine/wgsl.ts:598-603)."""
    _fields_ = [("view_proj", _F * 16), ("cam_pos", _F * 3), ("width", _F), ("res", _F * 2), ("trail", _F),
                ("alpha", _F), ("count", _U), ("palette", _U), ("fade_in", _F), ("pad", _F)]


class SDraw(ctypes.Structure):
    """SDraw uniform (render-wgsl.ts:579-584)."""
    _fields_ = [("view_proj", _F * 16), ("cam_pos", _F * 3), ("width", _F), ("res", _F * 2), ("time", _F),
                ("intensity", _F), ("lines", _U), ("steps", _U), ("palette", _U), ("pulse", _F)]


class Post(ctypes.Structure):
    """Post uniform (render-wgsl.ts:421)."""
    _fields_ = [("bloom", _F), ("exposure", _F), ("pad0", _F), ("pad1", _F)]


class MeshDraw(ctypes.Structure):
    """wt_mesh_draw: the MeshMat uniform (render-wgsl.ts:653-657), then count, texture, blend, optional."""
    _fields_ = [("color", _F * 4), ("metal", _F), ("rough", _F), ("coat", _F), ("alpha_cut", _F), ("emissive", _F),
                ("has_tex", _F), ("is_body", _F), ("first_index", _U), ("count", _U), ("texture", ctypes.c_int32),
                ("blend", _U), ("optional", _U)]


class MeshCam(ctypes.Structure):
    """MeshCam uniform (render-wgsl.ts:648-652)."""
    _fields_ = [("view_proj", _F * 16), ("cam_pos", _F * 3), ("ride_h", _F), ("jitter", _F * 2), ("rake", _F),
                ("base_ride", _F)]


(TARGET_SCENE, TARGET_HIST0, TARGET_HIST1, TARGET_GLOW, TARGET_BLOOM_A, TARGET_BLOOM_B, TARGET_OUTPUT,
 TARGET_GALBEDO, TARGET_GNORMAL, TARGET_GMATERIAL) = range(10)

_vp = ctypes.c_void_p
_PROTOS = {
    "wt_create": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(Sim), ctypes.POINTER(_vp)]),
    "wt_destroy": (ctypes.c_int, [_vp]),
    "wt_set_sim": (ctypes.c_int, [_vp, ctypes.POINTER(Sim)]),
    "wt_reset": (ctypes.c_int, [_vp]),
    "wt_voxelize": (ctypes.c_int, [_vp, ctypes.POINTER(Shape)]),
    "wt_set_solid": (ctypes.c_int, [_vp, _vp, _vp]),
    "wt_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "wt_read_forces": (ctypes.c_int, [_vp, ctypes.POINTER(Forces), ctypes.c_int]),
    "wt_read_force_history": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32]),
    "wt_read_forces_async": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]),
    "wt_forces_collect": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.POINTER(Forces)]),
    "wt_read_fields": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "wt_read_populations": (ctypes.c_int, [_vp, _vp]),
    "wt_write_state": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "wt_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "wt_load": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "wt_reset_from": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]),
    "wt_info_get": (ctypes.c_int, [_vp, ctypes.POINTER(Info)]),
    "wt_stream": (_vp, [_vp]),
    "wt_sync": (ctypes.c_int, [_vp]),
    "wt_last_error": (ctypes.c_char_p, [_vp]),
    "wt_tune": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "wt_batch_create": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.POINTER(Sim), ctypes.POINTER(_vp)]),
    "wt_batch_destroy": (ctypes.c_int, [_vp]),
    "wt_batch_count": (ctypes.c_uint32, [_vp]),
    "wt_batch_lattice": (_vp, [_vp, ctypes.c_uint32]),
    "wt_batch_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "wt_batch_tune": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "wt_batch_stream": (_vp, [_vp]),
    "wt_batch_persistent_grid": (ctypes.c_uint32, [_vp]),
    "wt_batch_last_error": (ctypes.c_char_p, [_vp]),
    "wt_version": (ctypes.c_char_p, []),
    "wt_read_coarse": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp]),
    "wt_sdf_sample": (ctypes.c_int, [ctypes.POINTER(Shape), ctypes.POINTER(Grid), _vp]),
    "wt_coef_ema_update": (None, [ctypes.POINTER(CoefEma), ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "wt_aeromap_sweep": (ctypes.c_int, [_vp, ctypes.POINTER(Shape), ctypes.POINTER(Sweep), _vp]),
    "wt_sample_flow": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, _vp, _vp]),
    "wt_particles_step": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.POINTER(PSim), ctypes.POINTER(View)]),
    "wt_streamlines": (ctypes.c_int, [_vp, ctypes.POINTER(StreamParams), ctypes.POINTER(View), _vp]),
    "wt_set_car_model": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "wt_render_create": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_vp)]),
    "wt_render_destroy": (None, [_vp]),
    "wt_render_scene": (ctypes.c_int, [_vp, ctypes.POINTER(Cam), ctypes.POINTER(Look), ctypes.POINTER(View)]),
    "wt_render_taa": (ctypes.c_int, [_vp, ctypes.POINTER(Taa), ctypes.c_int]),
    "wt_render_glow": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.POINTER(PDraw), _vp, ctypes.c_int,
                                      ctypes.POINTER(SDraw)]),
    "wt_render_bloom": (ctypes.c_int, [_vp]),
    "wt_render_present": (ctypes.c_int, [_vp, ctypes.POINTER(Post), ctypes.c_int]),
    "wt_render_read": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "wt_render_write": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "wt_mesh_create": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, _vp, ctypes.c_uint32, _vp, ctypes.POINTER(_vp)]),
    "wt_mesh_destroy": (None, [_vp]),
    "wt_mesh_add_texture": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                           ctypes.POINTER(ctypes.c_int32)]),
    "wt_mesh_add_draw": (ctypes.c_int, [_vp, ctypes.POINTER(MeshDraw)]),
    "wt_render_mesh": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(MeshCam), _vp, ctypes.c_int]),
    "wt_png_unfilter": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp]),
}

_lib = None


def load(path=None):
    """Open libwt.so and declare the prototypes.  Raises if it is not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise WindTunnelError(-6, f"{p} is missing: build it with `python f1-wind-tunnel_gb300/build.py`")
    lib = ctypes.CDLL(p)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(lib, ctx, rc, what):
    if rc != WT_OK:
        msg = lib.wt_last_error(ctx)
        raise WindTunnelError(rc, f"{what}: {msg.decode() if msg else ''}")
