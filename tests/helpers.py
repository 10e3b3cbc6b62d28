"""Shared helpers of the tests: replaying the golden scripts on the oracle or on libwt."""
import hashlib
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def shape_from_dict(d):
    from windtunnel import _abi
    s = _abi.Shape()
    for name, _ in s._fields_:
        v = d[name]
        if isinstance(v, list):
            arr = getattr(s, name)
            for k, x in enumerate(v):
                arr[k] = x
        else:
            setattr(s, name, v)
    return s


def golden_shapes(man):
    return {name: shape_from_dict(c["shape"]) for name, c in man["vox"].items()}


def corrupt(f, n, cells):
    f = f.copy()
    cells = np.asarray(cells)
    f[3 * n + cells[:4]] = np.nan
    f[1 * n + cells[4:8]] = 50.0
    f[7 * n + cells[8:]] = -40.0
    return f


def replay(sim_obj, man, case, read):
    """Run the golden script of `case` on an object with voxelize/frame/read/write_state.
    `read()` returns dict(fields, f, temps, forces).  Yields (frame_index, data)."""
    rec = man["lbm"][case]
    shapes = golden_shapes(man)
    k = 0
    for item in rec["script"]:
        if item[0] == "shape":
            sim_obj.voxelize(shapes[item[1]])
        elif item[0] == "corrupt":
            d = read()
            n = d["fields"].shape[0]
            sim_obj.write_state(f=corrupt(d["f"], n, item[2]))
        else:
            sim_obj.frame(item[1])
            yield k, read()
            k += 1


def shade_host_model():
    """The renderer's per-pixel device code built for the host
    (tests/cuda/shade_host_model.cpp) as a ctypes library, or None where g++ or
    the CUDA headers are missing.  Cached in the temp directory by source hash."""
    import ctypes
    import shutil
    import subprocess
    import tempfile
    src = os.path.join(ROOT, "tests", "cuda", "shade_host_model.cpp")
    csrc = os.path.join(ROOT, "f1-wind-tunnel_gb300", "csrc")
    cuda_inc = None
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(cand, "include")
            break
    gxx = shutil.which("g++")
    if cuda_inc is None or gxx is None:
        return None
    h = hashlib.sha256()
    for f in [src, os.path.join(ROOT, "include", "wt.h")] + sorted(
            os.path.join(csrc, n) for n in os.listdir(csrc) if n.endswith((".cuh", ".h"))):
        h.update(open(f, "rb").read())
    so = os.path.join(tempfile.gettempdir(), f"wt_shade_host_model_{h.hexdigest()[:16]}.so")
    if not os.path.exists(so):
        tmp = so + f".{os.getpid()}.tmp"
        subprocess.run([gxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                        "-I", os.path.join(ROOT, "include"), "-I", csrc, "-I", cuda_inc, "-o", tmp, src], check=True)
        os.replace(tmp, so)
    L = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    L.wthm_render.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.c_float, vp, vp, ctypes.c_uint32, ctypes.c_uint32, vp]
    L.wthm_scene_sdf.argtypes = [vp, vp, ctypes.c_uint32, vp]
    return L
