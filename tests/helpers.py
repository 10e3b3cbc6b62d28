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
    (oracle/shade_host_model.cpp) as a ctypes library, or None where the CUDA
    headers are missing."""
    from oracle import pyoracle
    return pyoracle.shade_model_lib()


def same_half(a, b):
    """binary16 arrays equal bit for bit, except that any NaN equals any NaN (the
    payload a NaN gets when rounded to binary16 is the implementation's)."""
    a = np.ascontiguousarray(a, np.float16)
    b = np.ascontiguousarray(b, np.float16)
    return (a.view(np.uint16) == b.view(np.uint16)) | (np.isnan(a) & np.isnan(b))
