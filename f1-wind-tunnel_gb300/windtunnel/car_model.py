"""The baked W17 car model the reference voxelizes and renders (scene kind 5):
a 368 x 84 x 67 r16float body SDF at 1.5 cm from (-0.3, 0, 0), per-part grids of
the articulated wing elements packed into one atlas, and the Rig uniform that
rotates them (src/engine/car-model.ts:22, 40-50, 56-136, 158-193;
src/engine/engine.ts:410-421 setCarModel, 450-462 the rig of setShape).

    model = load_w17("path/to/public/models", shape_params)   # the reference's asset files
    engine.set_car_model(model); engine.set_shape(shape_params)   # kind ShapeKind.W17

`synthetic_w17()` builds a stand-in with the same formats from simple analytic
shapes (numpy float64 with correctly rounded operations only, so the same bits
on every machine); the tests use it where the reference's assets are absent.
"""
import json
import math
import os
from dataclasses import dataclass

import numpy as np

SDF_DIMS = (368, 84, 67)          # car-model.ts:22 (x, y, z)
SDF_H = 0.015
SDF_ORIGIN = (-0.3, 0.0, 0.0)
PART_FAR = 0x2400                 # atlas padding: binary16 1/64 (car-model.ts:180)
FRONT_BINS = 71                   # RIG.front.bins (car-model.ts:47)
DEG = math.pi / 180.0
W17_FRONT_FLAP = [0, 7, -9]               # W17_FRONT_LEVELS[].flap (car-model.ts:140-143)
W17_REAR_LEVELS = [(0, 0), (3, 9), (-4, -13)]  # W17_REAR_LEVELS[] (main, flap) (car-model.ts:144-148)
REAR_SHAPE_TWIST = {0: 0.0, 1: -16.0, 2: 6.0}  # engine.ts:111
THIN_FLAP_SCALE = 0.72                      # engine.ts:112
COMPACT_POD_SQUEEZE = 0.32                  # engine.ts:113


@dataclass
class CarModel:
    body_sdf: np.ndarray   # [67, 84, 368] uint16 binary16 bits (z, y, x)
    parts: np.ndarray      # [nz, ny, nx] uint16 binary16 bits: the parts atlas
    parts_dims: tuple      # (nx, ny, nz)
    rig: np.ndarray        # [87, 4] float32: the Rig uniform
    rig_data: dict = None  # the rig JSON (w17.rig.json), so setShape can rebuild the Rig uniform


def rig_uniform(rig, angles, rear_twist=0.0, flap_scale=1.0, pod_squeeze=0.0, fly=(0.0, 0.0, 1.0, 1.0)):
    """rigUniform (car-model.ts:158-174) as the 87 vec4 of the Rig uniform:
    front[71], hinges, angles, extra, fly, grids[12]."""
    fh = rig["frontHinges"]
    front = [[a[0], a[1], fh[1][i][0], fh[1][i][1]] for i, a in enumerate(fh[0])]
    grids = []
    for g in rig["partGrids"]:
        grids.append([*g["origin"], g["h"]])
        grids.append([*g["dims"], 0])
    z = 0
    for i, g in enumerate(rig["partGrids"]):
        grids[i * 2 + 1][3] = z
        z += g["dims"][2] + 1
    grids += [[0, 0, 0, 1]] * max(0, 12 - len(grids))
    rows = (front + [[*rig["rearMainHinge"], *rig["rearFlapHinge"]], list(angles),
                     [rear_twist, flap_scale, pod_squeeze, 0], list(fly)] + grids)
    out = np.array(rows, np.float32)
    assert out.shape == (87, 4)
    return out


def parts_atlas(rig, data):
    """partsAtlas (car-model.ts:176-193): the part grids stacked along z with a
    padding slice between them.  Returns ([nz, ny, nx] uint16, (nx, ny, nz))."""
    grids = rig["partGrids"]
    nx = max(g["dims"][0] for g in grids)
    ny = max(g["dims"][1] for g in grids)
    nz = sum(g["dims"][2] + 1 for g in grids)
    out = np.full((nz, ny, nx), PART_FAR, np.uint16)
    data = np.asarray(data, np.uint16)
    z0 = 0
    for g in grids:
        gx, gy, gz = g["dims"]
        block = data[g["offset"]:g["offset"] + gx * gy * gz].reshape(gz, gy, gx)
        out[z0:z0 + gz, :gy, :gx] = block
        z0 += gz + 1
    return out, (nx, ny, nz)


def w17_rig(rig, p, fly_progress=(0.0, 0.0)):
    """The rig setShape derives for a W17 ShapeParams (engine.ts:450-462)."""
    front = W17_FRONT_FLAP[p.frontWing] if 0 <= p.frontWing < 3 else W17_FRONT_FLAP[0]
    rear_main, rear_flap = W17_REAR_LEVELS[p.rearWing] if 0 <= p.rearWing < 3 else W17_REAR_LEVELS[0]
    front_deg = p.frontFlapDeg + front
    angles = [front_deg * 0.8 * DEG, front_deg * DEG, (p.rearFlapDeg + rear_flap) * DEG,
              (rear_main + p.rearMainDeg) * DEG]
    return rig_uniform(rig, angles, REAR_SHAPE_TWIST.get(p.rearShape, 0.0) * DEG,
                       THIN_FLAP_SCALE if p.thinWings else 1.0, COMPACT_POD_SQUEEZE if p.sidepods == 1 else 0.0,
                       (fly_progress[0], fly_progress[1], 1.0 if p.frontWingOn else 0.0,
                        1.0 if p.rearWingOn else 0.0))


def load_w17(models_dir, p, fly_progress=(0.0, 0.0)):
    """The reference's W17 assets (w17.sdf.bin, w17.parts.bin, w17.rig.json) as a
    CarModel with the rig of ShapeParams p."""
    sx, sy, sz = SDF_DIMS
    sdf = np.fromfile(os.path.join(models_dir, "w17.sdf.bin"), np.uint16)
    assert sdf.size == sx * sy * sz
    with open(os.path.join(models_dir, "w17.rig.json")) as f:
        rig = json.load(f)
    atlas, dims = parts_atlas(rig, np.fromfile(os.path.join(models_dir, "w17.parts.bin"), np.uint16))
    return CarModel(sdf.reshape(sz, sy, sx), atlas, dims, w17_rig(rig, p, fly_progress), rig)


# ---------------------------------------------------------------- synthetic stand-in
def _round_box(px, py, pz, c, b, r):
    qx = np.abs(px - c[0]) - (b[0] - r)
    qy = np.abs(py - c[1]) - (b[1] - r)
    qz = np.abs(pz - c[2]) - (b[2] - r)
    out = np.sqrt(np.maximum(qx, 0) ** 2 + np.maximum(qy, 0) ** 2 + np.maximum(qz, 0) ** 2)
    return out + np.minimum(np.maximum(qx, np.maximum(qy, qz)), 0) - r


def _capsule(px, py, pz, a, b, r):
    ba = np.array(b, np.float64) - np.array(a, np.float64)
    pax, pay, paz = px - a[0], py - a[1], pz - a[2]
    h = np.clip((pax * ba[0] + pay * ba[1] + paz * ba[2]) / float(ba @ ba), 0.0, 1.0)
    dx, dy, dz = pax - ba[0] * h, pay - ba[1] * h, paz - ba[2] * h
    return np.sqrt(dx * dx + dy * dy + dz * dz) - r


def _grid(origin, h, dims):
    i = origin[0] + np.arange(dims[0], dtype=np.float64) * h
    j = origin[1] + np.arange(dims[1], dtype=np.float64) * h
    k = origin[2] + np.arange(dims[2], dtype=np.float64) * h
    return np.meshgrid(i, j, k, indexing="ij")


def _to_half_bits(d):
    """[x, y, z] float64 distances -> [z, y, x] binary16 bits (round to nearest even)."""
    return np.ascontiguousarray(np.transpose(d.astype(np.float16), (2, 1, 0))).view(np.uint16)


def synthetic_rig_data():
    """Rig JSON fields of the stand-in: six part grids at 1 cm (front flaps A
    and B, rear flap and main plane, front and rear static parts), front-flap
    hinges that climb along the span, rear hinges."""
    grids = [
        {"part": 1, "origin": [0.22, 0.16, 0.10], "h": 0.01, "dims": [36, 14, 50]},
        {"part": 2, "origin": [0.36, 0.22, 0.10], "h": 0.01, "dims": [30, 14, 50]},
        {"part": 3, "origin": [4.70, 0.94, 0.00], "h": 0.01, "dims": [22, 16, 54]},
        {"part": 4, "origin": [4.56, 0.82, 0.00], "h": 0.01, "dims": [40, 14, 54]},
        {"part": 5, "origin": [0.00, 0.06, 0.00], "h": 0.01, "dims": [64, 30, 96]},
        {"part": 6, "origin": [4.55, 0.52, 0.40], "h": 0.01, "dims": [64, 52, 22]},
    ]
    off = 0
    for g in grids:
        g["offset"] = off
        off += g["dims"][0] * g["dims"][1] * g["dims"][2]
    front_a = [[0.24, 0.205 + 0.0004 * i] for i in range(FRONT_BINS)]
    front_b = [[0.37, 0.262 + 0.0004 * i] for i in range(FRONT_BINS)]
    return {"frontHinges": [front_a, front_b], "rearMainHinge": [4.60, 0.88], "rearFlapHinge": [4.72, 1.00],
            "partGrids": grids}


def synthetic_w17(p=None, fly_progress=(0.0, 0.0)):
    """A stand-in W17 model in the reference's formats: a tub, nose, sidepods
    (around the cooling ducts), engine cover and floor in the body texture; thin
    slabs for the six wing parts."""
    from .engine import ShapeKind, ShapeParams
    if p is None:
        p = ShapeParams(kind=ShapeKind.W17)
    x, y, z = _grid(SDF_ORIGIN, SDF_H, SDF_DIMS)
    body = _round_box(x, y, z, (2.55, 0.45, 0.0), (1.75, 0.28, 0.30), 0.10)
    body = np.minimum(body, _capsule(x, y, z, (0.05, 0.30, 0.0), (1.6, 0.42, 0.0), 0.11))
    body = np.minimum(body, _round_box(x, y, z, (3.05, 0.46, 0.42), (0.95, 0.17, 0.22), 0.08))
    body = np.minimum(body, _capsule(x, y, z, (2.55, 0.86, 0.0), (4.75, 0.58, 0.0), 0.13))
    body = np.minimum(body, _round_box(x, y, z, (2.90, 0.115, 0.30), (1.65, 0.025, 0.55), 0.01))
    rig = synthetic_rig_data()
    slabs = {1: [((0.40, 0.225, 0.35), (0.15, 0.012, 0.24))],
             2: [((0.50, 0.285, 0.35), (0.12, 0.010, 0.24))],
             3: [((4.80, 1.020, 0.26), (0.08, 0.010, 0.24))],
             4: [((4.75, 0.880, 0.26), (0.17, 0.014, 0.24))],
             5: [((0.30, 0.120, 0.45), (0.28, 0.012, 0.44)), ((0.30, 0.260, 0.92), (0.28, 0.150, 0.010))],
             6: [((4.85, 0.760, 0.52), (0.28, 0.240, 0.010))]}
    data = []
    for g in rig["partGrids"]:
        gx, gy, gz = _grid(g["origin"], g["h"], g["dims"])
        d = np.full(gx.shape, 1e3)
        for c, b in slabs[g["part"]]:
            d = np.minimum(d, _round_box(gx, gy, gz, c, b, 0.005))
        data.append(_to_half_bits(d).ravel())
    atlas, dims = parts_atlas(rig, np.concatenate(data))
    return CarModel(_to_half_bits(body), atlas, dims, w17_rig(rig, p, fly_progress), rig)
