#!/usr/bin/env python3
"""Generate the W17 voxel fixture (w17.npz) from the reference itself.

The reference's VOXELIZE shader with its W17 path (src/engine/wgsl.ts:305-321,
src/engine/f1.ts:322-394, the rig of src/engine/car-model.ts:59-136),
translated to C++ (oracle/wgsl_translate.py, oracle/Makefile `ref`), voxelizes
the synthetic stand-in model of windtunnel.car_model.synthetic_w17 (the
reference's own W17 assets stay in its checkout) with two rig settings:
  A  default wings, closed cooling (no ducts)
  B  high-downforce front, low-downforce rear, front flap +5 deg, Monza spoon
     twist, thin flaps, compact sidepods, cooling open (ducts carved, emit -1)
on a 144x40x32 half tunnel at 4.5 cm from (-1, 0, 0).  Stored: solid flags and
emission per setting.  The synthetic model is regenerated bit for bit on any
machine (numpy float64, correctly rounded operations only), so the GPU test
rebuilds it instead of reading a stored copy.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))

from windtunnel.engine import ShapeKind, ShapeParams  # noqa: E402

OUT = os.path.join(HERE, "w17.npz")
DIMS, ORIGIN, H = (144, 40, 32), (-1.0, 0.0, 0.0), 0.045


def settings():
    return {
        "A": ShapeParams(kind=ShapeKind.W17, rideH=0.12, rearRideH=0.14, cooling=0),
        "B": ShapeParams(kind=ShapeKind.W17, rideH=0.10, rearRideH=0.15, frontWing=1, rearWing=2, frontFlapDeg=5.0,
                         rearShape=1, thinWings=True, sidepods=1, cooling=2),
    }


def main():
    from oracle import pyoracle
    from windtunnel.car_model import synthetic_w17
    from windtunnel.engine import pack_shape
    out = {}
    for name, p in settings().items():
        pyoracle.ref_set_car(synthetic_w17(p))
        r = pyoracle.Reference(DIMS, ORIGIN, H)
        r.voxelize(pack_shape(p))
        d = r.read()
        out[f"solid_{name}"] = d["solid"].astype(np.uint8)
        out[f"emit_{name}"] = d["emit"].astype(np.float32)
        print(name, "solid", int((d["solid"] > 0).sum()), "per group", np.bincount(d["solid"], minlength=4).tolist(),
              "duct cells", int((d["emit"] < 0).sum()), "hot cells", int((d["emit"] > 0).sum()))
    pyoracle.ref_set_car(None)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
