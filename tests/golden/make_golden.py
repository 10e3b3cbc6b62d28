#!/usr/bin/env python3
"""Generate the golden fixtures of this directory from the reference itself.

Runs the reference's own WGSL simulation shaders (translated to C++ and built
by oracle/Makefile `ref` from the reference checkout, see oracle/wgsl_translate.py)
through the engine's dispatch order, and writes small fixtures:

  vox_<case>.npz   solid flags (u8) and emission (f32) of VOXELIZE for several scenes
  lbm_<case>.npz   per-frame SHA-256 of fields / populations / temperatures, the i32
                   force accumulator read each frame, and strided samples of the fields
  manifest.json    the cases, their inputs, and the SHA-256 of the translated shader text

Needs the reference checkout (only present in the build container); the fixtures
travel with the repository so tests can pin the oracle and the GPU path anywhere.
"""
import hashlib
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))

from oracle import pyoracle  # noqa: E402
from windtunnel import _abi  # noqa: E402
from windtunnel.engine import ShapeParams, make_sim, pack_shape  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
DEG = math.pi / 180


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def shapes():
    """Scenes exercised: the headless-check car (scripts/headless-check.ts:21-24) and variants."""
    base = ShapeParams()  # kind F1, rideH 0.10, rearRideH 0.12, heat on
    out = {
        "f1_default": pack_shape(base),
        "f1_v1": pack_shape(ShapeParams(frontWing=1, rearWing=1, sidepod=2, cover=1, nose=1, frontFlapDeg=7,
                                        rearFlapDeg=-9, rideH=0.08, rearRideH=0.11, cooling=0)),
        "f1_v2": pack_shape(ShapeParams(frontWing=2, rearWing=2, sidepod=3, cover=2, nose=2, rideH=0.05,
                                        rearRideH=0.09, cooling=2)),
        "f1_v3": pack_shape(ShapeParams(frontWing=3, sidepod=1, rideH=0.03, rearRideH=0.06, heatRad=False)),
        "cube": pack_shape(ShapeParams(kind=2)),
        "sphere": pack_shape(ShapeParams(kind=1)),
        "wing": pack_shape(ShapeParams(kind=3, aoaDeg=9)),
        "empty": pack_shape(ShapeParams(kind=6)),
    }
    return out


VOX_GRID = dict(dims=(96, 36, 30), origin=(-2.4, 0.0, 0.0), h=0.09)
LBM_GRID = dict(dims=(64, 24, 20), origin=(-2.4, 0.0, 0.0), h=0.135)


def shape_dict(s):
    return {name: (list(getattr(s, name)) if hasattr(getattr(s, name), "__len__") else getattr(s, name))
            for name, _ in s._fields_}


def main():
    if pyoracle.ref_lib() is None:
        raise SystemExit("oracle/_ref not built: run `make -C oracle ref` with the reference checkout present")
    man = {"translated_shaders_sha256": {}, "vox": {}, "lbm": {}}
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    for f in sorted(os.listdir(ref_dir)):
        if f.endswith(".wgsl"):
            man["translated_shaders_sha256"][f] = hashlib.sha256(open(os.path.join(ref_dir, f), "rb").read()).hexdigest()

    sims = {"ref": make_sim()}
    # ---- voxelization
    g = VOX_GRID
    for name, s in shapes().items():
        r = pyoracle.Reference(g["dims"], g["origin"], g["h"], sims["ref"])
        r.voxelize(s)
        d = r.read()
        np.savez_compressed(os.path.join(OUT, f"vox_{name}.npz"), solid=d["solid"].astype(np.uint8), emit=d["emit"])
        man["vox"][name] = {"grid": g, "shape": shape_dict(s), "solid_sha256": sha(d["solid"]),
                            "emit_sha256": sha(d["emit"]), "solid_cells": int((d["solid"] > 0).sum())}
        print("vox", name, int((d["solid"] > 0).sum()))

    # ---- lattice runs
    g = LBM_GRID
    cases = {
        # reference defaults (engine.ts:249), headless-check car, two frames, re-voxelize, one frame
        "f1_revox": dict(sim=make_sim(), frames=[("shape", "f1_default"), 8, 8, ("shape", "f1_v2"), 8]),
        # benchmark collision parameters with the reference's 18-cell sponge
        "f1_cfg": dict(sim=make_sim(u_in=0.08, tau0=0.51, smag=0.1), frames=[("shape", "f1_v1"), 8, 8, 8]),
        # divergence guard: corrupted cells after a frame
        "f1_guard": dict(sim=make_sim(), frames=[("shape", "f1_default"), 4, ("corrupt", 0), 4]),
    }
    sh = shapes()
    for cname, c in cases.items():
        r = pyoracle.Reference(g["dims"], g["origin"], g["h"], c["sim"])
        r.reset()
        rec = {"frames": [], "sim": [c["sim"].u_in, c["sim"].tau0, c["sim"].smag], "script": []}
        arrays = {}
        k = 0
        for item in c["frames"]:
            if isinstance(item, tuple) and item[0] == "shape":
                r.voxelize(sh[item[1]])
                rec["script"].append(["shape", item[1]])
                continue
            if isinstance(item, tuple) and item[0] == "corrupt":
                d = r.read()
                f = d["f"].copy()
                n = r.n
                rng = np.random.default_rng(item[1])
                cells = rng.choice(np.nonzero(d["solid"] == 0)[0], 12, replace=False)
                f[3 * n + cells[:4]] = np.nan
                f[1 * n + cells[4:8]] = 50.0
                f[7 * n + cells[8:]] = -40.0
                r.write_state(f=f)
                rec["script"].append(["corrupt", item[1], cells.tolist()])
                continue
            r.frame(item)
            d = r.read(reset_forces=True)
            rec["script"].append(["frame", item])
            rec["frames"].append({
                "fields_sha256": sha(d["fields"]), "f_sha256": sha(d["f"]), "temps_sha256": sha(d["temps"]),
                "forces": d["forces"].tolist(),
                "fields_sum": float(d["fields"].astype(np.float64).sum()),
                "temps_sum": float(d["temps"].astype(np.float64).sum()),
            })
            arrays[f"fields_sample_{k}"] = d["fields"][::37]
            k += 1
        rec["grid"] = g
        np.savez_compressed(os.path.join(OUT, f"lbm_{cname}.npz"), **arrays)
        man["lbm"][cname] = rec
        print("lbm", cname, [fr["forces"][:9] for fr in rec["frames"]])
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump(man, f, indent=1)


if __name__ == "__main__":
    main()
