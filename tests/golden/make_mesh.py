#!/usr/bin/env python3
"""Generate the car mesh fixture (mesh.npz) from the reference itself.

The reference's MESH_DRAW shaders (src/engine/render-wgsl.ts:647-760, vs_main
and fs_main), translated to C++ by oracle/wgsl_translate.py, run in the
oracle's restatement of the WebGPU pipeline (oracle/ref_driver.cpp
wtr_mesh_gbuffer: clipping, rasterization, depth test and bias, decal
blending, the texture filter) over the stand-in car mesh
(windtunnel.mesh_car.synthetic_mesh(0.5), stored here with its textures), with
the rig of the stand-in W17 model.  Then the reference's RENDER shader
composites two of the G-buffers (meshMode) over the consumer fixture's flow.

Cases (128x72 unless noted), each the G-buffer albedo, normal-distance and
material targets:
  hero     the default W17 setup, three-quarter view, Halton jitter of frame 1
  rig      flaps opened, rear tips twisted, thin flaps, squeezed sidepods,
           gurney tab on; seen from the other side, higher
  fly      the front wing half way through its fly-away, the rear wing gone
  close    camera inside the front wing's span: triangles cross the near plane
  under    low camera under the floor (two large triangles), 97x61
Composites: hero and rig (scene target, binary16), cooling 1 and 2.

Needs the reference checkout (build container only).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))
sys.path.insert(0, HERE)

import make_consumers as mc  # noqa: E402
from windtunnel import render as R  # noqa: E402
from windtunnel.car_model import synthetic_w17  # noqa: E402
from windtunnel.engine import ShapeKind, ShapeParams, pack_shape  # noqa: E402
from windtunnel.mesh_car import mesh_cam, synthetic_mesh  # noqa: E402

OUT = os.path.join(HERE, "mesh.npz")
DETAIL = 0.5
W, H = 128, 72


def cases():
    """[(name, ShapeParams, fly progress, camera, size, frame number)]"""
    base = ShapeParams(kind=ShapeKind.W17, rideH=0.11, rearRideH=0.14)
    rig = ShapeParams(kind=ShapeKind.W17, rideH=0.10, rearRideH=0.16, frontFlapDeg=8.0, rearFlapDeg=-10.0,
                      rearShape=1, thinWings=True, sidepods=1, gurney=True)
    asp = W / H
    return [
        ("hero", base, (0.0, 0.0), R.orbit_camera((2.6, 0.45, 0.0), 2.4, 0.3, 6.2, asp), (W, H), 1),
        ("rig", rig, (0.0, 0.0), R.orbit_camera((3.2, 0.5, 0.0), -2.2, 0.55, 5.6, asp), (W, H), 2),
        ("fly", base, (0.45, 1.0), R.orbit_camera((2.2, 0.8, 0.0), 2.0, 0.25, 7.5, asp), (W, H), 3),
        ("close", base, (0.0, 0.0), R.orbit_camera((0.3, 0.16, 0.3), 2.9, 0.2, 0.35, asp), (W, H), 4),
        ("under", base, (0.0, 0.0), R.orbit_camera((2.8, 0.2, 0.0), 1.4, -0.02, 3.5, 97 / 61), (97, 61), 5),
    ]


def frame_halton(k):
    k = (k % 8) + 1
    return R.halton(k, 2) - 0.5, R.halton(k, 3) - 0.5


def main():
    from oracle import pyoracle as po
    if po.ref_lib() is None:
        raise SystemExit("translated reference not built")
    mesh = synthetic_mesh(DETAIL)
    out = {"verts": mesh.verts, "indices": mesh.indices, "tags": mesh.tags}
    for t, (w, h, rgba) in enumerate(mesh.textures):
        out[f"tex{t}"] = rgba
    c = {k: v for k, v in np.load(os.path.join(HERE, "consumers.npz")).items()}
    for name, p, fly, cam, size, k in cases():
        car = synthetic_w17(p, fly)
        mcam = mesh_cam(cam, size, frame_halton(k), p)
        a, n, m, d = po.ref_mesh_gbuffer(mesh, mcam, car.rig, size[0], size[1], gurney=p.gurney)
        out[f"{name}_rig"] = car.rig
        out[f"{name}_albedo"], out[f"{name}_normal"], out[f"{name}_material"] = a, n, m
        print(name, "car texels", int((n[..., 3].astype(np.float32) > 0).sum()))
        if name in ("hero", "rig"):
            st = R.FrameState()
            st.frame_no = k - 1
            u = st.next(cam, size)
            po.ref_set_car(car)
            po.ref_set_gbuffer(a, n, m)
            for cooling in (1, 2):
                look = R.make_look(p, palette=1, cooling=cooling)
                look.mesh_mode = 1
                sc = po.ref_render_scene(mc.DIMS, mc.ORIGIN, mc.H, c["fields"], c["temps"], pack_shape(p), u.cam,
                                         look, mc.view(), size[0], size[1])
                out[f"{name}_scene_c{cooling}"] = sc.astype(np.float16)
            po.ref_set_car(None)
            po.ref_set_gbuffer(None, None, None)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
