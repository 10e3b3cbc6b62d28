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
Plus `edge`: a small mesh of the pipeline's corner cases (edge_mesh), 80x48.

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


def edge_mesh():
    """A small mesh of the pipeline's corner cases, in MeshCar's formats: a wall of
    two triangles larger than the view (the tiled path), two coplanar quads in
    different draws (z-fighting: per pixel the smaller rounded depth wins, an
    exact tie goes to the first drawn), two decal layers in the same plane
    (blended in draw order, one textured with an alpha ramp), a zero-area triangle,
    one wholly behind the camera and one crossing the near plane, a draw whose
    count is not a multiple of 3 and an empty draw."""
    from windtunnel.mesh_car import DrawSpec, MeshData
    v = []

    def quad(p0, p1, p2, p3, n=(0.0, 0.0, -1.0)):
        base = len(v)
        for (x, y, z), (u, w) in zip((p0, p1, p2, p3), ((0, 0), (1, 0), (1, 1), (0, 1))):
            v.append([x, y, z, u, n[0], n[1], n[2], w])
        return [base, base + 1, base + 2, base + 0, base + 2, base + 3]
    wall = quad((-30.0, -20.0, 6.0), (30.0, -20.0, 6.0), (30.0, 20.0, 6.0), (-30.0, 20.0, 6.0))
    q_a = quad((-1.0, -0.5, 2.0), (0.5, -0.5, 2.0), (0.5, 0.8, 2.0), (-1.0, 0.8, 2.0))
    q_b = quad((-0.5, -0.8, 2.0), (1.0, -0.8, 2.0), (1.0, 0.5, 2.0), (-0.5, 0.5, 2.0))
    d_a = quad((-0.8, -0.3, 2.0), (0.3, -0.3, 2.0), (0.3, 0.6, 2.0), (-0.8, 0.6, 2.0))
    d_b = quad((-0.3, -0.6, 2.0), (0.8, -0.6, 2.0), (0.8, 0.3, 2.0), (-0.3, 0.3, 2.0))
    cutout = quad((0.3, 0.12, 1.2), (0.8, 0.12, 1.2), (0.8, 0.42, 1.2), (0.3, 0.42, 1.2))
    b = len(v)
    v += [[0.2, 0.2, 1.0, 0, 0, 0, -1, 0], [0.4, 0.4, 1.0, 1, 0, 0, -1, 0], [0.6, 0.6, 1.0, 0, 0, 0, -1, 1]]
    degenerate = [b, b + 1, b + 2]
    b = len(v)
    v += [[0.0, 0.0, -2.0, 0, 0, 0, -1, 0], [1.0, 0.0, -2.0, 1, 0, 0, -1, 0], [0.0, 1.0, -2.0, 0, 0, 0, -1, 1]]
    behind = [b, b + 1, b + 2]
    b = len(v)
    v += [[-0.6, -0.6, -0.5, 0, 0, 0, -1, 0], [0.6, -0.4, 3.0, 1, 0, 0, -1, 0], [0.1, 0.7, 3.0, 0, 0, 0, -1, 1]]
    crossing = [b, b + 1, b + 2]
    groups = [("wall", wall), ("quad_a", q_a), ("quad_b", q_b + degenerate + behind), ("crossing", crossing + [0]),
              ("cutout", cutout), ("decal_a", d_a), ("decal_b", d_b)]
    idx, ranges = [], {}
    for name, ii in groups:
        ranges[name] = (len(idx), len(ii))
        idx += ii
    verts = np.array(v, np.float32)
    tex = np.zeros((8, 8, 4), np.uint8)
    tex[..., 0] = 200
    tex[..., 3] = np.arange(8, dtype=np.uint8)[None, :] * 36
    m = dict(metal=0.2, rough=0.4, coat=0.2, emissive=0.0, is_body=0.0)
    draws = [
        DrawSpec("wall", (0.3, 0.3, 0.3, 1.0), alpha_cut=0.0, first=ranges["wall"][0], count=6, **m),
        DrawSpec("quad_a", (0.9, 0.1, 0.1, 1.0), alpha_cut=0.0, first=ranges["quad_a"][0], count=6, **m),
        DrawSpec("empty", (1.0, 1.0, 1.0, 1.0), alpha_cut=0.0, first=0, count=0, **m),
        DrawSpec("quad_b", (0.1, 0.9, 0.1, 1.0), alpha_cut=0.0, first=ranges["quad_b"][0], count=12, **m),
        DrawSpec("crossing", (0.1, 0.1, 0.9, 1.0), alpha_cut=0.0, first=ranges["crossing"][0], count=4, **m),
        # an opaque draw with an alpha cut (MeshCar never makes one; the pipeline allows it): the
        # texture's alpha ramp cuts it, and the cut fragments neither write nor hide the wall
        DrawSpec("cutout", (0.9, 0.8, 0.2, 1.0), alpha_cut=0.5, first=ranges["cutout"][0], count=6, texture=0, **m),
        DrawSpec("decal_a", (1.0, 1.0, 1.0, 0.7), alpha_cut=0.02, first=ranges["decal_a"][0], count=6, texture=0,
                 blend=True, **m),
        DrawSpec("decal_b", (0.2, 0.4, 1.0, 0.6), alpha_cut=0.02, first=ranges["decal_b"][0], count=6, blend=True, **m),
    ]
    return MeshData(verts, np.array(idx, np.uint32), np.zeros(len(v), np.uint8), draws, [(8, 8, tex)])


def edge_camera():
    """Looking down +z from the origin (so the wall and quads face it)."""
    return R.orbit_camera((0.0, 0.0, 1.0), -np.pi / 2, 0.0, 1.0, 80 / 48)


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
    # the corner-case mesh, 80x48, no rig motion (tags 0, not a body draw)
    em = edge_mesh()
    ecam = mesh_cam(edge_camera(), (80, 48), (0.0, 0.0), cases()[0][1])
    a, n, m, d = po.ref_mesh_gbuffer(em, ecam, synthetic_w17(cases()[0][1]).rig, 80, 48)
    out.update(edge_verts=em.verts, edge_indices=em.indices, edge_tex=em.textures[0][2],
               edge_albedo=a, edge_normal=n, edge_material=m)
    print("edge car texels", int((n[..., 3].astype(np.float32) > 0).sum()))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
