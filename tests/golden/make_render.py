#!/usr/bin/env python3
"""Generate the render fixture (render.npz) from the reference itself.

The reference's own render shaders (src/engine/render-wgsl.ts RENDER, TAA,
BLUR, PRESENT, STREAM_DRAW and src/engine/wgsl.ts PARTICLES_DRAW), translated
to C++ by oracle/wgsl_translate.py and built by oracle/Makefile `ref`, run in
the engine's pass order (engine.ts:714-725) over the flow of the consumer
fixture (consumers.npz: the generic F1 on a 64x24x20 lattice, its particles
after five passes and its streamlines).  The fixed-function stages (viewport,
rasterization, blending) are the oracle's restatement of the WebGPU pipeline
(oracle/ref_driver.cpp).

Eleven sequences of frames (128x72 unless noted) cover the scene pass's branches:
  hero      livery, ground reflection and belt, streamline glow; then a second
            frame from a slightly moved camera, which reprojects the history
  surface   pressure colour on the body surface (surfMode 1, palette 1)
  slice-z   z slice with temperature colours, particle glow (palette 2)
  slice-x   x slice with vorticity colours, vortex streamlines (palette 3)
  slice-y   y slice with the wake map (palette 4), a carbon-free paint livery
  cube, sphere, wing, empty
            the other analytic scenes: carbon and paint bodies, vorticity colour
            on a sphere's surface, a pressure slice past the wing, the bare tunnel
  w17       the baked W17 scene with the synthetic stand-in model (rig-rotated
            wing parts, squeezed sidepods), pressure colour on its surface
  tiny      a ragged 17x9 target (8x4 bloom) with particle and streamline glow,
            two frames
Stored per frame: the scene, resolved history, glow and bloom B targets
(binary16) and the presented RGBA8 output.

Needs the reference checkout (build container only); the fixture travels with
the repository so the GPU kernels are pinned anywhere.
"""
import math
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
from windtunnel.engine import ShapeKind, ShapeParams  # noqa: E402
from windtunnel.car_model import synthetic_w17  # noqa: E402
from windtunnel.workloads import config_f1_shape  # noqa: E402

OUT = os.path.join(HERE, "render.npz")
W, H = 128, 72
SHAPE_SEED = 3  # the consumer fixture's car


def sequences(z):
    """[(name, [frame dict, ...]), ...]; each frame: camera, look, glow inputs."""
    shape = config_f1_shape(SHAPE_SEED)
    p = ShapeParams(kind=ShapeKind.F1, rideH=shape.ride_h)  # the fields make_look reads
    parts = z["particles"][-1]
    asp = W / H
    hero = dict(cam=R.orbit_camera((2.75, 0.42, 0.0), 2.3, 0.3, 7.6, asp), look=R.make_look(p, palette=0),
                lines=z["lines_rake"], color_mode=0, flow_time=0.7)
    hero2 = dict(hero, cam=R.orbit_camera((2.75, 0.42, 0.0), 2.33, 0.29, 7.5, asp))
    surface = dict(cam=R.orbit_camera((2.4, 0.5, 0.0), math.pi + 0.001, 0.12, 5.0, asp),
                   look=R.make_look(p, palette=1, surface_field=True))
    slice_z = dict(cam=R.orbit_camera((2.0, 0.6, 0.0), 1.9, 0.35, 7.0, asp),
                   look=R.make_look(p, palette=2, slice_axis=3, slice_pos=0.35), parts=parts, color_mode=2, smoke=True)
    slice_x = dict(cam=R.orbit_camera((3.0, 0.5, 0.3), 2.7, 0.2, 6.0, asp),
                   look=R.make_look(p, palette=3, slice_axis=1, slice_pos=3.2), lines=z["lines_ring"], color_mode=3,
                   flow_time=1.3, vortices=True)
    slice_y = dict(cam=R.orbit_camera((2.5, 0.4, 0.0), 0.6, 0.5, 6.5, asp),
                   look=R.make_look(p, palette=4, slice_axis=2, slice_pos=0.3, paint=(0.7, 0.1, 0.1), carbon=False),
                   parts=parts, color_mode=4, smoke=False)
    seqs = [("hero", [hero, hero2]), ("surface", [surface]), ("slice-z", [slice_z]), ("slice-x", [slice_x]),
            ("slice-y", [slice_y])]
    # the other analytic scenes (engine.ts:474-486 bounds), over the same flow
    cube = ShapeParams(kind=ShapeKind.Cube)
    sphere = ShapeParams(kind=ShapeKind.Sphere)
    wing = ShapeParams(kind=ShapeKind.Wing, aoaDeg=8.0)
    empty = ShapeParams(kind=ShapeKind.Empty)
    seqs += [
        ("cube", [dict(cam=R.orbit_camera((2.6, 1.0, 0.0), 2.2, 0.35, 4.5, asp), look=R.make_look(cube, palette=0),
                       parts=parts, color_mode=0, smoke=True, shape=cube)]),
        ("sphere", [dict(cam=R.orbit_camera((2.6, 1.0, 0.0), 2.6, 0.25, 3.8, asp),
                         look=R.make_look(sphere, palette=3, surface_field=True, carbon=False, paint=(0.2, 0.5, 0.9)),
                         shape=sphere)]),
        ("wing", [dict(cam=R.orbit_camera((2.4, 1.2, 0.0), 1.7, 0.3, 6.0, asp),
                       look=R.make_look(wing, palette=1, slice_axis=3, slice_pos=0.2, carbon=False),
                       lines=z["lines_rake"], color_mode=1, flow_time=0.2, shape=wing)]),
        ("empty", [dict(cam=R.orbit_camera((2.0, 0.5, 0.0), 2.0, 0.4, 7.0, asp),
                        look=R.make_look(empty, palette=0, slice_axis=2, slice_pos=0.5), shape=empty)]),
    ]
    # the baked W17 scene (kind 5) with the synthetic stand-in model, open cooling
    w17 = ShapeParams(kind=ShapeKind.W17, rideH=0.10, rearRideH=0.15, frontFlapDeg=5.0, rearShape=1, sidepods=1,
                      cooling=2)
    seqs.append(("w17", [dict(cam=R.orbit_camera((2.6, 0.45, 0.0), 2.4, 0.3, 6.2, asp),
                              look=R.make_look(w17, palette=1, surface_field=True), shape=w17,
                              car=synthetic_w17(w17))]))
    # a ragged target: 17x9 (bloom targets 8x4), particle and streamline glow, two frames
    tiny = dict(cam=R.orbit_camera((2.75, 0.42, 0.0), 2.3, 0.3, 7.6, 17 / 9), look=R.make_look(p, palette=0),
                parts=parts, lines=z["lines_rake"], color_mode=0, flow_time=0.3, size=(17, 9))
    seqs.append(("tiny", [tiny, dict(tiny, cam=R.orbit_camera((2.75, 0.42, 0.0), 2.35, 0.31, 7.4, 17 / 9))]))
    return shape, seqs


def frame_shape(default, f):
    """The wt_shape a frame renders: its own analytic scene, or the fixture's F1."""
    from windtunnel.engine import pack_shape
    return pack_shape(f["shape"]) if "shape" in f else default


def frame_size(f):
    return f.get("size", (W, H))


def frame_uniforms(state, f):
    return state.next(f["cam"], frame_size(f), parts=f.get("parts"), color_mode=f.get("color_mode", 0),
                      smoke=f.get("smoke", True), lines=f.get("lines"), flow_time=f.get("flow_time", 0.0),
                      vortices=f.get("vortices", False))


def main():
    from oracle import pyoracle
    z = np.load(os.path.join(HERE, "consumers.npz"))
    shape, seqs = sequences(z)
    view = mc.view()
    out = {}
    for name, frames in seqs:
        st = R.FrameState()
        w, h = frame_size(frames[0])
        hw, hh = max(1, w // 2), max(1, h // 2)
        hist = [np.zeros((h, w, 4), np.float32), np.zeros((h, w, 4), np.float32)]
        for k, f in enumerate(frames):
            u = frame_uniforms(st, f)
            pyoracle.ref_set_car(f.get("car"))
            scene = pyoracle.ref_render_scene(mc.DIMS, mc.ORIGIN, mc.H, z["fields"], z["temps"], frame_shape(shape, f),
                                              u.cam, f["look"], view, w, h)
            hist[u.cur] = pyoracle.ref_taa(scene, hist[1 - u.cur], u.taa)
            glow = pyoracle.ref_glow(scene, f.get("parts"), u.pdraw, f.get("lines"), u.sdraw)
            ba = pyoracle.ref_blur(glow, (1.0, 0.0), 3.0, 1.0, hw, hh)
            bb = pyoracle.ref_blur(ba, (0.0, 1.0), 1.5, 1.0, hw, hh)
            rgba = pyoracle.ref_present(hist[u.cur], glow, bb, u.post)
            key = f"{name}_{k}"
            out[key + "_scene"] = scene.astype(np.float16)
            out[key + "_hist"] = hist[u.cur].astype(np.float16)
            out[key + "_glow"] = glow.astype(np.float16)
            out[key + "_bloom"] = bb.astype(np.float16)
            out[key + "_out"] = rgba
            print(key, "hit pixels", int((scene[..., 3] < 6e4).sum()), "glow pixels", int((glow[..., 3] > 0).sum()),
                  "mean rgb", rgba[..., :3].mean().round(2))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
