#!/usr/bin/env python3
"""Generate the field-consumer fixture (consumers.npz) from the reference itself.

The reference's own FIELD_SAMPLING, PARTICLES_SIM and STREAM_SIM shaders
(src/engine/wgsl.ts:324-366, 516-594; src/engine/render-wgsl.ts:520-576),
translated to C++ by oracle/wgsl_translate.py and built by oracle/Makefile
`ref`, run over the fields and temperatures of a short reference run of the
generic F1 on a 64x24x20 lattice:

  sample points   300 world points (both sides of the symmetry plane):
                  sampleFlow (u, rho, temp, fluid) and vorticityAt
  particles       600 particles through five passes (scatter spawn, rake
                  spawn, and the five colour modes), the state after each pass
  streamlines     a 4 x 3 rake and two ring emitters, 150 steps per line

Needs the reference checkout (build container only); the fixture travels with
the repository so the GPU kernels are pinned anywhere.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))

from oracle import pyoracle  # noqa: E402
from windtunnel import _abi  # noqa: E402
from windtunnel.engine import ORIGIN_X, make_sim  # noqa: E402
from windtunnel.workloads import config_f1_shape  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "consumers.npz")
DIMS, H = (64, 24, 20), 0.18
ORIGIN = (ORIGIN_X, 0.0, 0.0)


def view():
    v = _abi.View()
    v.u_in, v.v_real, v.cp_min, v.cp_max = 0.08, 69.4, -1.5, 1.0
    v.t_min, v.t_max, v.speed_max, v.vort_max = 0.0, 1.0, 1.5, 0.5
    return v


def passes():
    """(spawn_mode, colour_mode, scatter, frame) of the five particle passes."""
    return [(0, 0, 1, 0), (1, 1, 0, 1), (1, 3, 0, 2), (0, 2, 0, 3), (1, 4, 0, 4)]


def psim(count, spawn_mode, color_mode, scatter, frame):
    p = _abi.PSim()
    p.count, p.spawn_mode, p.color_mode, p.frame = count, spawn_mode, color_mode, frame
    p.dt, p.life, p.scatter, p.rake_rows, p.rake_cols = 8.0, 3.0, scatter, 6, 5
    p.spawn_min[:] = [-2.2, 0.05, 0.0]
    p.spawn_max[:] = [-1.0, 1.6, 1.5]
    return p


def stream_params():
    a = _abi.StreamParams()
    a.lines, a.steps, a.seed_mode, a.color_mode, a.rows, a.cols = 12, 150, 0, 0, 4, 3
    a.seed_min[:] = [-2.2, 0.1, 0.05]
    a.seed_max[:] = [-2.2, 1.5, 1.4]
    a.step_len, a.time = 0.09, 0.0
    b = _abi.StreamParams()
    b.lines, b.steps, b.seed_mode, b.color_mode, b.per_emitter, b.emitters = 10, 150, 1, 1, 5, 2
    b.step_len, b.time = 0.09, 0.7
    for e, c in enumerate([(-2.0, 0.5, 0.3, 0.2), (-2.0, 1.0, 0.6, 0.15)]):
        for k in range(4):
            b.emitter[e][k] = c[k]
    return [a, b]


def main():
    sim = make_sim(u_in=0.08, tau0=0.51, smag=0.1, sponge_cells=16.0)
    r = pyoracle.Reference(DIMS, ORIGIN, H, sim)
    r.reset()
    r.voxelize(config_f1_shape(3))
    for _ in range(40):
        r.frame(8)
    d = r.read()
    fields, temps = d["fields"], d["temps"]
    rng = np.random.default_rng(11)
    hi = np.array([ORIGIN[0] + DIMS[0] * H, DIMS[1] * H, DIMS[2] * H])
    pts = np.stack([rng.uniform(ORIGIN[0], hi[0], 300), rng.uniform(0.0, hi[1], 300),
                    rng.uniform(-hi[2], hi[2], 300)], axis=1).astype(np.float32)
    samp, vort = pyoracle.ref_sample_flow(DIMS, ORIGIN, H, fields, temps, pts)
    parts = np.zeros((600, 8), np.float32)
    states = []
    for sm, cm, sc, fr in passes():
        pyoracle.ref_particles(DIMS, ORIGIN, H, fields, temps, psim(600, sm, cm, sc, fr), view(), parts)
        states.append(parts.copy())
    lines = [pyoracle.ref_streamlines(DIMS, ORIGIN, H, fields, temps, p, view()) for p in stream_params()]
    np.savez_compressed(OUT, fields=fields, temps=temps, points=pts, sample=samp, vorticity=vort,
                        particles=np.stack(states), lines_rake=lines[0], lines_ring=lines[1])
    print("wrote", OUT, os.path.getsize(OUT), "bytes;", int((states[-1][:, 7] >= 0).sum()), "particles coloured,",
          int((lines[0][..., 3] >= 0).sum()), "+", int((lines[1][..., 3] >= 0).sum()), "live streamline points")


if __name__ == "__main__":
    main()
