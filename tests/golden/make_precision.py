"""Generate the FP64 oracle fixtures of the precision case (generic F1, seed 5,
128x48x40 cells at 9 cm, u_in 0.08, Cs 0.1, sponge 16):

  precision_fp64_128x48x40.json         tau0 0.51 (the benchmark's value), 20000
      steps, an ensemble of members that differ only by a 1e-5 perturbation of
      the initial populations (member 0 unperturbed).  The unsteady wake turns
      any difference of arithmetic into a different trajectory after a few
      hundred steps and the case has several long-lived states; the spread of
      the members' window means is the noise against which the stored formats'
      statistics are judged.
  precision_fp64_steady_128x48x40.json  tau0 0.6, 8000 steps, one run: the same
      car in steady flow, where window means are deterministic and a 1 %
      bound on Cd and Cl is decidable.

Both hold per-200-step block force means (tests/test_gpu_precision_study.py).

    python tests/golden/make_precision.py [--members 4] [--steady]

Test infrastructure: runs the oracle (oracle/pyoracle.py), minutes per member."""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "f1-wind-tunnel_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

DIMS, H, SEED = (128, 48, 40), 0.09, 5
STEPS, BLOCK = 20000, 200
PERTURB = 1e-5
OUT = os.path.join(HERE, "precision_fp64_128x48x40.json")
STEADY_TAU0, STEADY_STEPS = 0.6, 8000
OUT_STEADY = os.path.join(HERE, "precision_fp64_steady_128x48x40.json")


def case(tau0=None):
    from windtunnel import f1_config
    from windtunnel.engine import make_sim
    dims, origin, h, sim, shape = f1_config(dims=DIMS, h=H, seed=SEED)
    if tau0 is not None:
        sim = make_sim(u_in=sim.u_in, tau0=tau0, smag=sim.smag, sponge_cells=sim.sponge_cells)
    return dims, origin, h, sim, shape


def perturbation(member, n):
    """Additive noise on the 19 n initial populations (reference order f[i n + idx])."""
    if member == 0:
        return np.zeros(19 * n, np.float32)
    rng = np.random.default_rng(1000 + member)
    return (PERTURB * rng.standard_normal(19 * n)).astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--steady", action="store_true")
    args = ap.parse_args()
    from oracle import pyoracle
    from windtunnel import half_area_cells
    if args.steady:
        dims, origin, h, sim, shape = case(STEADY_TAU0)
        o = pyoracle.Oracle(dims, origin, h, sim, fp64=True)
        o.voxelize(shape)
        o.reset()
        d = o.read(reset_forces=True)
        blocks = []
        for k in range(STEADY_STEPS // BLOCK):
            o.steps(BLOCK)
            blocks.append((o.read(reset_forces=True)["forces64"] / BLOCK).tolist())
        rec = {"dims": list(dims), "h": H, "seed": SEED, "tau0": STEADY_TAU0, "steps": STEADY_STEPS, "block": BLOCK,
               "u_in": sim.u_in, "area_cells": half_area_cells(d["solid"], dims), "guarded": o.guarded(),
               "reference": "fp64 oracle (oracle/wt_oracle.hpp)", "blocks": blocks}
        with open(OUT_STEADY, "w") as f:
            json.dump(rec, f)
        print("wrote", OUT_STEADY)
        return
    dims, origin, h, sim, shape = case()
    n = int(np.prod(dims))
    members = []
    area = None
    for m in range(args.members):
        t0 = time.time()
        o = pyoracle.Oracle(dims, origin, h, sim, fp64=True)
        o.voxelize(shape)
        o.reset()
        d = o.read(reset_forces=True)
        fluid = d["solid"] == 0
        area = half_area_cells(d["solid"], dims)
        if m:
            o.write_state(f=d["f"] + perturbation(m, n))
        f0, _ = o.read64()
        mass0 = float(f0[fluid, 3].sum())
        blocks = []
        for k in range(STEPS // BLOCK):
            o.steps(BLOCK)
            blocks.append((o.read(reset_forces=True)["forces64"] / BLOCK).tolist())
        f1, _ = o.read64()
        members.append({"member": m, "blocks": blocks, "mass0": mass0, "mass1": float(f1[fluid, 3].sum()),
                        "guarded": o.guarded()})
        print(f"member {m}: {time.time() - t0:.0f} s", flush=True)
    rec = {"dims": list(dims), "h": H, "seed": SEED, "steps": STEPS, "block": BLOCK, "perturbation": PERTURB,
           "u_in": sim.u_in, "area_cells": area, "reference": "fp64 oracle (oracle/wt_oracle.hpp)",
           "members": members}
    with open(OUT, "w") as f:
        json.dump(rec, f)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
