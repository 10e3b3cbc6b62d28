"""Generate tests/golden/precision_fp64_128x48x40.json: the FP64 oracle's force
history of the precision case (generic F1, seed 5, 128x48x40 cells at 9 cm,
u_in 0.08, tau0 0.51, Cs 0.1, sponge 16), 20000 steps, for an ensemble of
members that differ only by a 1e-5 perturbation of the initial populations
(member 0 unperturbed).  The unsteady wake turns any difference of arithmetic
into a different trajectory after a few thousand steps; the spread of the
members' window means is the noise against which the stored formats are
judged (tests/test_gpu_precision_study.py).

    python tests/golden/make_precision.py [--members 4]

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


def case():
    from windtunnel import f1_config
    return f1_config(dims=DIMS, h=H, seed=SEED)


def perturbation(member, n):
    """Additive noise on the 19 n initial populations (reference order f[i n + idx])."""
    if member == 0:
        return np.zeros(19 * n, np.float32)
    rng = np.random.default_rng(1000 + member)
    return (PERTURB * rng.standard_normal(19 * n)).astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=4)
    args = ap.parse_args()
    from oracle import pyoracle
    from windtunnel import half_area_cells
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
