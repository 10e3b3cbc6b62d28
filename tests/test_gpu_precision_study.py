"""Precision sweep of the stored population formats (f32, and f - w_i shifted into
f16 / bf16, collision in f32, FP64 force and mass sums) against an FP64 run of
the FP64 oracle: the generic F1 at 128x48x40 cells for 20000 steps, and the
same car at 512x192x160 cells (15.7 M cells) where FP64 on the CPU is out of
reach and f32 is the reference.

Reported per format: relative L2 error of |u| at step 40 (the flow is still
deterministic then), relative errors of Cd and Cl averaged over steps
10000-20000, and the relative drift of the fluid mass from its initial value.
This is a study (minutes of CPU for the FP64 oracle); it runs when
WT_STUDY=1 and prints one JSON line per lattice.  The pass criterion for f16 is
1 % or, where f32 arithmetic itself already differs more from FP64 (the
unsteady wake amplifies round-off), 1.25 x the f32 error."""
import json
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(os.environ.get("WT_STUDY") != "1",
                                                  reason="study: set WT_STUDY=1 (several minutes)")]

STEPS, BLOCK, EARLY, AVG_FROM = 20000, 200, 40, 10000


def coefficients(f9, u, area):
    fx = f9[..., 0] + f9[..., 3] + f9[..., 6]
    fy = f9[..., 1] + f9[..., 4] + f9[..., 7]
    q = 0.5 * u * u * area
    return 2 * fx / q, -2 * fy / q


def run_gpu(dims, h, shape, sim, storage):
    from windtunnel import AeroEngine, make_sim
    s = make_sim(u_in=sim.u_in, tau0=sim.tau0, smag=sim.smag, sponge_cells=sim.sponge_cells, storage=storage)
    e = AeroEngine(dims=dims, origin=(-2.4, 0.0, 0.0), h=h, sim=s)
    e.set_shape_raw(shape)
    e.read_forces_raw(reset=True)
    e.step(EARLY)
    early = e.debug_read()["fields"].astype(np.float64)
    m0 = e.read_forces_raw(reset=True).mass
    blocks = []
    for k in range((STEPS - EARLY) // BLOCK):
        e.step(BLOCK)
        f = e.read_forces_raw(reset=True)
        blocks.append(np.array(f.sum[:]) / BLOCK)
    m1 = f.mass
    solid = e.debug_read()["solid"]
    e.close()
    return early, np.array(blocks), m0, m1, solid


def summarize(ref, got, u, area, fluid):
    early_r, blocks_r, m0r, m1r = ref
    early, blocks, m0, m1 = got
    k0 = (AVG_FROM - EARLY) // BLOCK
    cd_r, cl_r = coefficients(blocks_r[k0:].mean(0), u, area)
    cd, cl = coefficients(blocks[k0:].mean(0), u, area)
    ur = np.linalg.norm(early_r[fluid, :3], axis=1)
    ug = np.linalg.norm(early[fluid, :3], axis=1)
    return {"u_l2_rel_step40": float(np.linalg.norm(ug - ur) / np.linalg.norm(ur)),
            "cd": float(cd), "cl": float(cl), "cd_ref": float(cd_r), "cl_ref": float(cl_r),
            "cd_rel_err": float(abs(cd - cd_r) / abs(cd_r)), "cl_rel_err": float(abs(cl - cl_r) / abs(cl_r)),
            "mass_drift_rel": float((m1 - m0) / m0), "mass_rel_vs_ref": float((m1 - m1r) / m1r)}


def test_precision_vs_fp64_oracle_128x48x40(wt_lib, oracle_mod):
    from windtunnel import f1_config, half_area_cells
    dims, origin, h, sim, shape = f1_config(dims=(128, 48, 40), h=0.09, seed=5)
    o = oracle_mod.Oracle(dims, origin, h, sim, fp64=True)
    o.voxelize(shape)
    o.reset()
    o.steps(EARLY)
    early, _ = o.read64()
    d = o.read(reset_forces=True)
    f0, _ = o.read64()
    solid = d["solid"]
    fluid = solid == 0
    m0 = f0[fluid, 3].sum()
    blocks = []
    for k in range((STEPS - EARLY) // BLOCK):
        o.steps(BLOCK)
        blocks.append(o.read(reset_forces=True)["forces64"] / BLOCK)
    f1, _ = o.read64()
    ref = (early, np.array(blocks), m0, f1[fluid, 3].sum())
    area = half_area_cells(solid, dims)
    out = {"lattice": list(dims), "steps": STEPS, "reference": "fp64 oracle"}
    for storage in ("f32", "f16", "bf16"):
        early_g, blocks_g, m0g, m1g, _ = run_gpu(dims, h, shape, sim, storage)
        out[storage] = summarize(ref, (early_g, blocks_g, m0g, m1g), sim.u_in, area, fluid)
    print("\n" + json.dumps(out))
    assert out["f32"]["u_l2_rel_step40"] < 1e-5
    # f32 itself drifts ~1.3 % from FP64 in these window means (the unsteady wake
    # amplifies round-off differences); f16 storage must stay within that floor
    for k in ("cd_rel_err", "cl_rel_err"):
        assert out["f16"][k] < max(0.01, 1.25 * out["f32"][k])


def test_precision_512x192x160(wt_lib):
    from windtunnel.workloads import f1_large_config, half_area_cells
    dims, origin, h, sim, shape = f1_large_config(seed=5)
    runs = {s: run_gpu(dims, h, shape, sim, s) for s in ("f32", "f16", "bf16")}
    solid = runs["f32"][4]
    fluid = solid == 0
    area = half_area_cells(solid, dims)
    ref = runs["f32"][:4]
    out = {"lattice": list(dims), "steps": STEPS, "reference": "f32"}
    for storage in ("f16", "bf16"):
        out[storage] = summarize(ref, runs[storage][:4], sim.u_in, area, fluid)
    print("\n" + json.dumps(out))
    assert out["f16"]["u_l2_rel_step40"] < 1e-2
