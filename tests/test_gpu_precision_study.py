"""Stored population formats (f32; f - w_i shifted into f16 / bf16, whose step
runs the moment-form collision in FP32; FP64 force and mass sums) against the
FP64 oracle on the precision case: the generic F1 (seed 5) at 128x48x40 cells
(tests/golden/make_precision.py makes the FP64 fixtures).

Steady flow (tau0 0.6, 8000 steps): the same car at ten times the viscosity,
where the wake is steady and window means are deterministic.  Cd and Cl averaged
over the last 1000 steps against the FP64 run:
    f32 within 1e-4, f16 within 1 % (the stated bound for FP16 storage), bf16 reported.

Unsteady flow (tau0 0.51, the benchmark's value, 20000 steps): the case has
several long-lived flow states, and FP64 runs that differ by a 1e-5 perturbation
of the initial populations end the 10000-20000 window apart by about 7 % in Cd
and 20 % in Cl.  A single run's window mean is a draw from that distribution,
so each format runs as an ensemble of MEMBERS members with the fixture's
perturbations (FP64: the fixture's members); per coefficient
    delta = (mean_F - mean_ref) / |mean_ref|,  se = sqrt(se_F^2 + se_ref^2) / |mean_ref|
    pass  |delta| + 2 se < 1 %;  fail  |delta| - 2 se > 1 %;  undecided otherwise,
against the FP64 ensemble and the f32 ensemble.  f32 must not fail against FP64
and f16 must not fail against f32.  The early field (step 40, before the
trajectories part) is compared with the unperturbed FP64 run.  With
WT_RECORD_DIR set, the JSON record is written there.  The 512x192x160 sweep
(f32 as the reference) runs when WT_STUDY=1."""
import json
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_precision as mp  # noqa: E402

MEMBERS = 32
EARLY, AVG_FROM = 40, 10000
BOUND = 0.01
STEADY_WINDOW = 1000  # last steps of the steady runs


def coefficients(f9, u, area):
    f9 = np.asarray(f9)
    fx = f9[..., 0] + f9[..., 3] + f9[..., 6]
    fy = f9[..., 1] + f9[..., 4] + f9[..., 7]
    q = 0.5 * u * u * area
    return 2 * fx / q, -2 * fy / q


def run_gpu(storage, member, early=False, tau0=None, steps=mp.STEPS):
    from windtunnel import AeroEngine, make_sim
    dims, origin, h, sim, shape = mp.case(tau0)
    s = make_sim(u_in=sim.u_in, tau0=sim.tau0, smag=sim.smag, sponge_cells=sim.sponge_cells, storage=storage)
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=s)
    e.set_shape_raw(shape)
    n = int(np.prod(dims))
    if member:
        e.write_state(f=e.read_populations() + mp.perturbation(member, n))
    e.read_forces_raw(reset=True)
    out = {}
    if early:
        e.step(EARLY, 0)
        out["early"] = e.debug_read()["fields"].astype(np.float64)
        e.close()
        return out
    blocks, mass = [], []
    for k in range(steps // mp.BLOCK):
        e.step(mp.BLOCK, 0)
        fr = e.read_forces_raw(reset=True)
        blocks.append(np.array(fr.sum[:]) / mp.BLOCK)
        mass.append(fr.mass)
    out["blocks"] = np.array(blocks)
    out["mass0"], out["mass1"] = mass[0], mass[-1]
    e.close()
    return out


def stats(values):
    v = np.asarray(values, np.float64)
    return float(v.mean()), float(v.std(ddof=1)), float(v.std(ddof=1) / np.sqrt(v.size))


def verdict(delta, se):
    if abs(delta) + 2 * se < BOUND:
        return "pass"
    if abs(delta) - 2 * se > BOUND:
        return "fail"
    return "undecided"


def compare(s, ref):
    delta = (s[0] - ref[0]) / abs(ref[0])
    se = float(np.hypot(s[2], ref[2]) / abs(ref[0]))
    return {"delta": float(delta), "se": se, "verdict": verdict(delta, se)}


@pytest.fixture(scope="module")
def fp64():
    with open(mp.OUT) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def study(wt_lib, oracle_mod, fp64):
    dims, origin, h, sim, shape = mp.case()
    u, area = fp64["u_in"], fp64["area_cells"]
    k0 = AVG_FROM // mp.BLOCK
    rec = {"lattice": list(dims), "h": h, "seed": mp.SEED, "steps": mp.STEPS, "block": mp.BLOCK,
           "window_unsteady": [AVG_FROM, mp.STEPS], "perturbation": mp.PERTURB, "bound": BOUND,
           "fp64_members": len(fp64["members"]), "gpu_members": MEMBERS}
    # ---- FP64 reference: window means of the ensemble members
    wm64 = [coefficients(np.array(m["blocks"])[k0:].mean(0), u, area) for m in fp64["members"]]
    rec["fp64"] = {"cd": stats([w[0] for w in wm64]), "cl": stats([w[1] for w in wm64]),
                   "members_cd": [float(w[0]) for w in wm64], "members_cl": [float(w[1]) for w in wm64],
                   "mass_drift": float(np.mean([(m["mass1"] - m["mass0"]) / m["mass0"] for m in fp64["members"]]))}
    # ---- early field (step 40) against the unperturbed FP64 run
    o = oracle_mod.Oracle(dims, origin, h, sim, fp64=True)
    o.voxelize(shape)
    o.reset()
    fluid = o.read()["solid"] == 0
    o.steps(EARLY)
    early64, _ = o.read64()
    u64 = np.linalg.norm(early64[fluid, :3], axis=1)
    runs = {st: [run_gpu(st, m) for m in range(MEMBERS)] for st in ("f32", "f16", "bf16")}
    # ---- steady flow: window means of the last STEADY_WINDOW steps against FP64
    with open(mp.OUT_STEADY) as f:
        st64 = json.load(f)
    kw = STEADY_WINDOW // mp.BLOCK
    s_cd64, s_cl64 = coefficients(np.array(st64["blocks"])[-kw:].mean(0), u, area)
    rec["steady"] = {"tau0": st64["tau0"], "steps": st64["steps"], "window": STEADY_WINDOW,
                     "fp64": {"cd": float(s_cd64), "cl": float(s_cl64)}}
    for st in ("f32", "f16", "bf16"):
        b = run_gpu(st, 0, tau0=st64["tau0"], steps=st64["steps"])["blocks"]
        cd, cl = coefficients(b[-kw:].mean(0), u, area)
        cdl, cll = coefficients(b[-2 * kw:-kw].mean(0), u, area)
        rec["steady"][st] = {"cd": float(cd), "cl": float(cl), "cd_rel_err": float(abs(cd - s_cd64) / abs(s_cd64)),
                             "cl_rel_err": float(abs(cl - s_cl64) / abs(s_cl64)),
                             "window_drift": float(max(abs(cd - cdl) / abs(cd), abs(cl - cll) / abs(cl)))}
    for st in ("f32", "f16", "bf16"):
        eg = run_gpu(st, 0, early=True)["early"]
        ug = np.linalg.norm(eg[fluid, :3], axis=1)
        wm = [coefficients(r["blocks"][k0:].mean(0), u, area) for r in runs[st]]
        r = {"u_l2_rel_step40": float(np.linalg.norm(ug - u64) / np.linalg.norm(u64)),
             "cd": stats([w[0] for w in wm]), "cl": stats([w[1] for w in wm]),
             "mass_drift": float(np.mean([(x["mass1"] - x["mass0"]) / x["mass0"] for x in runs[st]])),
             "members_cd": [float(w[0]) for w in wm], "members_cl": [float(w[1]) for w in wm]}
        r["vs_fp64"] = {c: compare(r[c], rec["fp64"][c]) for c in ("cd", "cl")}
        if st != "f32":
            r["vs_f32"] = {c: compare(r[c], rec["f32"][c]) for c in ("cd", "cl")}
        rec[st] = r
    print("\n" + json.dumps({k: v for k, v in rec.items()}, default=float))
    out = os.environ.get("WT_RECORD_DIR")
    if out:
        with open(os.path.join(out, "precision_f1_128x48x40.json"), "w") as f:
            json.dump(rec, f, indent=1)
    return rec


def test_fp64_fixture_is_the_oracle(fp64):
    dims, origin, h, sim, shape = mp.case()
    assert fp64["dims"] == list(dims) and fp64["steps"] == mp.STEPS and fp64["block"] == mp.BLOCK
    assert len(fp64["members"]) >= 4
    assert all(m["guarded"] == 0 for m in fp64["members"])


def test_early_fields_against_fp64(study):
    assert study["f32"]["u_l2_rel_step40"] < 1e-5
    assert study["f16"]["u_l2_rel_step40"] < 2e-3
    assert study["bf16"]["u_l2_rel_step40"] < 2e-2


def test_steady_flow_within_bounds(study):
    """The decidable bound: in steady flow f16 Cd and Cl within 1 % of FP64 and
    f32 within 1e-4.  The f32 window is settled (drift between the last two
    1000-step windows < 1e-4, so the FP64 comparison is deterministic); the f16
    window keeps a drift of about 6e-4 from its rounding, small against the
    1 % bound.  bf16 is recorded only (measured 1.9 % / 3.1 %)."""
    st = study["steady"]
    assert st["f32"]["window_drift"] < 1e-4, st["f32"]
    assert st["f16"]["window_drift"] < BOUND / 5, st["f16"]
    assert st["f32"]["cd_rel_err"] < 1e-4 and st["f32"]["cl_rel_err"] < 1e-4, st["f32"]
    assert st["f16"]["cd_rel_err"] < BOUND and st["f16"]["cl_rel_err"] < BOUND, st["f16"]


def test_unsteady_statistics(study):
    """f32 does not fail against the FP64 ensemble; f16 does not fail against the
    f32 ensemble (verdicts recorded for all formats)."""
    for c in ("cd", "cl"):
        assert study["f32"]["vs_fp64"][c]["verdict"] != "fail", study["f32"]["vs_fp64"]
        assert study["f16"]["vs_f32"][c]["verdict"] != "fail", study["f16"]["vs_f32"]


@pytest.mark.skipif(os.environ.get("WT_STUDY") != "1", reason="study: set WT_STUDY=1 (minutes)")
def test_precision_512x192x160(wt_lib):
    """The same car at 512x192x160 (15.7 M cells), f16 / bf16 against f32 (FP64 on
    the CPU is out of reach at this size): early field and window means."""
    from windtunnel import AeroEngine, make_sim
    from windtunnel.workloads import f1_large_config, half_area_cells
    dims, origin, h, sim, shape = f1_large_config(seed=5)

    def run(storage):
        s = make_sim(u_in=sim.u_in, tau0=sim.tau0, smag=sim.smag, sponge_cells=sim.sponge_cells, storage=storage)
        e = AeroEngine(dims=dims, origin=origin, h=h, sim=s)
        e.set_shape_raw(shape)
        e.step(EARLY, 0)
        early = e.debug_read()["fields"].astype(np.float64)
        e.read_forces_raw(reset=True)
        blocks = []
        for _ in range((mp.STEPS - EARLY) // mp.BLOCK):
            e.step(mp.BLOCK, 0)
            blocks.append(np.array(e.read_forces_raw(reset=True).sum[:]) / mp.BLOCK)
        solid = e.debug_read()["solid"]
        e.close()
        return early, np.array(blocks), solid

    runs = {s: run(s) for s in ("f32", "f16", "bf16")}
    solid = runs["f32"][2]
    fluid = solid == 0
    area = half_area_cells(solid, dims)
    k0 = (AVG_FROM - EARLY) // mp.BLOCK
    cd32, cl32 = coefficients(runs["f32"][1][k0:].mean(0), sim.u_in, area)
    u32 = np.linalg.norm(runs["f32"][0][fluid, :3], axis=1)
    out = {"lattice": list(dims), "steps": mp.STEPS, "reference": "f32"}
    for s in ("f16", "bf16"):
        cd, cl = coefficients(runs[s][1][k0:].mean(0), sim.u_in, area)
        ug = np.linalg.norm(runs[s][0][fluid, :3], axis=1)
        out[s] = {"u_l2_rel_step40": float(np.linalg.norm(ug - u32) / np.linalg.norm(u32)),
                  "cd_rel": float(abs(cd - cd32) / abs(cd32)), "cl_rel": float(abs(cl - cl32) / abs(cl32))}
    print("\n" + json.dumps(out))
    assert out["f16"]["u_l2_rel_step40"] < 1e-2
