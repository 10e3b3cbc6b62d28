"""What the trained warm start gains over the cold start, evaluated by the LBM.

The committed network (windtunnel/data/warmstart_f1.npz) was trained on 100
seeded cars (seeds 1000-1099), its targets the coarse (u, rho) fields of their
cold FP32 runs averaged over steps 75000-100000: the same window the
evaluation's reference comes from.  For two held-out cars (seeds 5003 and 5029) a cold and a
warm-started FP32 run go 100000 steps; the reference is the mean of the cold
run's Cd and Cl over its last quarter, and a run has converged at the first
step after which its trailing 5760-step means of Cd and Cl stay within 1 % of
it (windtunnel/warmstart.py).

Asserted, as recorded over the 50 held-out seeds in
profiles/warmstart_eval_f1.json:
  * the prediction is much closer to the cold run's late coarse field than the
    uniform inlet state is;
  * the cold runs converge at the recorded steps (55488 and 34247);
  * the warm-started runs do not converge: they settle in another long-lived
    flow state, more than 1 % from the cold reference in Cd or Cl at the end.
So the steps saved to 1 % are not positive: the LBM evaluation rejects this warm
start and the cold start (LBM_INIT, src/engine/wgsl.ts:141-155) remains the
path that gives the reference's answer."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SEEDS = (5003, 5029)
HORIZON = 100000
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def runs(wt_lib):
    from windtunnel import warmstart as ws
    from windtunnel.studies import load_model, warm_fields
    here = os.path.dirname(os.path.abspath(ws.__file__))
    model = load_model(os.path.join(here, "data", "warmstart_f1.npz"))
    shapes = [ws.case_shape(s) for s in SEEDS]
    cases = [(ws.F1_DIMS, ws.F1_H, sh) for sh in shapes]
    fields = warm_fields(model, shapes)
    cold = ws.run_cases(cases, HORIZON, storage="f32", average=(75000, 500))
    warm = ws.run_cases(cases, HORIZON, warm=fields, storage="f32")
    with open(os.path.join(ROOT, "profiles", "warmstart_eval_f1.json")) as f:
        record = {r["seed"]: r for r in json.load(f)["cases"]}
    return ws, fields, cold, warm, record


def test_prediction_is_closer_than_uniform_state(runs):
    ws, fields, cold, _, _ = runs
    for k in range(len(SEEDS)):
        late = cold["coarse"][k]            # [20, 24, 64, 4], mean over steps 75000-100000
        fluid = late[..., 3] != 1.0
        uniform = np.zeros_like(late)
        uniform[..., 0], uniform[..., 3] = ws.U_IN, 1.0
        e_pred = np.linalg.norm((fields[k] - late)[fluid][:, :3])
        e_unif = np.linalg.norm((uniform - late)[fluid][:, :3])
        print(f"\nseed {SEEDS[k]}: velocity error of the prediction {e_pred:.4f}, of the uniform state {e_unif:.4f}")
        assert e_pred < 0.5 * e_unif


def test_warm_start_steps_to_one_percent(runs):
    ws, _, cold, warm, record = runs
    for k, seed in enumerate(SEEDS):
        ref_cd, ref_cl = ws.reference_values(cold["cd"][k], cold["cl"][k])
        c = ws.convergence_step(cold["cd"][k], cold["cl"][k], ref_cd, ref_cl)
        w = ws.convergence_step(warm["cd"][k], warm["cl"][k], ref_cd, ref_cl)
        end_cd = float(ws.trailing_mean(warm["cd"][k])[-1])
        end_cl = float(ws.trailing_mean(warm["cl"][k])[-1])
        print(f"\nseed {seed}: reference Cd {ref_cd:.4f} Cl {ref_cl:.4f}; cold converges at {c}, warm at {w} "
              f"(warm ends at Cd {end_cd:.4f} Cl {end_cl:.4f})")
        rec = record[seed]
        assert abs(ref_cd - rec["ref_cd"]) <= 1e-9 * abs(rec["ref_cd"])
        assert abs(ref_cl - rec["ref_cl"]) <= 1e-9 * abs(rec["ref_cl"])
        assert c is not None and abs(c - rec["cold_steps"]) <= 64
        assert w is None and rec["warm_steps"] is None
        assert abs(end_cd - ref_cd) > 0.01 * abs(ref_cd) or abs(end_cl - ref_cl) > 0.01 * abs(ref_cl)
