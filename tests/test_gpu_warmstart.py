"""What the trained warm start gains over the cold start, evaluated by the LBM.

The committed network (windtunnel/data/warmstart_f1.npz, trained on seeds
1000-1399) predicts the coarse flow of two held-out cars (seeds 5000 and 5003);
the prediction replaces the uniform initial state through wt_reset_from.  A
long cold FP32 run of each car gives the late-time reference (mean over steps
18000-24000).  Over steps 2000-8000 the warm run's mean Cd and Cl must be
closer to that reference than the cold run's, and its predicted coarse field
closer to the cold run's late coarse field than the uniform inlet state is."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SEEDS = (5000, 5003)


@pytest.fixture(scope="module")
def runs(wt_lib):
    from windtunnel import warmstart as ws
    from windtunnel.studies import load_model, warm_fields
    here = os.path.dirname(os.path.abspath(ws.__file__))
    model = load_model(os.path.join(here, "data", "warmstart_f1.npz"))
    shapes = [ws.case_shape(s) for s in SEEDS]
    cases = [(ws.F1_DIMS, ws.F1_H, sh) for sh in shapes]
    fields = warm_fields(model, shapes)
    cold = ws.run_cases(cases, 24000, storage="f32", average=(16000, 2000))
    warm = ws.run_cases(cases, 8000, warm=fields, storage="f32")
    return ws, fields, cold, warm


def test_prediction_is_closer_than_uniform_state(runs):
    ws, fields, cold, _ = runs
    for k in range(len(SEEDS)):
        late = cold["coarse"][k]            # [20, 24, 64, 4], mean over steps 16000-24000
        fluid = late[..., 3] != 1.0
        uniform = np.zeros_like(late)
        uniform[..., 0], uniform[..., 3] = ws.U_IN, 1.0
        e_pred = np.linalg.norm((fields[k] - late)[fluid][:, :3])
        e_unif = np.linalg.norm((uniform - late)[fluid][:, :3])
        print(f"\nseed {SEEDS[k]}: velocity error of the prediction {e_pred:.4f}, of the uniform state {e_unif:.4f}")
        assert e_pred < 0.5 * e_unif


def test_warm_start_forces_closer_to_late_values(runs):
    ws, _, cold, warm = runs
    for k in range(len(SEEDS)):
        ref_cd, ref_cl = float(np.mean(cold["cd"][k][18000:])), float(np.mean(cold["cl"][k][18000:]))
        c_cd, c_cl = float(np.mean(cold["cd"][k][2000:8000])), float(np.mean(cold["cl"][k][2000:8000]))
        w_cd, w_cl = float(np.mean(warm["cd"][k][2000:8000])), float(np.mean(warm["cl"][k][2000:8000]))
        err_c = abs(c_cd - ref_cd) / abs(ref_cd) + abs(c_cl - ref_cl) / abs(ref_cl)
        err_w = abs(w_cd - ref_cd) / abs(ref_cd) + abs(w_cl - ref_cl) / abs(ref_cl)
        print(f"\nseed {SEEDS[k]}: late Cd {ref_cd:.3f} Cl {ref_cl:.3f}; steps 2000-8000 cold Cd {c_cd:.3f} "
              f"Cl {c_cl:.3f} (error {err_c:.3f}), warm Cd {w_cd:.3f} Cl {w_cl:.3f} (error {err_w:.3f})")
        assert err_w < err_c
