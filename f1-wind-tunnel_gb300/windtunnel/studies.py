"""Measured studies of the warm start and the batched aero map.

    python -m windtunnel.studies warmstart [--small] [--data-storage f32] --out DIR
        generate the training set (seeded 256x96x80 F1 runs, fields averaged
        late in the run: by default over steps 75000-100000 of FP32 cold runs,
        the window the evaluation takes its reference from), train the network
        on the GPU with libwt's kernels and save the weights.
    python -m windtunnel.studies evaluate --weights FILE [--small] --out DIR
        warm vs cold FP32 starts of held-out seeds, evaluated by the LBM.
    python -m windtunnel.studies sweep --weights FILE [--small] [--eval-steps N] --out DIR
        the 25-point ride-height aero map plus 8 uneven lattices: time to 1 %
        convergence of every case's windowed Cd and Cl, plain FP32 cold start
        one case after another vs batched FP32 cold, batched FP32 and FP16
        warm-started (bench.py --workload aeromap-converge prints the same).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import warmstart as ws
from .surrogate import Surrogate
from .warmstart import run_cases
from .workloads import aeromap_cases


def log(msg):
    print(f"[{time.strftime('%H:%M:%S')}] {msg}", flush=True)


def dataset(seeds, settle, average_steps, every, group=64, storage="f16"):
    """Features and time-averaged coarse targets of seeded F1 runs."""
    shapes = [ws.case_shape(s) for s in seeds]
    cases = [(ws.F1_DIMS, ws.F1_H, sh) for sh in shapes]
    run = ws.run_cases(cases, settle + average_steps, warm=None, storage=storage, average=(settle, every),
                       group=group, log=log)
    X, M, T = [], [], []
    for sh, coarse in zip(shapes, run["coarse"]):
        x, m = ws.features(sh)
        X.append(x)
        M.append(m)
        T.append(ws.normalize_target(coarse))
    return np.stack(X), np.stack(T), np.stack(M), run


def save_weights(model, path):
    st = model.state()
    np.savez_compressed(path, **{k: v.astype(np.float32) for k, v in st.items()})


def load_model(path, seed=0):
    m = Surrogate(seed=seed)
    with np.load(path) as z:
        m.load_state({k: z[k] for k in z.files})
    return m


def warm_fields(model, shapes):
    X = np.stack([ws.features(sh)[0] for sh in shapes])
    P = ws.predict(model, X)
    return [ws.denormalize(p) for p in P]


def evaluate(model, seeds, steps, group=64, storage="f32"):
    """Cold and warm runs of the held-out seeds: per-seed convergence steps."""
    shapes = [ws.case_shape(s) for s in seeds]
    cases = [(ws.F1_DIMS, ws.F1_H, sh) for sh in shapes]
    cold = ws.run_cases(cases, steps, storage="f32", group=group)
    warm = ws.run_cases(cases, steps, warm=warm_fields(model, shapes), storage=storage, group=group)
    rows = []
    for i, s in enumerate(seeds):
        rcd, rcl = ws.reference_values(cold["cd"][i], cold["cl"][i])
        c = ws.convergence_step(cold["cd"][i], cold["cl"][i], rcd, rcl)
        w = ws.convergence_step(warm["cd"][i], warm["cl"][i], rcd, rcl)
        rows.append({"seed": int(s), "ref_cd": rcd, "ref_cl": rcl, "cold_steps": c, "warm_steps": w,
                     "cold_steps_cd": ws.convergence_step_cd(cold["cd"][i], rcd),
                     "warm_steps_cd": ws.convergence_step_cd(warm["cd"][i], rcd)})
    return rows, cold, warm


def summarize_evaluation(rows, horizon):
    cold = np.array([r["cold_steps"] if r["cold_steps"] is not None else horizon for r in rows], float)
    warm = np.array([r["warm_steps"] if r["warm_steps"] is not None else horizon for r in rows], float)
    cold_cd = np.array([r["cold_steps_cd"] if r["cold_steps_cd"] is not None else horizon for r in rows], float)
    warm_cd = np.array([r["warm_steps_cd"] if r["warm_steps_cd"] is not None else horizon for r in rows], float)
    return {"cases": len(rows), "cold_mean_steps": float(cold.mean()), "warm_mean_steps": float(warm.mean()),
            "cold_mean_steps_cd_only": float(cold_cd.mean()), "warm_mean_steps_cd_only": float(warm_cd.mean()),
            "steps_saved_mean": float((cold - warm).mean()), "steps_saved_median": float(np.median(cold - warm)),
            "warm_better_or_equal": int((warm <= cold).sum()),
            "not_converged_cold": int(sum(r["cold_steps"] is None for r in rows)),
            "not_converged_warm": int(sum(r["warm_steps"] is None for r in rows))}


def study_warmstart(args):
    """Training set, training, validation loss and weights (the LBM evaluation is `evaluate`)."""
    os.makedirs(args.out, exist_ok=True)
    small = args.small
    n_train, n_val = (16, 4) if small else (args.train_cases, args.val_cases)
    settle, avg, every = (1200, 800, 200) if small else (args.settle, args.average, 500)
    t0 = time.time()
    train_seeds = list(range(1000, 1000 + n_train))
    val_seeds = list(range(5000, 5000 + n_val))
    log(f"generating {n_train} training + {n_val} held-out runs ({settle}+{avg} steps)")
    Xt, Tt, Mt, run_t = dataset(train_seeds, settle, avg, every, storage=args.data_storage)
    Xv, Tv, Mv, _ = dataset(val_seeds, settle, avg, every, storage=args.data_storage)
    t_data = time.time() - t0
    log(f"data done in {t_data:.1f} s; lattice step {np.mean(run_t['group_step_s']) * 1e3:.3f} ms per group step")
    model = Surrogate(seed=0)
    epochs = 6 if small else args.epochs
    t1 = time.time()
    hist = ws.train(model, Xt, Tt, Mt, epochs=epochs, batch=16 if not small else 8, lr=args.lr, log=log)
    t_train = time.time() - t1
    vloss = ws.validation_loss(model, Xv, Tv, Mv)
    zero = float(((Tv) ** 2 * Mv[..., None]).sum() / max(1.0, 4 * Mv.sum()))
    log(f"validation loss {vloss:.5f} (predicting the uniform inlet state: {zero:.5f})")
    wpath = os.path.join(args.out, "warmstart_f1.npz")
    save_weights(model, wpath)
    res = {"train_cases": n_train, "val_cases": n_val, "settle_steps": settle, "average_steps": avg,
           "data_storage": args.data_storage, "epochs": epochs, "train_loss": hist, "val_loss": vloss,
           "val_loss_uniform_state": zero, "data_seconds": t_data, "train_seconds": t_train,
           "lattice_step_s_per_group": run_t["group_step_s"]}
    with open(os.path.join(args.out, "warmstart_train.json"), "w") as f:
        json.dump(res, f, indent=1)


def study_evaluate(args):
    """Held-out seeds: cold and warm FP32 runs evaluated by the LBM."""
    os.makedirs(args.out, exist_ok=True)
    model = load_model(args.weights)
    seeds = list(range(5000, 5000 + (2 if args.small else args.val_cases)))
    horizon = 4000 if args.small else args.eval_steps
    rows, cold, warm = evaluate(model, seeds, horizon)
    summary = summarize_evaluation(rows, horizon)
    log(f"evaluation: {summary}")
    with open(os.path.join(args.out, "warmstart_eval.json"), "w") as f:
        json.dump({"horizon": horizon, "window": ws.WINDOW, "tolerance": ws.TOLERANCE, "cases": rows,
                   "summary": summary}, f, indent=1)
    # trailing-window means every 64 steps (the per-step series would be too large to keep)
    series = {}
    for i, r in enumerate(rows):
        for tag, run in (("cold", cold), ("warm", warm)):
            series[f"{tag}_cd_{r['seed']}"] = ws.trailing_mean(run["cd"][i])[63::64].astype(np.float32)
            series[f"{tag}_cl_{r['seed']}"] = ws.trailing_mean(run["cl"][i])[63::64].astype(np.float32)
    np.savez_compressed(os.path.join(args.out, "eval_window_means.npz"), **series)


def single_lattice_step_s(dims, h, shape, steps=2048):
    """Device seconds per LBM step of the plain path: one FP32 lattice through
    wt_step (autotuned block shape, graphed step sequences)."""
    import torch
    from .engine import AeroEngine, ORIGIN_X, make_sim
    from .workloads import CONFIG_SIM
    e = AeroEngine(dims=dims, origin=(ORIGIN_X, 0.0, 0.0), h=h, sim=make_sim(**CONFIG_SIM))
    try:
        e.set_shape_raw(shape)
        e.tune()
        e.step(512)
        st = torch.cuda.ExternalStream(e.stream())
        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(steps // 512):
            e.step(512)
        c.record(st)
        c.synchronize()
        return a.elapsed_time(c) / 1e3 / steps
    finally:
        e.close()


def sweep_cases(small=False):
    cases = aeromap_cases()
    if small:
        cases = cases[:3] + cases[25:27]
    return [(d, h, shape) for d, _, h, shape, _ in cases], [lab for *_, lab in cases]


def convergence_times(cases, labels, horizon, model, log_fn=log):
    """Seconds to 1 % convergence of every aero-map case (trailing 5760-step means
    of Cd and Cl within 1 % of the case's long-run value from its cold FP32 run,
    and staying there to the horizon), for four ways of running the map:
      plain FP32 cold, one case after another (single-lattice launches);
      batched FP32 cold; batched FP32 warm-started; batched FP16 warm-started.
    The batched FP32 run is bit-identical to the single-lattice one (same
    trajectories), so the plain path's time is every case's convergence step
    times its measured single-lattice step time; a batch takes as long as its
    slowest case.  A case that never converges counts the horizon (and is
    reported)."""
    cold = run_cases(cases, horizon, storage="f32")
    refs = [ws.reference_values(cold["cd"][i], cold["cl"][i]) for i in range(len(cases))]

    def steps_of(run):
        return [ws.convergence_step(run["cd"][i], run["cl"][i], *refs[i]) for i in range(len(cases))]

    cold_steps = steps_of(cold)
    t_single = {}
    for d, h, sh in cases:
        if d not in t_single:
            t_single[d] = single_lattice_step_s(d, h, sh)
    t0 = time.time()
    fields = warm_fields(model, [sh for _, _, sh in cases])
    t_infer = time.time() - t0
    warm32 = run_cases(cases, horizon, warm=fields, storage="f32")
    warm16 = run_cases(cases, horizon, warm=fields, storage="f16")
    w32, w16 = steps_of(warm32), steps_of(warm16)
    H = horizon

    def last(steps):
        return max((s if s is not None else H) for s in steps)

    plain_s = sum((c if c is not None else H) * t_single[d] for c, (d, _, _) in zip(cold_steps, cases))
    res = {"cases": labels, "horizon": H, "window": ws.WINDOW, "tolerance": ws.TOLERANCE,
           "cold_fp32_steps": cold_steps, "warm_fp32_batched_steps": w32, "warm_fp16_batched_steps": w16,
           "not_converged": {"cold_fp32": sum(c is None for c in cold_steps), "warm_fp32": sum(c is None for c in w32),
                             "warm_fp16": sum(c is None for c in w16)},
           "single_lattice_step_s": {"x".join(map(str, k)): v for k, v in t_single.items()},
           "batched_fp32_step_s": cold["group_step_s"][0], "batched_fp16_step_s": warm16["group_step_s"][0],
           "inference_s": t_infer,
           "seconds": {"plain_fp32_cold_sequential": plain_s,
                       "batched_fp32_cold": last(cold_steps) * cold["group_step_s"][0],
                       "batched_fp32_warm": last(w32) * warm32["group_step_s"][0] + t_infer,
                       "batched_fp16_warm": last(w16) * warm16["group_step_s"][0] + t_infer},
           "refs": refs}
    res["speedup_vs_plain"] = {k: plain_s / v for k, v in res["seconds"].items()}
    log_fn(json.dumps({k: v for k, v in res.items() if k not in ("cases", "refs", "cold_fp32_steps",
                                                              "warm_fp32_batched_steps", "warm_fp16_batched_steps")}))
    return res


def study_sweep(args):
    """Time to 1 % convergence of all aero-map cases, four ways (convergence_times)."""
    os.makedirs(args.out, exist_ok=True)
    cases, labels = sweep_cases(args.small)
    horizon = 4000 if args.small else args.eval_steps
    log(f"{len(cases)} cases, horizon {horizon} steps")
    res = convergence_times(cases, labels, horizon, load_model(args.weights))
    with open(os.path.join(args.out, "sweep_study.json"), "w") as f:
        json.dump(res, f, indent=1)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["warmstart", "evaluate", "sweep"])
    ap.add_argument("--train-cases", type=int, default=400)
    ap.add_argument("--val-cases", type=int, default=50)
    ap.add_argument("--settle", type=int, default=75000)
    ap.add_argument("--average", type=int, default=25000)
    ap.add_argument("--data-storage", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--out", default="study_out")
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--eval-steps", type=int, default=100000)
    ap.add_argument("--weights", default=None)
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    {"warmstart": study_warmstart, "evaluate": study_evaluate, "sweep": study_sweep}[args.study](args)


if __name__ == "__main__":
    sys.exit(main())
