#!/usr/bin/env python3
"""Benchmark of the wind-tunnel simulation step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl wt|reference]
                    [--workload f1|cube] [--storage f32|f16|bf16]

One bench step = one frame of the reference engine's compute pass
(src/engine/engine.ts:708-712) at the headless check's 8 steps per frame:
8 D3Q19 collide-stream steps + 2 semi-Lagrangian heat passes, with the
per-component forces recorded every step.  Default workload: the generic
analytic F1 voxelized at 4.5 cm into a 256x96x80 half tunnel (FP32, moving
belt, heat from brakes/exhaust/radiator at T=1), synthetic geometry from a
seeded shape.  The FP32 lattice (157 MB of populations and cell words) is
larger than the 126 MB L2, so no flush is needed between timed steps; a
working set that fits the L2 (f16 / bf16 at this size: 83 MB) gets an L2
flush before each timed frame and kernel batch.

value   = MLUPS over the timed frames (inputs resident in HBM, CUDA events on
          the library's stream, max over ranks).
e2e     = the same metric through the public Python API (ctypes -> C ABI) with
          a per-frame parameter upload from host memory and a per-frame force
          readback to host, host wall clock.
roofline: the collide-stream kernel alone, 156 algorithmic B per lattice update
          (f32; 80 B for f16/bf16) over its CUDA-event duration.
cpu_baseline: the reference's shader arithmetic on the host cores (translated
          reference build when present, else the oracle port), bounded sample.
Multi-GPU (torchrun, N>1): independent replicas, one lattice per GPU (weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "f1-wind-tunnel_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

THROTTLE_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
    0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
    0x100: "display_clock_setting",
}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 5:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                bits = int(parts[4], 16) if parts[4].startswith("0x") else int(parts[4])
            except ValueError:
                continue
            for b, name in THROTTLE_BITS.items():
                if bits & b and name != "gpu_idle":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(storage):
    """Per-launch DRAM bytes of the collide-stream kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "collide_stream_traffic.json")) as f:
            t = json.load(f)
        return t.get(storage)
    except (OSError, ValueError):
        return None


def workload(args, rank):
    import windtunnel
    if args.workload == "cube":
        dims, origin, h, sim, shape = windtunnel.cube_config(storage=args.storage)
        desc = "half tunnel 128x64x64, cube edge 22 cells at x=40 on the floor, u_in 0.08, tau0 0.51, Cs 0.1, sponge 16"
    elif args.workload == "f1-512":
        dims, origin, h, sim, shape = windtunnel.workloads.f1_large_config(storage=args.storage, seed=args.seed + rank)
        desc = ("generic analytic F1 at 2.25 cm in a 512x192x160 half tunnel (15.7 M cells), seeded wing angles, "
                "u_in 0.08, tau0 0.51, Cs 0.1, sponge 16")
    else:
        dims, origin, h, sim, shape = windtunnel.f1_config(seed=args.seed + rank, storage=args.storage)
        desc = ("generic analytic F1 voxelized at 4.5 cm into a 256x96x80 half tunnel, seeded wing angles 5-25 deg, "
                "moving belt, heat sources at T=1, u_in 0.08, tau0 0.51, Cs 0.1, sponge 16")
    return dims, origin, h, sim, shape, desc


def cpu_baseline(args, seconds_budget=20.0):
    """The reference's arithmetic on all host cores, bounded sample of the same workload."""
    import windtunnel
    from oracle import pyoracle
    dims, origin, h, sim, shape, _ = workload(args, 0)
    kind = "reference" if pyoracle.ref_lib() is not None and args.storage == "f32" else "port"
    if kind == "reference":
        m = pyoracle.Reference(dims, origin, h, sim)
        threads = pyoracle.ref_lib().wtr_threads()
    else:
        m = pyoracle.Oracle(dims, origin, h, sim)
        threads = pyoracle.oracle_lib().wto_threads()
    m.voxelize(shape)
    m.reset()
    n = int(dims[0] * dims[1] * dims[2])
    m.frame(2)  # warm-up
    frames, t0 = 0, time.perf_counter()
    while True:
        m.frame(8)
        frames += 1
        el = time.perf_counter() - t0
        if el > seconds_budget or frames >= args.cpu_frames:
            break
    mlups = n * 8 * frames / el / 1e6
    sample = f"{frames} frames x (8 LBM steps + 2 heat passes) of the {dims[0]}x{dims[1]}x{dims[2]} workload"
    return {"value": mlups, "unit": "MLUPS", "cores": int(threads), "kind": kind, "sample": sample,
            "seconds": el}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    base = cpu_baseline(args, seconds_budget=args.ref_seconds)
    dims = workload(args, 0)[:1][0]
    line = {
        "metric": "MLUPS", "value": base["value"], "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload(args, 0)[5], "cells": int(dims[0] * dims[1] * dims[2]),
                   "lbm_steps_per_step": 8, "heat_passes_per_step": 2},
        "cpu_baseline": {"value": base["value"], "unit": "MLUPS", "cores": base["cores"], "kind": base["kind"],
                         "sample": base["sample"]},
        "e2e": {"value": base["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_aeromap(args, rank, world, dist):
    """Batched aero map: all cases advanced by one launch per LBM step."""
    import torch
    import windtunnel
    from windtunnel.workloads import aeromap_cases
    cases = aeromap_cases(seed=args.seed)
    sim = windtunnel.make_sim(storage=args.storage, **windtunnel.workloads.CONFIG_SIM)
    b = windtunnel.AeroBatch([(d, o, h) for d, o, h, _, _ in cases], sim=sim)
    for (d, o, h, shape, _), e in zip(cases, b.lattices):
        e.set_shape_raw(shape)
    tuned = b.tune()
    cells = sum(int(d[0] * d[1] * d[2]) for d, _, _, _, _ in cases)
    stream = torch.cuda.ExternalStream(b.stream())
    for _ in range(max(3, args.warmup)):
        b.step(8)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.step(8)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    value = cells * 8 * args.steps / (ms / 1e3) / 1e6
    bpl = windtunnel.workloads.bytes_per_lup(args.storage)
    peak, kind = measured_peaks()
    line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.storage, "data": "synthetic",
            "config": {"workload": f"batched aero map: {len(cases)} lattices ({cells} cells), 8 LBM steps per step, "
                                   "one launch per LBM step, CUDA graph", "block": f"{tuned[0]}x{tuned[1]} (autotuned)"},
            "roofline": {"bound": "hbm", "achieved": cells * bpl * 8 * args.steps / (ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "peak_source": kind}}
    line["roofline"]["frac"] = line["roofline"]["achieved"] / peak
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()


def run_aeromap_converge(args, rank, world):
    """The aero-map metric: seconds until all 33 cases' windowed Cd and Cl are
    within 1 % of their long-run FP32 values (windtunnel.studies.convergence_times):
    plain FP32 cold one case after another, batched FP32 cold, batched FP32 and
    FP16 warm-started.  value = the batched FP16 warm-started time (the north
    star's method); the other three are in `times`."""
    from windtunnel import studies
    cases, labels = studies.sweep_cases(False)
    model = studies.load_model(os.path.join(PKG, "windtunnel", "data", "warmstart_f1.npz"))
    res = studies.convergence_times(cases, labels, args.horizon, model, log_fn=lambda m: None)
    if args.record:
        with open(args.record, "w") as f:
            json.dump(res, f, indent=1)
    if rank == 0:
        sec = res["seconds"]
        print(json.dumps({
            "metric": "aeromap_seconds_to_1pct", "value": sec["batched_fp16_warm"], "unit": "s", "n_gpus": world,
            "steps": args.horizon, "warmup": 0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f16", "data": "synthetic",
            "config": {"workload": f"aero map: 25 ride-height cases 256x96x80 + 8 uneven lattices, horizon "
                                   f"{args.horizon} steps, 1 % of the cold FP32 long-run Cd/Cl over 5760-step windows"},
            "times": sec, "speedup_vs_plain": res["speedup_vs_plain"], "not_converged": res["not_converged"]}),
              flush=True)


def surrogate_flops(batch, d, h, w):
    """Multiply-add FLOPs (2 per MAC) of one training step's convolutions: forward,
    data gradient (not for the first layer) and weight gradient of every layer."""
    from windtunnel.surrogate import Surrogate
    level = {"e0": 0, "e1": 1, "e2": 2, "e3": 3, "d2": 2, "d1": 1, "d0": 0, "he": 0}
    total = 0
    for name, cin, cout, taps, _ in Surrogate.LAYERS:
        lv = level[name[:2]]
        vox = batch * (d >> lv) * (h >> lv) * (w >> lv)
        mac = vox * cout * cin * taps
        total += 2 * mac * (2 if name == "e0a" else 3)
    return total


def run_surrogate(args, rank, world):
    """Training steps of the warm-start network (tensor-core convolutions) on
    synthetic inputs of the network's shape: samples/s and conv TFLOP/s."""
    import numpy as np
    import torch
    from windtunnel.surrogate import Surrogate
    B, D, H, W = 16, 24, 24, 64
    rng = np.random.default_rng(args.seed)
    model = Surrogate(seed=args.seed)
    x = torch.tensor(rng.standard_normal((B, D, H, W, 8)).astype(np.float32) * 0.5, device="cuda").to(torch.bfloat16)
    t = torch.tensor(rng.standard_normal((B, D, H, W, 4)).astype(np.float32) * 0.1, device="cuda")
    m = torch.ones((B, D, H, W), dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        model.train_step(x, t, m, 1e-4)
    torch.cuda.synchronize()
    model.ops.check()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(st)
        for _ in range(args.steps):
            model.train_step(x, t, m, 1e-4)
        e1.record(st)
        torch.cuda.synchronize()
    model.ops.check()
    ms = e0.elapsed_time(e1) / args.steps
    flops = surrogate_flops(B, D, H, W)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, kind = float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, kind = 1900.0, "fallback"
    tf = flops / (ms / 1e3) / 1e12
    clocks = clk.summary()
    line = {"metric": "samples/s", "value": B / (ms / 1e3), "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "warm-start network training step (forward, backward, Adam), batch 16 at "
                                   "64x24x24 with 8 input channels, 15 convolution layers",
                       "conv_flops_per_step": flops},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                         "traffic": None, "peak_source": kind,
                         "note": "convolution FLOPs over the whole step time (element-wise kernels included)"},
            "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]}}
    if rank == 0:
        print(json.dumps(line), flush=True)


MESH_DETAIL = 2.8  # stand-in mesh tessellation: about the W17 mesh's 268k triangles


def run_render(args, rank, world):
    """The render passes of the headless check's hero frame at 1280x720 (scene
    ray march, TAA, streamline glow, bloom, present) over a developed flow of
    the generic F1 at the medium quality (232x68x52): ms per frame.  e2e: the
    whole engine frame through the public API (8 LBM steps, heat, the
    streamline pass, the render passes) with the RGBA8 image read back."""
    import numpy as np
    import torch
    from oracle import pyoracle
    from windtunnel import AeroEngine
    from windtunnel.render import FrameState, make_look
    from windtunnel.viewer import HEADLESS_SHAPE, Viewer, orbit
    W, H = 1280, 720
    w17 = args.workload == "render-w17"
    eng = AeroEngine("medium")
    viewer = Viewer(eng, W, H, particles=1)
    shape_p = HEADLESS_SHAPE
    mesh = None
    if w17:
        from windtunnel.car_model import synthetic_w17
        from windtunnel.mesh_car import MeshCar, synthetic_mesh
        from windtunnel.viewer import W17_SHAPE
        shape_p = W17_SHAPE
        eng.set_car_model(synthetic_w17(shape_p))
        mesh = MeshCar(eng, synthetic_mesh(MESH_DETAIL))
        viewer.set_mesh(mesh)
    eng.set_shape(shape_p)
    eng.reset()
    cam = orbit({}, W / H)
    if args.profile:
        # whole engine frames only, few launches before them (for ncu captures):
        # 8 LBM steps, heat, the streamline pass and the render passes per frame
        t0 = time.perf_counter()
        for _ in range(args.steps):
            viewer.frame(cam, 8)
        eng.sync()
        if rank == 0:
            print(json.dumps({"profile_frames": args.steps, "s": time.perf_counter() - t0}), flush=True)
        if mesh is not None:
            mesh.close()
        viewer.close()
        eng.close()
        return
    for _ in range(40):                       # develop the flow
        viewer.frame(cam, 8)
    view = viewer.view_uniform()
    sp = viewer.stream_params()
    lines = eng.streamlines(sp, view)
    look = make_look(shape_p)
    r = viewer.renderer
    stream = torch.cuda.ExternalStream(eng.stream())
    mesh_args = dict(mesh=mesh, rig=eng.car_model.rig, params=shape_p) if w17 else {}

    def passes():
        r.frame(cam, look, view, lines=lines, flow_time=0.5, **mesh_args)

    for _ in range(max(3, args.warmup)):
        passes()
    eng.sync()
    steps = max(5, min(args.steps, 60))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(steps):
            passes()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the scene pass alone (the dominant kernel), and the mesh pass alone
    u = FrameState().next(cam, (W, H), lines=lines)
    look_s = look
    mesh_ms = None
    if w17:
        from windtunnel.mesh_car import mesh_cam
        mcam = mesh_cam(cam, (W, H), u.halton, shape_p)
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0.record(stream)
        for _ in range(steps):
            r.mesh(mesh, mcam, eng.car_model.rig)
        m1.record(stream)
        torch.cuda.synchronize()
        mesh_ms = m0.elapsed_time(m1) / steps
        look_s = type(look).from_buffer_copy(look)
        look_s.mesh_mode = 1
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(steps):
        r.scene(u.cam, look_s, view)
    s1.record(stream)
    torch.cuda.synchronize()
    scene_ms = s0.elapsed_time(s1) / steps
    # end to end: whole frames through the public API, image read back each frame
    e2e_frames = max(5, min(args.steps, 30))
    t0 = time.perf_counter()
    for _ in range(e2e_frames):
        viewer.frame(cam, 8)
        img = viewer.image()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_frames
    line_bytes = sp.lines * sp.steps * 16
    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not w17:
        # the render passes' dominant part, the scene pass, in the device code built
        # for the host, on all host cores: a band of rows, scaled to the full frame
        from windtunnel.engine import pack_shape
        if pyoracle.shade_model_lib() is not None:
            cores = os.cpu_count() or 1
            d = eng.debug_read()
            rows = list(range(0, H, 10))
            t0 = time.perf_counter()
            pyoracle.shade_model_render(pack_shape(HEADLESS_SHAPE), u.cam, look, view, eng.dims, eng.origin, eng.h,
                                        d["fields"], d["temps"], W, H, threads=cores, rows=rows)
            dt = time.perf_counter() - t0
            base = {"value": dt * 1e3 * H / len(rows), "unit": "ms/frame", "cores": cores, "kind": "port",
                    "sample": f"scene pass (RENDER fs_main) on every 10th row ({len(rows)} of {H}) of the 1280x720 "
                              "frame, device shading code compiled for the host, one row per task over all cores, "
                              "scaled by rows"}
    if rank == 0:
        clocks = clk.summary()
        print(json.dumps({
            "metric": "render_ms_per_frame", "value": ms, "unit": "ms", "n_gpus": world, "steps": steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": (
                           "headless-check hero frame at 1280x720 of the W17 scene drawn from its mesh: G-buffer "
                           f"pass of the stand-in mesh ({mesh.data.indices.size // 3} triangles, textured, 2 decal "
                           "draws), scene composite with ground reflection march, TAA, streamline glow (90 lines x "
                           "360 points), bloom, present; medium lattice 232x68x52 after 40 frames") if w17 else (
                           "headless-check hero frame at 1280x720: scene ray march of the generic F1, TAA, "
                           "streamline glow (90 lines x 360 points), bloom, present; medium lattice "
                           "232x68x52 after 40 frames"),
                       "image": [W, H], "scene_pass_ms": scene_ms, "mesh_pass_ms": mesh_ms,
                       "l2": "targets (29 MB) fit L2: the passes are compute-bound, no flush"},
            "roofline": None,
            "roofline_note": "scene pass: ALU / instruction-issue bound ray march, not HBM or tensor; "
                             "issue utilisation in profiles/render_scene_f1_1280x720.md",
            "cpu_baseline": base,
            "cpu_baseline_note": ("the mesh pass's CPU form is the oracle's pipeline around the reference's "
                                  "translated shaders, built only where the reference checkout is") if w17 else None,
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": line_bytes + 4 * 24 * 4,
                    "d2h_bytes_per_step": line_bytes + W * H * 4},
            "gpu_launches": steps * (7 + (14 if w17 else 0)),
            "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
        }), flush=True)
    if mesh is not None:
        mesh.close()
    viewer.close()
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200, help="timed frames")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="wt", choices=["wt", "reference"])
    ap.add_argument("--workload", default="f1", choices=["f1", "cube", "f1-512", "aeromap", "aeromap-converge",
                                                              "surrogate", "render", "render-w17"])
    ap.add_argument("--horizon", type=int, default=150000, help="aeromap-converge: LBM steps per case")
    ap.add_argument("--record", default=None, help="aeromap-converge: write the full JSON record here")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-frames", type=int, default=64, help="CPU-baseline frames (stops at 20 s)")
    ap.add_argument("--ref-seconds", type=float, default=60.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel-steps", type=int, default=64, help="LBM steps per kernel-timing launch batch")
    ap.add_argument("--kernel-seconds", type=float, default=1.5,
                    help="device time of the kernel-only timing region (clocks are sampled through it)")
    ap.add_argument("--e2e-frames", type=int, default=4000, help="at most this many end-to-end frames (~1.5 s)")
    ap.add_argument("--no-tune", action="store_true", help="skip the block-shape autotuner")
    ap.add_argument("--profile", action="store_true",
                    help="warm-up and timed frames only (for ncu captures); prints a short line")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        import __graft_entry__ as ge
        ge._build_oracle()
        run_reference_arm(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    import __graft_entry__ as ge
    if rank == 0:
        ge.build()
    if dist:
        dist.barrier()
    torch.cuda.set_device(local)
    torch.cuda.init()
    import windtunnel
    from windtunnel.workloads import bytes_per_lup
    if args.workload == "surrogate":
        run_surrogate(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in ("render", "render-w17"):
        run_render(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == "aeromap-converge":
        run_aeromap_converge(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == "aeromap":
        run_aeromap(args, rank, world, dist)
        if dist:
            dist.destroy_process_group()
        return

    dims, origin, h, sim, shape, desc = workload(args, rank)
    n = int(dims[0] * dims[1] * dims[2])
    eng = windtunnel.AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    eng.set_shape_raw(shape)
    tuned = None if args.no_tune else eng.tune()
    stream = torch.cuda.ExternalStream(eng.stream(), device=torch.device("cuda", local))
    lbm_per_frame = 8

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- warm-up
    for _ in range(max(3, args.warmup)):
        eng.step(lbm_per_frame, 2, lbm_per_frame / 2.0)
    eng.read_forces_raw()
    barrier()

    # Working set against L2.  When the populations and cell words fit the L2
    # (f16 / bf16 at 256x96x80: 83 MB), every timed frame and every kernel-only
    # batch starts after a write of twice the L2 size, outside its events; the
    # steps inside one frame still find the previous step's output in L2, as
    # they do in any run of that size.
    l2_bytes = int(getattr(torch.cuda.get_device_properties(local), "L2_cache_size", 126 << 20))
    ws_bytes = n * (19 * (4 if args.storage == "f32" else 2) + 4)
    flush_buf = None
    if ws_bytes < l2_bytes:
        flush_buf = torch.empty(2 * l2_bytes // 4, dtype=torch.int32, device=torch.device("cuda", local))
    l2_note = (f"working set (populations + cell words, {ws_bytes / 1e6:.0f} MB) larger than the "
               f"{l2_bytes / 2**20:.0f} MB L2; no flush" if flush_buf is None else
               f"working set ({ws_bytes / 1e6:.0f} MB) fits the {l2_bytes / 2**20:.0f} MB L2: a "
               f"{2 * l2_bytes / 2**20:.0f} MB write flushes it before each timed frame and kernel batch, "
               f"each timed on its own")

    def timed(fn, count):
        """Device milliseconds of `count` calls of fn on the engine's stream."""
        if flush_buf is None:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(count):
                fn()
            b.record(stream)
            barrier()
            return a.elapsed_time(b)
        pairs = []
        for _ in range(count):
            with torch.cuda.stream(stream):
                flush_buf.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            pairs.append((a, b))
        barrier()
        return sum(a.elapsed_time(b) for a, b in pairs)

    # ---- timed device region: K frames, inputs resident in HBM.  The clock
    # sampler stays on through the kernel-only region below, which runs for at
    # least --kernel-seconds of device time, so the clock record holds several
    # samples under load even when K frames take only milliseconds.
    clk = ClockSampler(local).__enter__()
    ms = timed(lambda: eng.step(lbm_per_frame, 2, lbm_per_frame / 2.0), args.steps)
    ms = max_over_ranks(ms)
    frames = args.steps
    total_cells = n * world
    value = total_cells * lbm_per_frame * frames / (ms / 1e3) / 1e6
    fr = eng.read_forces_raw()
    if args.profile:
        clk.__exit__(None, None, None)
        if rank == 0:
            print(json.dumps({"profile_frames": frames, "ms": ms, "mlups": value}), flush=True)
        eng.close()
        if dist:
            dist.destroy_process_group()
        return
    if fr.guarded:
        print(f"warning: {fr.guarded} cells hit the divergence guard", file=sys.stderr)
    # per frame: the step kernels and two heat passes; one force reduction per 64 steps
    launches_timed = args.steps * (lbm_per_frame + 2) + (args.steps * lbm_per_frame) // 64

    # ---- the collide-stream kernel alone: batches of kernel_steps steps, no heat,
    # repeated for at least --kernel-seconds of device time
    ks = max(2, args.kernel_steps - args.kernel_steps % 2)
    eng.step(ks, 0)
    barrier()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(4):
        eng.step(ks, 0)
    p1.record(stream)
    barrier()
    est = p0.elapsed_time(p1) / 4 / 1e3  # seconds per batch
    reps = max(8, int(args.kernel_seconds / max(est, 1e-6)) + 1)
    kernel_region_ms = timed(lambda: eng.step(ks, 0), reps)
    clk.__exit__(None, None, None)
    kms = kernel_region_ms / (reps * ks)  # per LBM step (one reduction launch per ks steps included)
    bpl = bytes_per_lup(args.storage)
    achieved = n * bpl / (kms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()

    # ---- end to end through the public API: per-frame parameter upload + force readback.
    # Every frame's forces come back to the host, read asynchronously like the
    # reference's mapped readback (engine.ts:746-760): frame k's copy is collected
    # while frame k+1 runs, and the last one before the clock stops.
    # about a second and a half of frames (at most --e2e-frames), so its host clock is not noise
    e2e_frames = max(5, min(args.e2e_frames, int(1500.0 / max(ms / frames, 1e-3))))
    barrier()
    t0 = time.perf_counter()
    prev = None
    for _ in range(e2e_frames):
        eng.set_sim(sim)                     # Sim uniform + sponge table upload (syncSim, engine.ts:497)
        eng.step(lbm_per_frame, 2, lbm_per_frame / 2.0)
        ticket = eng.read_forces_async(reset=True)   # maybeReadForces readback (engine.ts:746-747)
        if prev is not None:
            eng.collect_forces(prev)
        prev = ticket
    eng.collect_forces(prev)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = total_cells * lbm_per_frame * e2e_frames / e2e_s / 1e6
    h2d = dims[0] * 4
    d2h = 18 * 8 + 12 * 4 + 4

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(args)

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": frames,
            "warmup": max(3, args.warmup), "ms_per_step": ms / frames, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.storage, "data": "synthetic",
            "config": {
                "workload": desc, "cells": n, "lattice": list(dims), "lbm_steps_per_step": lbm_per_frame,
                "heat_passes_per_step": 2, "storage": args.storage, "parallelism": f"replicas x{world}",
                "l2": l2_note,
                "block": None if tuned is None else f"{tuned[0]}x{tuned[1]} (autotuned)",
                "launch": "CUDA graph per frame",
            },
            "roofline": {
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profiled_traffic(args.storage), "peak_source": peak_kind,
                "kernel": "collide-stream step", "algorithmic_bytes_per_lup": bpl,
                "kernel_ms_per_step": kms, "kernel_mlups": n / (kms / 1e3) / 1e6,
                "kernel_steps_timed": reps * ks, "kernel_region_ms": kernel_region_ms,
            },
            "cpu_baseline": base,
            "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches_timed,
            "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"],
                       "samples": clocks["samples"],
                       "window": "the timed frames and the kernel-only region that follows them"},
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
