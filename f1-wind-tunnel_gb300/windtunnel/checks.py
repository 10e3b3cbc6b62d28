"""The reference's simulation check scripts as library functions.

    python -m windtunnel.checks wings [--w17] [--assets DIR] [--only LABEL]
        scripts/wing-sensitivity.ts: settle the generic F1 (or the W17) at the
        medium quality for 1200 frames, then for each setup case re-voxelize
        into the running flow, settle 200 frames and average the force readings
        of 320 frames (8 steps per frame, one reading every 8 frames, as
        engine.ts:739-761), each case after a fresh measurement of the base
        setup.  Prints and returns total / front-wing / rear-wing drag and
        downforce in N per case.

The headless check (scripts/headless-check.ts) is windtunnel.viewer.headless_check.
"""
import argparse
import json
import math
from dataclasses import dataclass, replace

from .engine import AeroEngine, ShapeKind, ShapeParams

# wing-sensitivity.ts:12 (heat sources off, 6 deg angle of attack, 12 cm ride)
BASE = ShapeParams(kind=ShapeKind.F1, frontWing=0, rearWing=0, sidepod=0, cover=0, nose=0, rearRideH=0.12,
                   rearMainDeg=0.0, gurney=False, frontWingOn=True, rearWingOn=True, rearShape=0, thinWings=False,
                   sidepods=0, cooling=1, frontFlapDeg=0.0, rearFlapDeg=0.0, rideH=0.12, aoaDeg=6.0,
                   heatBrakes=False, heatEngine=False, heatRad=False)
F1_CASES = [  # wing-sensitivity.ts:42-58
    ("base", {}),
    ("straight mode", {"rearFlapDeg": -28.0, "frontFlapDeg": -12.0}),
    ("front: outwash", {"frontWing": 1}),
    ("front: spoon", {"frontWing": 2}),
    ("front: low", {"frontWing": 3}),
    ("rear: high", {"rearWing": 1}),
    ("rear: low", {"rearWing": 2}),
    ("sidepod: zero", {"sidepod": 1}),
    ("sidepod: tub", {"sidepod": 2}),
    ("sidepod: high", {"sidepod": 3}),
    ("cover: wide", {"cover": 1}),
    ("cover: coke", {"cover": 2}),
    ("nose: short", {"nose": 1}),
    ("nose: high", {"nose": 2}),
    ("rake +8cm", {"rearRideH": 0.20}),
]
W17_CASES = [  # wing-sensitivity.ts:59-66
    ("base", {}),
    ("straight mode", {"rearFlapDeg": -28.0, "frontFlapDeg": -12.0}),
    ("front: high", {"frontWing": 1}),
    ("front: low", {"frontWing": 2}),
    ("rear: high", {"rearWing": 1}),
    ("rear: low", {"rearWing": 2}),
]


@dataclass
class Loads:
    """Mean of the force readings (N): total, front-wing and rear-wing drag and downforce."""
    drag: float
    down: float
    front_drag: float
    front_down: float
    rear_drag: float
    rear_down: float
    readings: int


def wing_sensitivity(w17=False, assets=None, only=None, quality="medium", warmup=1200, settle=200, measure=320,
                     kmh=250.0, log=print):
    """scripts/wing-sensitivity.ts; returns [(label, Loads), ...] in the script's order."""
    from .car_model import load_w17, synthetic_w17
    e = AeroEngine(quality)
    base = replace(BASE, kind=ShapeKind.W17, rideH=0.12, rearRideH=0.14) if w17 else BASE

    def set_shape(p):
        if w17:  # setShape hands the rig of p to the model (engine.ts:450-462)
            e.set_car_model(load_w17(assets, p) if assets else synthetic_w17(p))
        e.set_shape(p)

    frame_no = [0]
    acc = []

    def run(frames):
        for _ in range(frames):
            e.frame(8)
            frame_no[0] += 1
            if frame_no[0] % 8 == 0:  # maybeReadForces (engine.ts:739-741)
                acc.append(e.read_forces(kmh))

    rows = []

    def measure_case(label, changes):
        set_shape(replace(base, **changes))
        run(settle)
        acc.clear()
        run(measure)
        n = len(acc)
        loads = Loads(sum(r.dragN for r in acc) / n, sum(r.downforceN for r in acc) / n,
                      sum(r.frontWing.drag for r in acc) / n, sum(r.frontWing.down for r in acc) / n,
                      sum(r.rearWing.drag for r in acc) / n, sum(r.rearWing.down for r in acc) / n, n)
        rows.append((label, loads))
        log(f"{label:18s} total D/L {round(loads.drag)} {round(loads.down)} | front D/L {round(loads.front_drag)} "
            f"{round(loads.front_down)} | rear D/L {round(loads.rear_drag)} {round(loads.rear_down)}")

    set_shape(base)
    e.reset()
    run(warmup)
    for label, changes in (W17_CASES if w17 else F1_CASES):
        if only and only not in label:
            continue
        if label != "base":
            measure_case("  base (ref)", {})
        measure_case(label, changes)
    e.close()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description="the reference's simulation check scripts")
    sub = ap.add_subparsers(dest="cmd", required=True)
    w = sub.add_parser("wings", help="scripts/wing-sensitivity.ts")
    w.add_argument("--w17", action="store_true")
    w.add_argument("--assets", default=None, help="the reference's public/models directory (W17 assets)")
    w.add_argument("--only", default=None)
    w.add_argument("--json", action="store_true", help="print the rows as one JSON line at the end")
    a = ap.parse_args(argv)
    rows = wing_sensitivity(a.w17, a.assets, a.only)
    if a.json:
        print(json.dumps([{"label": k, **{f: (v if not isinstance(v, float) or math.isfinite(v) else None)
                                          for f, v in vars(l).items()}} for k, l in rows]))


if __name__ == "__main__":
    main()
