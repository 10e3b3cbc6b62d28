"""The reference's check scripts on the GPU: scripts/wing-sensitivity.ts
(windtunnel.checks.wing_sensitivity) runs its settle / measure protocol and
shows the setup responses it is there to show (the runs are deterministic, so
these are fixed numbers, not a statistical test)."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_wing_sensitivity_straight_mode(wt_lib):
    from windtunnel.checks import wing_sensitivity
    rows = dict(wing_sensitivity(only="straight", log=lambda s: None))
    assert set(rows) == {"  base (ref)", "straight mode"}
    base, straight = rows["  base (ref)"], rows["straight mode"]
    for loads in (base, straight):
        assert loads.readings == 40                                   # 320 frames, a reading every 8
        assert all(math.isfinite(v) for v in vars(loads).values())
        assert 1000 < loads.drag < 20000                               # N at 250 km/h, medium lattice
    # flattening both flaps (DRS-like "straight mode") unloads the rear wing
    assert straight.rear_down < base.rear_down - 100


def test_wing_sensitivity_w17_runs(wt_lib):
    from windtunnel.checks import wing_sensitivity
    rows = wing_sensitivity(w17=True, only="rear: high", log=lambda s: None, warmup=200)
    assert [k for k, _ in rows] == ["  base (ref)", "rear: high"]
    assert all(math.isfinite(v) for _, l in rows for v in vars(l).values())
