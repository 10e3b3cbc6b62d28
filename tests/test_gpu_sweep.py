"""wt_aeromap_sweep (the reference's aero-map loop, src/ui/aeromap.ts:73-114, run
into the running flow of one lattice) against the same sequence driven call by
call through the public API on a second, identical lattice: serpentine order,
re-voxelization keeping the populations, settle readings dropped, force
readings scaled as engine.ts:750-753 and averaged.  Identical GPU work on both
sides, so the cells agree exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sweep_driver_matches_call_by_call(wt_lib):
    from windtunnel import AeroEngine, make_sim
    from windtunnel.sweep import serpentine
    from windtunnel.workloads import config_f1_shape
    dims, h, origin = (64, 24, 20), 0.18, (-2.4, 0.0, 0.0)
    sim = make_sim(u_in=0.08, tau0=0.51, smag=0.1, sponge_cells=16.0)
    front, rear = [0.02, 0.05], [0.03, 0.06, 0.09]
    settle, measure, every, kmh = 64, 128, 64, 250.0
    base = config_f1_shape(2)
    a = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    cells = a.aeromap_sweep(base, front, rear, settle, measure, every, kmh)
    b = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    u = float(np.float32(sim.u_in))
    hh = float(np.float32(h))
    v = kmh / 3.6
    for k, (i, j) in enumerate(serpentine(len(front), len(rear))):
        s = config_f1_shape(2)
        s.ride_h, s.rear_ride = front[i], rear[j]
        b.set_shape_raw(s)
        b.step(settle, 0)
        b.read_forces_raw(reset=True)
        down, drag = [0.0] * 3, [0.0] * 3
        n = measure // every
        for _ in range(n):
            b.step(every, 0)
            f = b.read_forces_raw(reset=True)
            scale = (1.0 / 10000.0 / f.steps) * 1.225 * (v / u) * (v / u) * hh * hh * 2.0
            for g in range(3):
                drag[g] += f.raw[3 * g] * scale
                down[g] += -f.raw[3 * g + 1] * scale
        c = cells[i][j]
        assert c.order == k and c.readings == n
        for g in range(3):
            assert c.group_down_n[g] == down[g] / n and c.group_drag_n[g] == drag[g] / n
        tot_down = tot_drag = 0.0  # plain left-to-right sums (Python's sum() compensates)
        for g in range(3):
            tot_down += down[g] / n
            tot_drag += drag[g] / n
        assert c.down_kg == tot_down / 9.81 and c.drag_n == tot_drag
        assert c.efficiency == tot_down / max(tot_drag, 1.0)
    a.close()
    b.close()
