"""Known answers of the lattice physics on the GPU through the C ABI (the oracle
twin is tests/test_known_answers.py): uniform flow is a fixed point, the
single-cell momentum exchange is 2 rho u, a closed box keeps its mass up to the
float weights' excess per step, and the drag coefficient of the
reference's cube scene in the medium tunnel, averaged over steps 500-999, is the
README's Cd of about 1.04."""
import numpy as np
import pytest

from test_known_answers import (BOX_DIMS, BOX_U, DIMS, U_IN, W_EXCESS, closed_box, single_cell,
                                uniform_equilibrium)

pytestmark = pytest.mark.gpu


def test_uniform_flow_is_a_fixed_point_gpu(wt_lib):
    from windtunnel import AeroEngine
    from windtunnel.engine import make_sim
    e = AeroEngine(dims=DIMS, origin=(0, 0, 0), h=0.1, sim=make_sim(u_in=U_IN, tau0=0.52, smag=0.15))
    e.reset()
    f0 = e.read_populations().astype(np.float64)
    np.testing.assert_allclose(f0, uniform_equilibrium(int(np.prod(DIMS)), U_IN), atol=3e-8)
    e.step(240, 0)
    early = np.abs(e.read_populations() - f0).max()
    e.step(960, 0)
    late = np.abs(e.read_populations() - f0).max()
    assert early < 2e-6 and late < 2e-6 and late <= 1.5 * early
    d = e.debug_read()
    np.testing.assert_allclose(d["fields"][:, 0], U_IN, atol=2e-6)
    np.testing.assert_allclose(d["fields"][:, 3], 1.0, atol=2e-6)
    e.close()


def test_single_cell_momentum_exchange_gpu(wt_lib):
    from windtunnel import AeroEngine
    from windtunnel.engine import make_sim
    e = AeroEngine(dims=DIMS, origin=(0, 0, 0), h=0.1, sim=make_sim(u_in=U_IN, tau0=0.52, smag=0.15))
    e.set_solid(*single_cell(DIMS, 20, 6, 7))
    e.reset()
    e.step(2, 0)
    first = e.force_history(2)[0]       # the first step's per-component sums
    assert abs(first[0] - 2 * U_IN) < 1e-6 and abs(first[1]) < 1e-7 and abs(first[2]) < 1e-7
    e.close()


def test_closed_box_conserves_mass_gpu(wt_lib, oracle_mod):
    """The FP64 fluid mass the step kernel sums (wt_read_forces' mass) over 2398
    steps of the closed box grows by the f32 weights' excess per step, as the
    oracle's does, and agrees with the oracle's fields to FP64 summation order."""
    from windtunnel import AeroEngine
    from windtunnel.engine import make_sim
    solid, emit = closed_box()
    fluid = solid == 0
    sim = make_sim(u_in=BOX_U, tau0=0.52, smag=0.15)
    e = AeroEngine(dims=BOX_DIMS, origin=(0, 0, 0), h=0.1, sim=sim)
    e.set_solid(solid, emit)
    e.reset()
    e.step(2, 0)
    m2 = e.read_forces_raw(reset=True).mass
    e.step(2398, 0)
    fr = e.read_forces_raw(reset=True)
    drift = (fr.mass - m2) / m2
    print(f"\nGPU FP32 mass drift over 2398 steps {drift:.3e}, weights' excess x steps {2398 * W_EXCESS:.3e}")
    assert 0.5 * 2398 * W_EXCESS <= drift <= 1.5 * 2398 * W_EXCESS and fr.guarded == 0
    o = oracle_mod.Oracle(BOX_DIMS, (0, 0, 0), 0.1, sim)
    o.set_solid(solid, emit)
    o.reset()
    o.steps(2400)
    od = o.read()
    assert abs(fr.mass - od["fields"][fluid, 3].astype(np.float64).sum()) <= 1e-12 * fr.mass
    np.testing.assert_array_equal(e.debug_read()["fields"], od["fields"])
    e.close()


def test_cube_drag_coefficient_band(wt_lib):
    """The reference's own cube scene (wgsl.ts:105: a 1 m rounded cube at (2.6, 1, 0))
    in the medium tunnel (232x68x52) from the engine's default flow: the mean
    drag coefficient over steps 500-999 is the README's "Cd about 1.04" to a
    few percent (measured 1.067; the impulsively started flow keeps developing
    afterwards, to about 1.37 by step 12000)."""
    from windtunnel import AeroEngine
    from windtunnel.engine import ShapeKind, ShapeParams
    from windtunnel.workloads import drag_coefficient, half_area_cells
    e = AeroEngine("medium")
    e.set_shape(ShapeParams(kind=ShapeKind.Cube))
    e.reset()
    e.step(500, 0)
    e.read_forces_raw(reset=True)
    e.step(500, 0)
    fr = e.read_forces_raw(reset=True)
    area = half_area_cells(e.debug_read()["solid"], e.dims)
    cd = drag_coefficient(fr.sum[0] / fr.steps, e.sim.u_in, area)
    print(f"\ncube Cd over steps 500-999: {cd:.4f} (area {area} cells)")
    assert 0.95 < cd < 1.15
    e.close()
