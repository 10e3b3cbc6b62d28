"""Shifted low-precision population storage (f - w_i kept as f16 / bf16, the
step running its collision in FP32 on them) and plain f32 storage against the
FP64 oracle of the same case: the generic F1 at 96x36x30 in steady flow (tau0
0.6; at the benchmark's tau0 0.51 the wake is unsteady with several long-lived
states, and single-run window means are draws from that distribution - the
ensemble comparison of tests/test_gpu_precision_study.py covers that regime).

Two measures:
  * early |u| field (40 steps): relative L2 error;
  * Cd and Cl of the whole car averaged over steps 2040-6040, deterministic in
    steady flow.
Mass drift is reported too.

Measured on a GB300 (relative errors, early |u| / Cd / Cl):
  f32   2.1e-6 / 9.3e-6 / 1.1e-4
  f16   8.3e-5 / 1.6e-3 / 1.6e-2   (the textbook-order collision on the same
                                    storage: 1.3e-4 / 1.7e-3 / 1.8e-2)
  bf16  6.5e-4 / 1.2e-2 / 1.2e-1
At this coarse lattice (h 0.12) the f16 Cl error is above the 1 % target: Cl
is five times smaller than Cd here, so the same absolute force error weighs
five times more.  The 1 % check for f16 runs at 128x48x40 in
tests/test_gpu_precision_study.py (0.25 % / 0.6 %).  The bounds below are the
measured errors with margin, so that a regression of the storage formats shows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# stated bounds: early |u| relative L2, time-averaged Cd and Cl relative error
# (steady flow: the window means are deterministic)
BOUNDS = {"f32": (1e-5, 1e-3), "f16": (2e-3, 2.5e-2), "bf16": (2e-2, 0.2)}
TAU0_STEADY = 0.6
EARLY, BLOCK, BLOCKS, WINDOW = 40, 200, 30, slice(10, 30)


def coefficients(f9, u, area):
    fx = f9[..., 0] + f9[..., 3] + f9[..., 6]
    fy = f9[..., 1] + f9[..., 4] + f9[..., 7]
    q = 0.5 * u * u * area
    return 2 * fx / q, -2 * fy / q


@pytest.fixture(scope="module")
def fp64_run(oracle_mod):
    from windtunnel import f1_config, half_area_cells
    from windtunnel.engine import make_sim
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=5)
    sim = make_sim(u_in=sim.u_in, tau0=TAU0_STEADY, smag=sim.smag, sponge_cells=sim.sponge_cells)
    o = oracle_mod.Oracle(dims, origin, h, sim, fp64=True)
    o.voxelize(shape)
    o.reset()
    o.steps(EARLY)
    early, _ = o.read64()
    d = o.read(reset_forces=True)
    hist = []
    for k in range(BLOCKS):
        o.steps(BLOCK)
        hist.append(o.read(reset_forces=True)["forces64"] / BLOCK)
    fields, _ = o.read64()
    area = half_area_cells(d["solid"], dims)
    return dict(dims=dims, origin=origin, h=h, sim=sim, shape=shape, early=early, fields=fields,
                forces=np.array(hist), solid=d["solid"], area=area)


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_storage_vs_fp64(wt_lib, fp64_run, storage):
    from windtunnel import AeroEngine, make_sim
    r = fp64_run
    s = r["sim"]
    sim = make_sim(u_in=s.u_in, tau0=s.tau0, smag=s.smag, sponge_cells=s.sponge_cells, storage=storage)
    e = AeroEngine(dims=r["dims"], origin=r["origin"], h=r["h"], sim=sim)
    e.set_shape_raw(r["shape"])
    e.step(EARLY, 0)
    early = e.debug_read()["fields"].astype(np.float64)
    e.read_forces_raw(reset=True)
    hist = []
    for k in range(BLOCKS):
        e.step(BLOCK, 0)
        hist.append(np.array(e.read_forces_raw(reset=True).sum[:]) / BLOCK)
    fr_mass = e.read_forces_raw(reset=False).mass
    e.close()
    fluid = r["solid"] == 0
    u64 = np.linalg.norm(r["early"][fluid, :3], axis=1)
    u = np.linalg.norm(early[fluid, :3], axis=1)
    err_u = np.linalg.norm(u - u64) / np.linalg.norm(u64)
    mass64 = r["fields"][fluid, 3].sum()
    cd64, cl64 = coefficients(r["forces"][WINDOW].mean(axis=0), s.u_in, r["area"])
    cd, cl = coefficients(np.array(hist)[WINDOW].mean(axis=0), s.u_in, r["area"])
    err_cd, err_cl = abs(cd - cd64) / abs(cd64), abs(cl - cl64) / abs(cl64)
    print(f"\n[{storage}] early |u| L2 rel {err_u:.3e}  Cd {cd:.4f} (fp64 {cd64:.4f}, rel {err_cd:.2e})  "
          f"Cl {cl:.4f} (fp64 {cl64:.4f}, rel {err_cl:.2e})  mass rel {abs(fr_mass - mass64) / mass64:.2e}")
    bu, bc = BOUNDS[storage]
    assert err_u < bu
    assert err_cd < bc and err_cl < bc
