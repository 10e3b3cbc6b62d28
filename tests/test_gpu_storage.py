"""Shifted low-precision population storage (f - w_i kept as f16 / bf16, collision
in f32) and plain f32 storage against the FP64 oracle of the same case.

Two measures, because the wake of the car is unsteady and instantaneous fields of
any two arithmetics drift apart by chaos after a few hundred steps:
  * early |u| field (40 steps, flow still deterministic): relative L2 error;
  * Cd and Cl of the whole car averaged over steps 2040-6040 (the benchmark spec's
    "within 1 % Cd/Cl of FP64" criterion for f16).
Mass drift is reported too."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# stated bounds: early |u| relative L2, time-averaged Cd and Cl relative error.
# f32 vs f64 already differ by ~0.5 % in window-averaged Cl (the unsteady wake
# decorrelates; this is the noise floor of a 4000-step window), f16 meets the
# 1 % target, bf16 does not (measured Cd ~6 %, Cl ~18 %) and is bounded loosely.
BOUNDS = {"f32": (1e-5, 1e-2), "f16": (2e-3, 1e-2), "bf16": (2e-2, 3e-1)}
EARLY, BLOCK, BLOCKS, WINDOW = 40, 200, 30, slice(10, 30)


def coefficients(f9, u, area):
    fx = f9[..., 0] + f9[..., 3] + f9[..., 6]
    fy = f9[..., 1] + f9[..., 4] + f9[..., 7]
    q = 0.5 * u * u * area
    return 2 * fx / q, -2 * fy / q


@pytest.fixture(scope="module")
def fp64_run(oracle_mod):
    from windtunnel import f1_config, half_area_cells
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=5)
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
