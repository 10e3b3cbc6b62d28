"""Known answers of the lattice physics, independent of any reference run, on
the oracle (the GPU twin is tests/test_gpu_known_answers.py):

* uniform flow through the empty tunnel (velocity inlet, moving belt at the
  inlet speed, far field, symmetry plane, outlet) is a fixed point: an
  equilibrium start stays there to float round-off;
* momentum exchange on a single solid cell in uniform flow after one step is
  the analytic 2 rho u (wgsl.ts:221-223: every one of the 18 fluid neighbours
  bounces feq_opp(i) back and records -2 (v - w_i) c_i, which sums to
  2 sum_j (feq_j - w_j) c_j = 2 rho u), with no lift or side force;
* mass is conserved in a closed box: solid walls on every face but the
  symmetry plane z = 0 (half-way bounce-back returns each population to its
  cell; the mirror reflects it into one cell), a solid block inside.  The FP64
  oracle holds the fluid mass to round-off; the reference's FP32 arithmetic
  gains mass by the float weights' excess, 1/3, 1/18 and 1/36 as f32 literals
  (wgsl.ts:133) summing to 1 + 1.49e-8, each step;
* the heat pass (wgsl.ts:460-511) on a temperature field linear in x, in
  uniform flow without sources: the trilinear backtrace of a linear field and
  the mean of its six neighbours are exact, so each pass maps a + b x to
  (1 - cool) (a + b x - (1 - diffuse) b u dt) away from the boundaries.
"""
import numpy as np

U_IN = 0.08
DIMS = (48, 20, 16)


def uniform_equilibrium(n, u):
    cx = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], np.float64)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    feq = w * (1 + 3 * cx * u + 4.5 * (cx * u) ** 2 - 1.5 * u * u)
    return np.repeat(feq, n)


def single_cell(dims, x, y, z):
    n = int(np.prod(dims))
    solid = np.zeros(n, np.uint32)
    solid[x + dims[0] * (y + dims[1] * z)] = 1
    return solid, np.zeros(n, np.float32)


def test_uniform_flow_is_a_fixed_point(oracle_mod):
    from windtunnel.engine import make_sim
    o = oracle_mod.Oracle(DIMS, (0, 0, 0), 0.1, make_sim(u_in=U_IN, tau0=0.52, smag=0.15))
    o.reset()
    f0 = o.read()["f"].astype(np.float64)
    np.testing.assert_allclose(f0, uniform_equilibrium(int(np.prod(DIMS)), U_IN), atol=3e-8)
    o.steps(240)
    early = np.abs(o.read()["f"] - f0).max()
    o.steps(960)
    d = o.read()
    late = np.abs(d["f"] - f0).max()
    # float round-off of the moments and feq (a few ulp of 1/3), bounded: no drift
    assert early < 2e-6 and late < 2e-6 and late <= 1.5 * early
    np.testing.assert_allclose(d["fields"][:, 0], U_IN, atol=2e-6)
    np.testing.assert_allclose(d["fields"][:, 1:3], 0.0, atol=2e-6)
    np.testing.assert_allclose(d["fields"][:, 3], 1.0, atol=2e-6)


W_EXCESS = float(np.float64(np.float32(0.33333334)) + 6 * np.float64(np.float32(0.055555556))
                 + 12 * np.float64(np.float32(0.027777778)) - 1.0)   # 1.49e-8
BOX_DIMS = (48, 20, 16)
BOX_U = 0.05


def closed_box(dims=BOX_DIMS):
    """Solid flags (u32) of the closed box: walls at x = 0, nx-1, y = 0, ny-1,
    z = nz-1 and a block in the flow; z = 0 stays the symmetry plane."""
    nx, ny, nz = dims
    n = nx * ny * nz
    i = np.arange(n)
    x, y, z = i % nx, (i // nx) % ny, i // (nx * ny)
    solid = ((x == 0) | (x == nx - 1) | (y == 0) | (y == ny - 1) | (z == nz - 1)).astype(np.uint32)
    solid[(x >= 18) & (x < 24) & (y >= 6) & (y < 12) & (z < 5)] = 2
    return solid, np.zeros(n, np.float32)


def test_closed_box_conserves_mass(oracle_mod):
    from windtunnel.engine import make_sim
    solid, emit = closed_box()
    fluid = solid == 0
    sim = make_sim(u_in=BOX_U, tau0=0.52, smag=0.15)
    o64 = oracle_mod.Oracle(BOX_DIMS, (0, 0, 0), 0.1, sim, fp64=True)
    o64.set_solid(solid, emit)
    o64.reset()
    m0 = o64.read64()[0][fluid, 3].sum()
    o64.steps(2400)
    m = o64.read64()[0][fluid, 3].sum()
    assert abs(m - m0) <= 1e-12 * m0
    o32 = oracle_mod.Oracle(BOX_DIMS, (0, 0, 0), 0.1, sim)
    o32.set_solid(solid, emit)
    o32.reset()
    o32.steps(2)
    m2 = o32.read()["fields"][fluid, 3].astype(np.float64).sum()
    o32.steps(2398)
    d = o32.read()
    m = d["fields"][fluid, 3].astype(np.float64).sum()
    drift = (m - m2) / m2
    print(f"\nFP32 mass drift over 2398 steps {drift:.3e}, weights' excess x steps {2398 * W_EXCESS:.3e}")
    assert 0.5 * 2398 * W_EXCESS <= drift <= 1.5 * 2398 * W_EXCESS
    assert o32.guarded() == 0 and np.abs(d["fields"][fluid, :3]).max() < BOX_U


def test_heat_pass_on_a_linear_field(oracle_mod):
    from windtunnel.engine import make_sim
    dims = (32, 12, 10)
    nx, ny, nz = dims
    n = nx * ny * nz
    u, dt, a, b = 0.05, 4.0, 0.3, 0.01
    sim = make_sim(u_in=u, tau0=0.52, smag=0.15)
    o = oracle_mod.Oracle(dims, (0, 0, 0), 0.1, sim)
    o.set_solid(np.zeros(n, np.uint32), np.zeros(n, np.float32))
    o.reset()
    x = (np.arange(n) % nx).astype(np.float64)
    fields = np.zeros((n, 4), np.float32)
    fields[:, 0], fields[:, 3] = u, 1.0
    o.write_state(fields=fields, temps=(a + b * x).astype(np.float32))
    o.heat(dt)  # the frame's two passes
    got = o.read()["temps"].astype(np.float64)
    keep = (1.0 - sim.heat_cool) ** 2
    want = keep * (a + b * x - 2.0 * (1.0 - sim.heat_diffuse) * b * u * dt)
    inner = (x >= 3) & (x <= nx - 4)
    np.testing.assert_allclose(got[inner], want[inner], rtol=2e-6, atol=0)
    assert np.all(got[x == 0] < want[x == 0])  # the inlet side mixes in the T = 0 inflow


def test_single_cell_momentum_exchange(oracle_mod):
    from windtunnel.engine import make_sim
    o = oracle_mod.Oracle(DIMS, (0, 0, 0), 0.1, make_sim(u_in=U_IN, tau0=0.52, smag=0.15))
    o.set_solid(*single_cell(DIMS, 20, 6, 7))
    o.reset()
    o.steps(1)
    fx, fy, fz = o.read(reset_forces=True)["forces64"][:3]
    assert abs(fx - 2 * U_IN) < 1e-6 and abs(fy) < 1e-7 and abs(fz) < 1e-7
