"""The CUDA path (libwt through its C ABI) against the oracle and the golden
fixtures.  Flags, emission and link masks are compared bit for bit; lattice
states bit for bit as well (the kernels keep the reference's float operation
order and are built without contraction).  The stated acceptance tolerance
for FP32 fields, 1e-4 relative, is asserted too, so a failure report shows
which bar broke."""
import os

import numpy as np
import pytest

from helpers import golden_shapes, replay, sha

pytestmark = pytest.mark.gpu
FIELD_RTOL = 1e-4


class GpuSim:
    """Adapter: the golden-script interface over windtunnel.AeroEngine."""

    def __init__(self, dims, origin, h, sim):
        from windtunnel import AeroEngine
        self.e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)

    def voxelize(self, shape):
        self.e.set_shape_raw(shape)

    def frame(self, steps):
        self.e.step(steps, 2, steps / 2.0)

    def reset(self):
        self.e.reset()

    def write_state(self, f=None, fields=None, temps=None):
        self.e.write_state(f=f, fields=fields, temps=temps)

    def read(self):
        d = self.e.debug_read()
        fr = self.e.read_forces_raw(reset=True)
        return dict(fields=d["fields"], temps=d["temps"], f=self.e.read_populations(),
                    forces=np.array(fr.raw[:], np.int32), forces64=np.array(fr.sum[:]), mass=fr.mass,
                    solid=d["solid"])


@pytest.mark.parametrize("case", ["f1_default", "f1_v1", "f1_v2", "f1_v3", "cube", "sphere", "wing", "empty"])
def test_voxelize_bitexact(wt_lib, oracle_mod, golden, case):
    from windtunnel import AeroEngine
    gdir, man = golden
    c = man["vox"][case]
    g = c["grid"]
    e = AeroEngine(dims=g["dims"], origin=g["origin"], h=g["h"])
    shape = golden_shapes(man)[case]
    e.set_shape_raw(shape)
    d = e.debug_read(links=True, emit=True)
    ref = np.load(os.path.join(gdir, f"vox_{case}.npz"))
    np.testing.assert_array_equal(d["solid"], ref["solid"].astype(np.uint32))
    np.testing.assert_array_equal(d["emit"], ref["emit"])
    o = oracle_mod.Oracle(g["dims"], g["origin"], g["h"])
    o.voxelize(shape)
    np.testing.assert_array_equal(d["links"], o.link_mask())
    info = e.info()
    assert info.fluid_cells == int((ref["solid"] == 0).sum())
    e.close()


@pytest.mark.parametrize("case", ["f1_revox", "f1_cfg", "f1_guard"])
def test_lattice_bitexact(wt_lib, oracle_mod, golden, case):
    from windtunnel.engine import make_sim
    gdir, man = golden
    rec = man["lbm"][case]
    g = rec["grid"]
    u, t0, sm = rec["sim"]
    sim = make_sim(u_in=u, tau0=t0, smag=sm)
    gpu = GpuSim(g["dims"], g["origin"], g["h"], sim)
    o = oracle_mod.Oracle(g["dims"], g["origin"], g["h"], sim)
    o.reset()
    oracle_frames = list(replay(o, man, case, lambda: o.read(reset_forces=True)))
    for k, d in replay(gpu, man, case, gpu.read):
        fr = rec["frames"][k]
        od = oracle_frames[k][1]
        # stated tolerance first, then the bit-exact claim
        np.testing.assert_allclose(d["fields"], od["fields"], rtol=FIELD_RTOL, atol=1e-6)
        np.testing.assert_array_equal(d["fields"], od["fields"])
        np.testing.assert_array_equal(d["f"], od["f"])
        np.testing.assert_array_equal(d["temps"], od["temps"])
        assert d["forces"].tolist() == fr["forces"]
        assert sha(d["fields"]) == fr["fields_sha256"]
        assert sha(d["f"]) == fr["f_sha256"]
        assert sha(d["temps"]) == fr["temps_sha256"]
        np.testing.assert_allclose(d["forces64"], od["forces64"], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("dims", [(8, 2, 2), (33, 7, 5), (300, 9, 6), (40, 40, 3)])
def test_odd_sizes_bitexact(wt_lib, oracle_mod, dims):
    """Ragged and minimal lattices: partial blocks, single-row faces, tiny z."""
    from windtunnel import box_scene, AeroEngine
    from windtunnel.engine import make_sim
    nx, ny, nz = dims
    h = 0.05
    sim = make_sim(u_in=0.07, tau0=0.52, smag=0.12)
    shape = box_scene((nx * h * 0.4, ny * h * 0.3, 0.0), (max(2, nx // 8) * h, max(1, ny // 4) * h, max(1, nz // 3) * h))
    e = AeroEngine(dims=dims, origin=(0, 0, 0), h=h, sim=sim)
    o = oracle_mod.Oracle(dims, (0, 0, 0), h, sim)
    e.set_shape_raw(shape)
    o.voxelize(shape)
    o.reset()
    for _ in range(3):
        e.step(4, 2, 2.0)
        o.frame(4)
        d = e.debug_read()
        od = o.read(reset_forces=True)
        fr = e.read_forces_raw()
        np.testing.assert_array_equal(d["solid"], od["solid"])
        np.testing.assert_array_equal(d["fields"], od["fields"])
        np.testing.assert_array_equal(e.read_populations(), od["f"])
        np.testing.assert_array_equal(d["temps"], od["temps"])
        assert list(fr.raw) == od["forces"].tolist()
    e.close()


def test_config_cube_bitexact(wt_lib, oracle_mod):
    """The benchmark's box geometry and collision parameters (sponge 16) at reduced size."""
    from windtunnel import AeroEngine, cube_config
    dims, origin, h, sim, shape = cube_config(dims=(64, 32, 32), edge=12, center_x=20)
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    o = oracle_mod.Oracle(dims, origin, h, sim)
    e.set_shape_raw(shape)
    o.voxelize(shape)
    o.reset()
    for _ in range(4):
        e.step(10, 0)
        o.steps(10)
    d = e.debug_read()
    od = o.read()
    np.testing.assert_array_equal(d["solid"], od["solid"])
    assert int((d["solid"] > 0).sum()) == 12 * 12 * 6
    np.testing.assert_array_equal(d["fields"], od["fields"])
    np.testing.assert_array_equal(e.read_populations(), od["f"])
    fr = e.read_forces_raw()
    assert list(fr.raw) == od["forces"].tolist()
    np.testing.assert_allclose(np.array(fr.sum[:]), od["forces64"], rtol=1e-9, atol=1e-9)
    e.close()


def test_errors_are_reported(wt_lib):
    from windtunnel import AeroEngine, WindTunnelError, Shape
    e = AeroEngine(dims=(16, 8, 8), h=0.1)
    with pytest.raises(WindTunnelError, match="even"):
        e.step(3)
    with pytest.raises(WindTunnelError, match="heat_passes"):
        e.step(2, 1)
    s = Shape()
    s.kind = 4  # the custom 2-D profile scene
    with pytest.raises(WindTunnelError, match="not built"):
        e.set_shape_raw(s)
    s.kind = 5  # the W17 scene without its model
    with pytest.raises(WindTunnelError, match="car model"):
        e.set_shape_raw(s)
    with pytest.raises(WindTunnelError):
        AeroEngine(dims=(4, 1, 1), h=0.1)
    from windtunnel.engine import make_sim
    with pytest.raises(WindTunnelError, match="relaxation time"):
        e.set_sim(make_sim(tau0=1e-4, sponge_amp=0.0, inlet_amp=0.0))
    with pytest.raises(WindTunnelError, match="relaxation time"):
        AeroEngine(dims=(16, 8, 8), h=0.1, sim=make_sim(tau0=float("nan")))
    e.step(2)  # the rejected parameters left the context usable
    e.close()


def test_state_roundtrip_and_history(wt_lib):
    from windtunnel import AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12)
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    e.set_shape_raw(shape)
    e.step(10, 2)
    f = e.read_populations()
    e.write_state(f=f)
    np.testing.assert_array_equal(e.read_populations(), f)
    hist = e.force_history(10)
    fr = e.read_forces_raw()
    np.testing.assert_allclose(hist.sum(axis=0), np.array(fr.sum[:]), rtol=1e-12, atol=1e-12)
    assert fr.steps == 10
    e.close()


def test_async_force_readback(wt_lib):
    """wt_read_forces_async + wt_forces_collect give what wt_read_forces gives,
    frame after frame, and refuse tickets whose slot was reused."""
    from windtunnel import AeroEngine, WindTunnelError, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(64, 24, 20), h=0.18)
    a = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    b = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    for e in (a, b):
        e.set_shape_raw(shape)
    tickets, sync = [], []
    for k in range(5):
        for e in (a, b):
            e.step(8, 2, 4.0)
        tickets.append(a.read_forces_async(reset=(k % 2 == 0)))
        sync.append(b.read_forces_raw(reset=(k % 2 == 0)))
    for t, f in zip(tickets, sync):
        g = a.collect_forces(t)
        assert list(g.raw) == list(f.raw) and list(g.sum) == list(f.sum)
        assert (g.mass, g.steps, g.guarded) == (f.mass, f.steps, f.guarded)
    assert sync[1].steps == 8 and sync[2].steps == 16
    first = a.read_forces_async()
    for _ in range(16):
        a.read_forces_async()
    with pytest.raises(WindTunnelError, match="ticket"):
        a.collect_forces(first)
    with pytest.raises(WindTunnelError, match="ticket"):
        a.collect_forces(first + 100)
    a.close()
    b.close()


def test_full_size_f1_properties(wt_lib):
    """256x96x80 F1 (the benchmark lattice): finite, deterministic run to run,
    per-step force records sum to the accumulator, mass stays near the initial."""
    from windtunnel import AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config()
    runs = []
    for _ in range(2):
        e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
        e.set_shape_raw(shape)
        for _ in range(5):
            e.step(8, 2)
        d = e.debug_read()
        fr = e.read_forces_raw(reset=False)
        hist = e.force_history(40)
        runs.append((sha(d["fields"]), sha(d["temps"]), list(fr.raw), fr.mass))
        fl = d["fields"]
        fluid = d["solid"] == 0
        assert np.isfinite(fl).all()
        assert fr.guarded == 0
        np.testing.assert_allclose(hist.sum(axis=0), np.array(fr.sum[:]), rtol=1e-12, atol=1e-12)
        assert abs(fr.mass / fluid.sum() - 1.0) < 0.05
        assert fr.raw[0] > 0  # body drag is positive
        e.close()
    assert runs[0] == runs[1]


def test_tune_between_steps_is_transparent(wt_lib):
    """Autotuning a lattice that has unreduced force records (steps taken since the
    last read) changes nothing: forces, mass and fields after more steps equal those
    of an untuned twin bit for bit.  (The tuner's block-shape changes free and
    re-create the per-block buffers the pending records are summed from.)"""
    from windtunnel import AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=4)
    a = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    b = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    for e in (a, b):
        e.set_shape_raw(shape)
        e.step(10, 0)
    a.tune()
    for e in (a, b):
        e.step(6, 0)
    fa, fb = a.read_forces_raw(), b.read_forces_raw()
    assert list(fa.raw) == list(fb.raw) and list(fa.sum) == list(fb.sum) and fa.mass == fb.mass
    assert fa.steps == fb.steps == 16
    assert np.array_equal(a.debug_read()["fields"], b.debug_read()["fields"])
    assert np.array_equal(a.force_history(16), b.force_history(16))
    a.close()
    b.close()
