"""Batched lattices (one launch per step for all of them, CUDA-graph replay) and
the autotuner, against the oracle run lattice by lattice.  Bit-exact."""
import numpy as np
import pytest

from helpers import golden_shapes

pytestmark = pytest.mark.gpu


def cases(man):
    from windtunnel import box_scene
    sh = golden_shapes(man)
    return [
        (((64, 24, 20), (-2.4, 0.0, 0.0), 0.135), sh["f1_default"]),
        (((48, 20, 16), (0.0, 0.0, 0.0), 0.05), box_scene((0.8, 0.25, 0.0), (0.2, 0.25, 0.2))),
        (((33, 7, 5), (0.0, 0.0, 0.0), 0.05), box_scene((0.6, 0.1, 0.0), (0.1, 0.1, 0.1))),
        (((96, 36, 30), (-2.4, 0.0, 0.0), 0.09), sh["f1_v2"]),
    ]


def run_oracle(oracle_mod, grid, shape, sim, frames):
    o = oracle_mod.Oracle(*grid, sim)
    o.voxelize(shape)
    o.reset()
    out = []
    for n in frames:
        o.frame(n)
        out.append(o.read(reset_forces=True))
    return out


def test_batch_bitexact_vs_oracle(wt_lib, oracle_mod, golden):
    from windtunnel import AeroBatch
    from windtunnel.engine import make_sim
    _, man = golden
    cs = cases(man)
    sim = make_sim()
    b = AeroBatch([g for g, _ in cs], sim=sim)
    for (g, shape), e in zip(cs, b.lattices):
        e.set_shape_raw(shape)
    frames = [8, 8, 8]
    want = [run_oracle(oracle_mod, g, shape, sim, frames) for g, shape in cs]
    for k, n in enumerate(frames):
        b.step(n, 2, n / 2.0)
        for i, e in enumerate(b.lattices):
            d = e.debug_read()
            od = want[i][k]
            np.testing.assert_array_equal(d["fields"], od["fields"], err_msg=f"lattice {i} frame {k}")
            np.testing.assert_array_equal(d["temps"], od["temps"])
            np.testing.assert_array_equal(e.read_populations(), od["f"])
            fr = e.read_forces_raw()
            assert list(fr.raw) == od["forces"].tolist()
            np.testing.assert_allclose(np.array(fr.sum[:]), od["forces64"], rtol=1e-9, atol=1e-9)
    b.close()


def test_tune_keeps_state(wt_lib, oracle_mod, golden):
    from windtunnel import AeroBatch, AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12)
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    e.set_shape_raw(shape)
    e.step(8, 0)
    before = e.read_populations()
    bx, by, ms = e.tune()
    assert bx * by <= 256 and bx % 32 == 0 and ms > 0
    np.testing.assert_array_equal(e.read_populations(), before)
    o = oracle_mod.Oracle(dims, origin, h, sim)
    o.voxelize(shape)
    o.reset()
    o.steps(8)
    e.read_forces_raw()
    o.read(reset_forces=True)
    e.step(8, 0)
    o.steps(8)
    np.testing.assert_array_equal(e.read_populations(), o.read()["f"])
    e.close()
    _, man = golden
    b = AeroBatch([((64, 24, 20), (-2.4, 0.0, 0.0), 0.135)] * 3, sim=sim)
    for l in b.lattices:
        l.set_shape_raw(shape)
    b.step(4)
    snap = [l.read_populations() for l in b.lattices]
    bx, by, ms = b.tune()
    for l, s in zip(b.lattices, snap):
        np.testing.assert_array_equal(l.read_populations(), s)
    b.close()


def test_batch_after_block_change_bitexact(wt_lib, oracle_mod, golden):
    """Mixed lattice sizes, the batch moved to another block shape (what the tuner
    does), then stepped: still bit-exact against the oracle."""
    from windtunnel import AeroBatch
    from windtunnel.engine import make_sim
    _, man = golden
    cs = cases(man)
    sim = make_sim()
    b = AeroBatch([g for g, _ in cs], sim=sim)
    for (g, shape), e in zip(cs, b.lattices):
        e.set_shape_raw(shape)
    b.step(2)  # tables and graph for the default shape
    bx, by, ms = b.tune()
    assert bx * by <= 256
    want = []
    for g, shape in cs:
        o = oracle_mod.Oracle(*g, sim)
        o.voxelize(shape)
        o.reset()
        o.steps(2)
        o.read(reset_forces=True)
        want.append(o)
    for e in b.lattices:
        e.read_forces_raw()
    b.step(8)
    b.step(8)
    for e, o in zip(b.lattices, want):
        o.steps(16)
        od = o.read(reset_forces=True)
        np.testing.assert_array_equal(e.read_populations(), od["f"])
        np.testing.assert_array_equal(e.debug_read()["fields"], od["fields"])
        assert list(e.read_forces_raw().raw) == od["forces"].tolist()
    b.close()
