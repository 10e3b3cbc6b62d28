"""Checkpoint and resume (wt_save / wt_load): a run saved mid-way and resumed in
a fresh context continues bit for bit like the uninterrupted run (populations,
fields, temperatures, both force accumulators, mass, step counters), for f32
and the shifted f16 storage; files of another lattice, damaged or truncated
files are refused."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def snapshot(e):
    d = e.debug_read()
    fr = e.read_forces_raw(reset=False)
    return (e.read_populations(), d["fields"], d["temps"], list(fr.raw), list(fr.sum), fr.mass, fr.steps,
            fr.guarded, e.info().steps_total)


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_resume_is_bitexact(wt_lib, tmp_path, storage):
    from windtunnel import AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=6, storage=storage)
    a = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    a.set_shape_raw(shape)
    for _ in range(4):
        a.step(8, 2, 4.0)
    a.read_forces_raw(reset=True)
    a.step(8, 2, 4.0)  # forces accumulated since the last read travel in the file
    path = str(tmp_path / "run.wtck")
    a.save(path)
    for _ in range(3):
        a.step(8, 2, 4.0)
    want = snapshot(a)
    # a fresh context with other parameters and another scene: the file restores all of it
    from windtunnel.engine import make_sim
    b = AeroEngine(dims=dims, origin=origin, h=h, sim=make_sim(u_in=0.05, tau0=0.6, storage=storage))
    b.load(path)
    for _ in range(3):
        b.step(8, 2, 4.0)
    got = snapshot(b)
    for x, y in zip(want, got):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y))
    # the history restarts at the load: the last 24 steps are there, not more
    assert b.force_history(24).shape == (24, 9)
    a.close()
    b.close()


def test_bad_files_are_refused(wt_lib, tmp_path):
    from windtunnel import AeroEngine, WindTunnelError, f1_config
    dims, origin, h, sim, shape = f1_config(dims=(64, 24, 20), h=0.18)
    a = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    a.set_shape_raw(shape)
    a.step(4, 2, 2.0)
    path = str(tmp_path / "a.wtck")
    a.save(path)
    raw = open(path, "rb").read()
    other = AeroEngine(dims=(64, 24, 22), origin=origin, h=h, sim=sim)
    with pytest.raises(WindTunnelError, match="does not match"):
        other.load(path)
    bad = bytearray(raw)
    bad[len(raw) // 2] ^= 0x40
    open(str(tmp_path / "b.wtck"), "wb").write(bytes(bad))
    with pytest.raises(WindTunnelError, match="checksum"):
        a.load(str(tmp_path / "b.wtck"))
    open(str(tmp_path / "c.wtck"), "wb").write(raw[: len(raw) - 100])
    with pytest.raises(WindTunnelError, match="truncated"):
        a.load(str(tmp_path / "c.wtck"))
    open(str(tmp_path / "d.wtck"), "wb").write(b"not a checkpoint at all")
    with pytest.raises(WindTunnelError, match="not a libwt checkpoint"):
        a.load(str(tmp_path / "d.wtck"))
    with pytest.raises(WindTunnelError):
        a.load(str(tmp_path / "missing.wtck"))
    a.load(path)  # the context still works after refused loads
    a.step(4, 2, 2.0)
    a.close()
    other.close()
