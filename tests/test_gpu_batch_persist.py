"""The persistent batch launch against the launch-per-step batch, bit for bit.

One cooperative kernel advances every lattice of the batch by up to 64 steps
(the force-record capacity) with a grid barrier between steps; per tile it runs
the per-step batch kernel's arithmetic and writes the same force and mass
records.  Both launch kinds (WT_BATCH_PERSIST, read at wt_batch_create) run the
same scenario on lattices of four sizes, the 33x7x5 one with ragged tiles:

  * voxelization and a 70-step call (a 64-step persistent launch, the force
    reduction, a 6-step launch) with 2 heat passes,
  * re-voxelization of one lattice and an 8-step call,

and each lattice's checkpoint (populations in the storage format's bits, fields,
temperatures, outlet velocities, force and mass accumulators, guard count) and
per-step FP64 force records must agree, for FP32 and FP16 storage.  The FP32
batch path itself is bit-exact against the oracle (tests/test_gpu_batch.py)."""
import numpy as np
import pytest

from helpers import golden_shapes

pytestmark = pytest.mark.gpu


def _run(man, storage, persist, tmp_path, monkeypatch):
    from test_gpu_batch import cases
    from windtunnel import AeroBatch
    from windtunnel.engine import make_sim
    monkeypatch.setenv("WT_BATCH_PERSIST", "1" if persist else "0")
    cs = cases(man)
    sh = golden_shapes(man)
    b = AeroBatch([g for g, _ in cs], sim=make_sim(storage=storage))
    for (g, shape), e in zip(cs, b.lattices):
        e.set_shape_raw(shape)
    out = []
    for k, (n, heat) in enumerate(((70, 2), (8, 0))):
        if k == 1:
            b.lattices[0].set_shape_raw(sh["f1_v3"])
        b.step(n, heat, n / 2.0)
        for i, e in enumerate(b.lattices):
            hist = np.array(e.force_history(n))
            fr = e.read_forces_raw(reset=True)
            path = tmp_path / f"{storage}_{int(persist)}_{k}_{i}.wtc"
            e.save(str(path))
            out.append((hist, list(fr.raw), list(fr.sum), fr.mass, fr.guarded, fr.steps, path.read_bytes()))
    grid = b.persistent_grid()
    b.close()
    return out, grid


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_persistent_batch_bitexact(wt_lib, golden, storage, tmp_path, monkeypatch):
    _, man = golden
    step, g0 = _run(man, storage, False, tmp_path, monkeypatch)
    pers, g1 = _run(man, storage, True, tmp_path, monkeypatch)
    assert g0 == 0 and g1 > 0
    for k, (a, c) in enumerate(zip(step, pers)):
        assert np.array_equal(a[0], c[0]), f"record {k}: per-step forces differ"
        assert a[1:6] == c[1:6], f"record {k}: accumulators differ"
        assert a[6] == c[6], f"record {k}: lattice state differs"
    assert any(np.abs(a[0]).max() > 0 for a in step)
