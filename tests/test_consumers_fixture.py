"""The field-consumer fixture (tests/golden/consumers.npz) against the
reference's own shaders: where the translated reference is built (the build
container), rerunning it over the fixture's fields reproduces every output bit
for bit; everywhere, the fixture's contents are self-consistent."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)


def fixture():
    return np.load(os.path.join(GOLDEN, "consumers.npz"))


def test_fixture_is_consistent():
    z = fixture()
    fluid = z["fields"][:, 3] > 0
    assert fluid.sum() > 0.8 * len(fluid)
    s = z["sample"]
    assert np.all(s[:, 5] >= 0) and np.all(s[:, 5] <= 1.0 + 1e-6)
    p = z["particles"]
    c = p[:, :, 7]
    assert np.all(((c >= 0) & (c <= 1)) | (c == -1))                   # coloured, or respawned (-1) this pass
    assert (c >= 0).mean() > 0.8
    assert np.all(p[-1][:, 3] >= 1)                                     # ages advance
    for k in ("lines_rake", "lines_ring"):
        live = (z[k][..., 3] >= 0).sum(axis=1)
        assert live.min() > 10 and live.max() < z[k].shape[1]           # lines start and end


def test_reference_reproduces_fixture():
    from oracle import pyoracle
    if pyoracle.ref_lib() is None:
        pytest.skip("translated reference not built (needs the reference checkout)")
    import make_consumers as mc
    z = fixture()
    f, t = z["fields"], z["temps"]
    samp, vort = pyoracle.ref_sample_flow(mc.DIMS, mc.ORIGIN, mc.H, f, t, z["points"])
    assert np.array_equal(samp, z["sample"]) and np.array_equal(vort, z["vorticity"])
    parts = np.zeros((600, 8), np.float32)
    for k, (sm, cm, sc, fr) in enumerate(mc.passes()):
        pyoracle.ref_particles(mc.DIMS, mc.ORIGIN, mc.H, f, t, mc.psim(600, sm, cm, sc, fr), mc.view(), parts)
        assert np.array_equal(parts, z["particles"][k])
    a, b = mc.stream_params()
    assert np.array_equal(pyoracle.ref_streamlines(mc.DIMS, mc.ORIGIN, mc.H, f, t, a, mc.view()), z["lines_rake"])
    assert np.array_equal(pyoracle.ref_streamlines(mc.DIMS, mc.ORIGIN, mc.H, f, t, b, mc.view()), z["lines_ring"])
