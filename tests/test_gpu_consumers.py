"""The reference's field consumers on the GPU (wt_sample_flow, wt_particles_step,
wt_streamlines) bit for bit against the fixture generated from the reference's
own shaders (tests/golden/consumers.npz, tests/golden/make_consumers.py), over
the same fields and temperatures written into a lattice."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


@pytest.fixture(scope="module")
def setup(wt_lib):
    import make_consumers as mc
    from windtunnel import AeroEngine
    z = np.load(os.path.join(ROOT, "tests", "golden", "consumers.npz"))
    e = AeroEngine(dims=mc.DIMS, origin=mc.ORIGIN, h=mc.H)
    e.write_state(fields=z["fields"], temps=z["temps"])
    yield mc, z, e
    e.close()


def test_sample_flow_and_vorticity_bitexact(setup):
    mc, z, e = setup
    out, vort = e.sample_flow(z["points"], vorticity=True)
    assert np.array_equal(out, z["sample"])
    assert np.array_equal(vort, z["vorticity"])


def test_particle_passes_bitexact(setup):
    mc, z, e = setup
    parts = np.zeros((600, 8), np.float32)
    for k, (sm, cm, sc, fr) in enumerate(mc.passes()):
        e.particles_step(parts, mc.psim(600, sm, cm, sc, fr), mc.view())
        bad = np.nonzero(np.any(parts != z["particles"][k], axis=1))[0]
        assert len(bad) == 0, f"pass {k}: {len(bad)} particles differ, first {bad[:5]}"


def test_streamlines_bitexact(setup):
    mc, z, e = setup
    a, b = mc.stream_params()
    assert np.array_equal(e.streamlines(a, mc.view()), z["lines_rake"])
    assert np.array_equal(e.streamlines(b, mc.view()), z["lines_ring"])
