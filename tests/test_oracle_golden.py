"""The oracle (CPU restatement) against the golden fixtures made by running the
reference's own shader text (tests/golden/make_golden.py).  Bit-exact."""
import os

import numpy as np
import pytest

from helpers import golden_shapes, replay, sha


def test_manifest_has_cases(golden):
    _, man = golden
    assert len(man["vox"]) >= 8 and len(man["lbm"]) >= 3
    assert man["translated_shaders_sha256"], "fixtures must record which shader text produced them"


@pytest.mark.parametrize("case", ["f1_default", "f1_v1", "f1_v2", "f1_v3", "cube", "sphere", "wing", "empty"])
def test_voxelize_matches_reference(oracle_mod, golden, case):
    gdir, man = golden
    c = man["vox"][case]
    g = c["grid"]
    o = oracle_mod.Oracle(g["dims"], g["origin"], g["h"])
    o.voxelize(golden_shapes(man)[case])
    d = o.read()
    ref = np.load(os.path.join(gdir, f"vox_{case}.npz"))
    np.testing.assert_array_equal(d["solid"], ref["solid"].astype(np.uint32))
    np.testing.assert_array_equal(d["emit"], ref["emit"])
    assert sha(d["solid"]) == c["solid_sha256"]
    assert sha(d["emit"]) == c["emit_sha256"]


@pytest.mark.parametrize("case", ["f1_revox", "f1_cfg", "f1_guard"])
def test_lattice_matches_reference(oracle_mod, golden, case):
    gdir, man = golden
    rec = man["lbm"][case]
    g = rec["grid"]
    from windtunnel.engine import make_sim
    u, t0, sm = rec["sim"]
    o = oracle_mod.Oracle(g["dims"], g["origin"], g["h"], make_sim(u_in=u, tau0=t0, smag=sm))
    o.reset()
    samples = np.load(os.path.join(gdir, f"lbm_{case}.npz"))
    for k, d in replay(o, man, case, lambda: o.read(reset_forces=True)):
        fr = rec["frames"][k]
        np.testing.assert_array_equal(d["fields"][::37], samples[f"fields_sample_{k}"])
        assert d["forces"].tolist() == fr["forces"]
        assert sha(d["fields"]) == fr["fields_sha256"]
        assert sha(d["f"]) == fr["f_sha256"]
        assert sha(d["temps"]) == fr["temps_sha256"]
    if case == "f1_guard":
        assert o.guarded() > 0


def test_link_mask_definition(oracle_mod, golden):
    """The oracle's link mask equals an independent numpy derivation from the solid
    flags with the reference's boundary precedence (wgsl.ts:207-221)."""
    _, man = golden
    c = man["vox"]["f1_default"]
    g = c["grid"]
    o = oracle_mod.Oracle(g["dims"], g["origin"], g["h"])
    o.voxelize(golden_shapes(man)["f1_default"])
    d = o.read()
    nx, ny, nz = g["dims"]
    s = d["solid"].reshape(nz, ny, nx)
    CX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
    CY = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
    CZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    want = np.zeros((nz, ny, nx), np.uint32)
    for i in range(1, 19):
        sx, sy, sz = x - CX[i], y - CY[i], z - CZ[i]
        ok = (sx >= 0) & (sx < nx) & (sy >= 0) & (sy < ny) & (sz < nz)
        szm = np.maximum(sz, 0)
        src = s[np.clip(szm, 0, nz - 1), np.clip(sy, 0, ny - 1), np.clip(sx, 0, nx - 1)]
        want |= np.where(ok & (src != 0) & (s == 0), np.uint32(1 << i), np.uint32(0))
    # belt bit (wgsl.ts:192-197)
    belt = np.zeros_like(want)
    yy = 0
    for zz in range(nz):
        for xx in range(nx):
            if s[zz, yy, xx]:
                continue
            xl, xr = max(xx - 2, 0), min(xx + 2, nx - 1)
            zl, zr = max(zz - 1, 0), min(zz + 1, nz - 1)
            if s[zz, 0, xl] or s[zz, 0, xr] or s[zz, 1, xx] or s[zl, 0, xx] or s[zr, 0, xx]:
                belt[zz, 0, xx] = 1 << 19
    want |= belt
    got = o.link_mask().reshape(nz, ny, nx)
    np.testing.assert_array_equal(got, want)
    assert (got != 0).sum() > 100
