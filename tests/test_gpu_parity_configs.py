"""The CUDA path against the oracle at the benchmark configurations' own sizes.

C1  plain FP32 half tunnel 128x64x64, cube of edge 22 cells on the moving belt at
    x = 40, inlet 0.08, tau0 0.51, Cs 0.1, sponge 16; 1000 steps from the rest
    state.  Acceptance: fields within 1e-4 relative after step 1000 and the drag
    coefficient averaged over steps 500-999 within 0.5 %; both are asserted
    first, then the bit-exact claim (fields, populations, i32 fixed-point forces).
C2  generic F1 voxelized at 4.5 cm into 256x96x80 (the throughput lattice):
    solid flags, emission and bounce-back link masks bit for bit, then 25 frames
    of 8 collide-stream steps + 2 heat passes (200 steps) with fields,
    temperatures and per-frame forces bit for bit.

Reference semantics: LBM_STEP (src/engine/wgsl.ts:179-291), VOXELIZE
(wgsl.ts:305-321), the frame's dispatch loop (src/engine/engine.ts:708-712) and
the force readback (engine.ts:739-761)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FIELD_RTOL = 1e-4
CD_RTOL = 5e-3


def _cd(fx_sum, steps, u_in, area):
    from windtunnel.workloads import drag_coefficient
    return drag_coefficient(fx_sum / steps, u_in, area)


def test_c1_cube_1000_steps(wt_lib, oracle_mod):
    from windtunnel import AeroEngine, cube_config
    from windtunnel.workloads import half_area_cells
    dims, origin, h, sim, shape = cube_config()
    assert dims == (128, 64, 64)
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    o = oracle_mod.Oracle(dims, origin, h, sim)
    e.set_shape_raw(shape)
    o.voxelize(shape)
    o.reset()
    d = e.debug_read(links=True, emit=True)
    od = o.read()
    np.testing.assert_array_equal(d["solid"], od["solid"])
    np.testing.assert_array_equal(d["links"], o.link_mask())
    assert int((d["solid"] > 0).sum()) == 22 * 22 * 11
    area = half_area_cells(d["solid"], dims)

    # steps 0-499: settle; steps 500-999: the averaging window
    e.step(500, 0)
    o.steps(500)
    e.read_forces_raw(reset=True)
    o.read(reset_forces=True)
    e.step(500, 0)
    o.steps(500)
    fr = e.read_forces_raw(reset=True)
    od = o.read(reset_forces=True)
    d = e.debug_read()
    assert fr.steps == 500 and fr.guarded == 0 and o.guarded() == 0

    cd_gpu = _cd(fr.sum[0], 500, sim.u_in, area)
    cd_orc = _cd(od["forces64"][0], 500, sim.u_in, area)
    print(f"C1 cube: Cd(steps 500-999) GPU {cd_gpu:.6f} oracle {cd_orc:.6f} (area {area} cells)")
    assert abs(cd_gpu - cd_orc) <= CD_RTOL * abs(cd_orc)
    np.testing.assert_allclose(d["fields"], od["fields"], rtol=FIELD_RTOL, atol=1e-6)
    # the kernels keep the reference's operation order: every bit agrees
    np.testing.assert_array_equal(d["fields"], od["fields"])
    np.testing.assert_array_equal(e.read_populations(), od["f"])
    assert list(fr.raw) == od["forces"].tolist()
    np.testing.assert_allclose(np.array(fr.sum[:]), od["forces64"], rtol=1e-9, atol=1e-9)
    e.close()


def test_c2_f1_voxels_and_200_steps(wt_lib, oracle_mod):
    from windtunnel import AeroEngine, f1_config
    dims, origin, h, sim, shape = f1_config()
    assert dims == (256, 96, 80) and abs(h - 0.045) < 1e-12
    e = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    o = oracle_mod.Oracle(dims, origin, h, sim)
    e.set_shape_raw(shape)
    o.voxelize(shape)
    o.reset()
    d = e.debug_read(links=True, emit=True)
    od = o.read()
    np.testing.assert_array_equal(d["solid"], od["solid"])
    np.testing.assert_array_equal(d["emit"], od["emit"])
    np.testing.assert_array_equal(d["links"], o.link_mask())
    groups = np.bincount(d["solid"].astype(np.int64), minlength=4)
    assert groups[1] > 0 and groups[2] > 0 and groups[3] > 0  # body, front wing, rear wing
    assert (d["emit"] > 0).any()  # heat sources voxelized

    for k in range(25):
        e.step(8, 2, 4.0)
        o.frame(8)
        fr = e.read_forces_raw(reset=True)
        od = o.read(reset_forces=True)
        assert list(fr.raw) == od["forces"].tolist(), f"frame {k}"
        np.testing.assert_allclose(np.array(fr.sum[:]), od["forces64"], rtol=1e-9, atol=1e-9)
        if k % 6 == 0 or k == 24:
            d = e.debug_read()
            np.testing.assert_allclose(d["fields"], od["fields"], rtol=FIELD_RTOL, atol=1e-6)
            np.testing.assert_array_equal(d["fields"], od["fields"])
            np.testing.assert_array_equal(d["temps"], od["temps"])
    np.testing.assert_array_equal(e.read_populations(), od["f"])
    assert (od["temps"] > 0).any()
    e.close()
