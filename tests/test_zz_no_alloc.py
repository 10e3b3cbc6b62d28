"""wt_forces_noalloc: the force probe for callers that cannot allocate device
memory (hosts that own every GPU buffer through their own allocator or share
the lattice through interop memory, and cannot create a wt_ctx).

It is called through the C ABI on device buffers the test allocates itself,
twice in a row, and must give the force of the step that consumes the same
state: the FP64 sums against the existing path (wt_step +
wt_read_force_history) within the FP64 force tolerance the other GPU tests
use, the i32 fixed-point sums and the guard count bit for bit against one
oracle step from that state.  A second case injects cells that trip the
divergence guard (src/engine/wgsl.ts:238-243), whose forces the step drops."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL, ATOL = 1e-9, 1e-9


def noalloc_fn(lib):
    from windtunnel import _abi
    fn = lib.wt_forces_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p, ctypes.POINTER(_abi.Forces)]
    return fn


def _probe_twice(fn, dims, u_in, pops, d):
    import torch
    from windtunnel import _abi
    dev = torch.device("cuda", torch.cuda.current_device())
    f_d = torch.from_numpy(pops).to(dev)
    s_d = torch.from_numpy(d["solid"].view(np.int32)).to(dev)
    e_d = torch.from_numpy(d["emit"]).to(dev)
    u_d = torch.from_numpy(np.ascontiguousarray(d["fields"])).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    outs = []
    for _ in range(2):  # two calls in a row share the static scratch
        out = _abi.Forces()
        rc = fn(f_d.data_ptr(), s_d.data_ptr(), e_d.data_ptr(), u_d.data_ptr(), dims[0], dims[1], dims[2], u_in,
                stream, ctypes.byref(out))
        assert rc == 0
        outs.append(out)
    assert list(outs[0].raw) == list(outs[1].raw)
    assert list(outs[0].sum) == list(outs[1].sum)
    assert outs[0].guarded == outs[1].guarded
    return outs


def _oracle_one_step(oracle_mod, dims, origin, h, sim, shape, pops, fields):
    o = oracle_mod.Oracle(dims, origin, h, sim)
    o.voxelize(shape)
    o.write_state(f=pops, fields=fields)
    g0 = o.guarded()
    o.read(reset_forces=True)
    o.steps(1)
    od = o.read(reset_forces=True)
    return od["forces"].tolist(), od["forces64"], o.guarded() - g0


def _check(outs, eng, orc):
    raw, f64, guarded = orc
    eng.read_forces_raw(reset=True)
    eng.step(2, 0)
    rec = eng.force_history(2)[0]  # the first of the two steps consumes the probed state
    assert np.abs(rec).max() > 0
    for out in outs:
        np.testing.assert_allclose(np.array(out.sum[:]), rec, rtol=RTOL, atol=ATOL)
        np.testing.assert_allclose(np.array(out.sum[:]), f64, rtol=RTOL, atol=ATOL)
        assert list(out.raw) == raw  # bit-compatible with the reference's i32 accumulator
        assert out.guarded == guarded
        assert out.steps == 1


def test_noalloc_forces_match_step_path(wt_lib, oracle_mod):
    from windtunnel import AeroEngine, f1_config
    fn = noalloc_fn(wt_lib)
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=3)
    eng = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    eng.set_shape_raw(shape)
    for _ in range(3):
        eng.step(8, 2)
    pops = eng.read_populations()
    d = eng.debug_read(emit=True)
    outs = _probe_twice(fn, dims, sim.u_in, pops, d)
    orc = _oracle_one_step(oracle_mod, dims, origin, h, sim, shape, pops, d["fields"])
    assert orc[2] == 0 and outs[0].guarded == 0
    _check(outs, eng, orc)
    eng.close()


def test_noalloc_drops_guarded_cells(wt_lib, oracle_mod):
    """Cells next to the body with non-finite or huge populations: the step resets
    them by the divergence guard and drops their link forces; so does the probe."""
    from windtunnel import AeroEngine, f1_config
    fn = noalloc_fn(wt_lib)
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=3)
    n = int(np.prod(dims))
    eng = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    eng.set_shape_raw(shape)
    for _ in range(2):
        eng.step(8, 2)
    d = eng.debug_read(emit=True, links=True)
    boundary = np.flatnonzero((d["links"] & 0x7fffe) != 0)
    cells = boundary[np.linspace(0, boundary.size - 1, 9).astype(np.int64)]
    pops = eng.read_populations()
    for k, c in enumerate(cells):
        pops[np.arange(19) * n + c] = (np.nan, 50.0, -40.0)[k % 3]
    eng.write_state(f=pops)
    outs = _probe_twice(fn, dims, sim.u_in, pops, d)
    orc = _oracle_one_step(oracle_mod, dims, origin, h, sim, shape, pops, d["fields"])
    assert orc[2] >= len(cells)  # the injected cells (and neighbours pulling from them) are guarded
    _check(outs, eng, orc)
    eng.close()


def test_noalloc_rejects_bad_calls(wt_lib):
    import torch
    from windtunnel import _abi

    fn = noalloc_fn(wt_lib)
    dev = torch.device("cuda", torch.cuda.current_device())
    tiny = torch.zeros(16, device=dev)
    out = _abi.Forces()
    rc = fn(tiny.data_ptr(), tiny.data_ptr(), None, None, 1024, 1024, 129, 0.08, None, ctypes.byref(out))
    assert rc == -7  # WT_ERR_NOALLOC_LIMIT: more than WT_NOALLOC_MAX_CELLS cells
    rc = fn(tiny.data_ptr(), tiny.data_ptr(), None, None, 4, 3, 3, 0.08, None, ctypes.byref(out))
    assert rc == -1  # WT_ERR_ARG: below the 8x3x3 minimum lattice
