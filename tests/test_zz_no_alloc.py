"""wt_forces_noalloc: the force probe for callers that cannot allocate device
memory (hosts that own every GPU buffer through their own allocator or share
the lattice through interop memory, and cannot create a wt_ctx).

It is called through the C ABI on device buffers the test allocates itself,
twice in a row, and must give the force that the existing path (wt_step +
wt_read_force_history) reports for the step that consumes the same state,
within the FP64 force tolerance the other GPU tests use."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL, ATOL = 1e-9, 1e-9


def noalloc_fn(lib):
    from windtunnel import _abi
    fn = lib.wt_forces_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(_abi.Forces)]
    return fn


def test_noalloc_forces_match_step_path(wt_lib):
    import torch
    from windtunnel import AeroEngine, _abi, f1_config

    fn = noalloc_fn(wt_lib)
    dims, origin, h, sim, shape = f1_config(dims=(96, 36, 30), h=0.12, seed=3)
    eng = AeroEngine(dims=dims, origin=origin, h=h, sim=sim)
    eng.set_shape_raw(shape)
    for _ in range(3):
        eng.step(8, 2)
    pops = eng.read_populations()
    d = eng.debug_read(emit=True)
    dev = torch.device("cuda", torch.cuda.current_device())
    f_d = torch.from_numpy(pops).to(dev)
    s_d = torch.from_numpy(d["solid"].view(np.int32)).to(dev)
    e_d = torch.from_numpy(d["emit"]).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)

    outs = []
    for _ in range(2):  # two calls in a row share the static scratch
        out = _abi.Forces()
        rc = fn(f_d.data_ptr(), s_d.data_ptr(), e_d.data_ptr(), dims[0], dims[1], dims[2], stream, ctypes.byref(out))
        assert rc == 0
        outs.append(out)

    # existing path: the next step takes its force from the same state
    eng.read_forces_raw(reset=True)
    eng.step(2, 0)
    fr = eng.read_forces_raw(reset=False)
    assert fr.guarded == 0
    rec = eng.force_history(2)[0]
    assert np.abs(rec).max() > 0
    for out in outs:
        np.testing.assert_allclose(np.array(out.sum[:]), rec, rtol=RTOL, atol=ATOL)
        assert out.steps == 1
    assert list(outs[0].raw) == list(outs[1].raw)
    assert list(outs[0].sum) == list(outs[1].sum)
    eng.close()


def test_noalloc_rejects_oversized_lattice(wt_lib):
    import torch
    from windtunnel import _abi

    fn = noalloc_fn(wt_lib)
    dev = torch.device("cuda", torch.cuda.current_device())
    tiny = torch.zeros(16, device=dev)
    out = _abi.Forces()
    rc = fn(tiny.data_ptr(), tiny.data_ptr(), None, 1024, 1024, 129, None, ctypes.byref(out))
    assert rc == -7  # WT_ERR_NOALLOC_LIMIT: more than WT_NOALLOC_MAX_CELLS cells
