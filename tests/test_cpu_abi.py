"""libwt's C ABI on a machine without a GPU: the library loads, exports every
entry point include/wt.h declares, the ctypes structures match the C layout,
and creating a context without an sm_103a device fails cleanly."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT


def declared():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(wt_[a-z_0-9]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(wt_lib):
    names = declared()
    assert len(names) >= 45
    for name in names:
        assert hasattr(wt_lib, name), f"libwt.so does not export {name}"
    assert wt_lib.wt_version().decode().endswith("sm_103a")


def test_struct_layout_matches_header():
    from windtunnel import _abi
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "wt.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(wt_grid), sizeof(wt_sim), sizeof(wt_shape), sizeof(wt_forces), sizeof(wt_info));
  printf("%zu %zu %zu %zu\n", offsetof(wt_shape, p_origin), offsetof(wt_shape, duct), offsetof(wt_shape, box_half), offsetof(wt_forces, mass));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = [int(x) for x in out[0].split()]
    offs = [int(x) for x in out[1].split()]
    assert sizes == [ctypes.sizeof(t) for t in (_abi.Grid, _abi.Sim, _abi.Shape, _abi.Forces, _abi.Info)]
    assert offs == [_abi.Shape.p_origin.offset, _abi.Shape.duct.offset, _abi.Shape.box_half.offset,
                    _abi.Forces.mass.offset]
    # the reference's Shape uniform is 24 words (wgsl.ts:9-18); the box extension follows it
    assert _abi.Shape.duct.offset == 23 * 4


def test_create_without_gpu_fails_cleanly(wt_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from windtunnel import AeroEngine, WindTunnelError
    with pytest.raises(WindTunnelError) as ei:
        AeroEngine(dims=(16, 8, 8), h=0.1)
    assert ei.value.code in (-6, -2)
