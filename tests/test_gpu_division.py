"""The collision kernel divides by rho through one correctly rounded reciprocal
and a Markstein correction per quotient (div_rcp, wt_lattice.cuh).  This test
builds tests/cuda/div_check.cu and checks div_rcp against IEEE division bit for
bit over every significand against 4096 denominators in [0.3, 3] and 2^30
random pairs over the stated operand range."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "f1-wind-tunnel_gb300"))


def test_div_rcp_matches_ieee_division(tmp_path):
    import build
    exe = str(tmp_path / "div_check")
    subprocess.run([build.nvcc(), *[f for f in build.NVCC_FLAGS if f != "-lineinfo"], "-I", build.CSRC,
                    os.path.join(HERE, "cuda", "div_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout.split()
    bad, cases = int(out[0]), int(out[1])
    print(f"\n{bad} mismatches in {cases} quotients")
    assert cases > 30_000_000_000 and bad == 0
