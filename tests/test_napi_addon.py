"""The N-API addon of the TypeScript host (f1-wind-tunnel_gb300/napi/wt_napi.c),
without Node: compiled with -Wall -Wextra -Werror against a stand-in node_api.h
that declares the N-API functions it uses (tests/napi_mock/), linked with
libwt.so and a mock N-API runtime, and run.  The module registers every export,
marshals typed arrays and numbers into the C ABI and turns libwt's error codes
into thrown errors carrying wt_last_error's text.  (On a machine without a
GB300 wt_create fails, which exercises the error path; with one, the calls run.)"""
import os
import subprocess
import tempfile

from conftest import ROOT

SRC = os.path.join(ROOT, "f1-wind-tunnel_gb300", "napi", "wt_napi.c")
MOCK = os.path.join(ROOT, "tests", "napi_mock")
EXPORTS = ["create", "reset", "setSim", "setShape", "step", "readForces", "readForcesAsync", "collectForces",
           "debugRead", "save", "load", "resetFrom", "renderCreate", "renderFrame", "renderRead", "meshCreate",
           "renderMesh"]


def test_addon_compiles_and_runs(wt_lib):
    build = os.path.join(ROOT, "f1-wind-tunnel_gb300", "_build")
    inc = ["-I" + MOCK, "-I" + os.path.join(ROOT, "include")]
    flags = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror"]
    subprocess.run(flags + ["-fsyntax-only"] + inc + [SRC], check=True)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "napi_run")
        subprocess.run(flags + inc + [SRC, os.path.join(MOCK, "mock_napi.c"), "-L" + build, "-lwt",
                                      "-Wl,-rpath," + build, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    assert out[0] == f"exports {len(EXPORTS)}"
    assert [ln.split()[1] for ln in out[1:1 + len(EXPORTS)]] == EXPORTS
    calls = {ln.split()[0]: ln for ln in out[1 + len(EXPORTS):]}
    assert calls["create_bad"].startswith("create_bad threw create: origin and cell size")
    if calls["create"].startswith("create threw"):
        assert "libwt error -6" in calls["create"]  # no sm_103a device here
        assert calls["step_odd"].startswith("step_odd threw libwt error -1")
    else:
        assert calls["create"] == "create ok 0"
        assert "even" in calls["step_odd"]  # wt_step refuses an odd step count
        assert calls["step"] == "step ok 0" and calls["readForces"] == "readForces ok 8"
