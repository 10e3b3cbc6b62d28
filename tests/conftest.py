import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "f1-wind-tunnel_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU (GB300); runs the CUDA path")
    config.addinivalue_line("markers", "slow: long CPU oracle run")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import pyoracle
    pyoracle.build_oracle()
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    import json
    gdir = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(gdir, "manifest.json")) as f:
        man = json.load(f)
    return gdir, man


@pytest.fixture(scope="session")
def wt_lib():
    """libwt built in-tree and loaded; on a GPU machine a missing or broken build is an error."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("wt_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import windtunnel
    return windtunnel.load()
