"""Test configuration: the `gpu` marker, import paths and shared fixtures.

Tests marked `gpu` need a CUDA device and the built library; everything else runs
on the CPU (the oracle, host-side logic, the library's exports and host loading).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "genesis-1.3-version4_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import build_oracle
    build_oracle.build_oracle()
    import g4oracle
    return g4oracle.oracle()


@pytest.fixture(scope="session")
def lib():
    build_path = os.path.join(PKG, "build.py")
    import importlib.util
    spec = importlib.util.spec_from_file_location("g4build", build_path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build()
    import g4gpu
    return g4gpu.load_library()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def test_plugins(tmp_path_factory):
    """The test diagnostic plugins (tests/plugins/g4_test_plugin.cpp) built with the
    host compiler: {"field": ..., "multi": ..., "beam": ...} paths."""
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(here, "plugins", "g4_test_plugin.cpp")
    inc = os.path.join(os.path.dirname(here), "include")
    out = tmp_path_factory.mktemp("plugins")
    libs = {}
    for name, defs in (("field", []), ("multi", ["-DG4_TEST_MULTI"]), ("beam", ["-DG4_TEST_BEAM"])):
        path = str(out / f"libg4test_{name}.so")
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", inc] + defs +
                              ["-o", path, src])
        libs[name] = path
    return libs
