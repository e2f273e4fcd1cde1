"""Test configuration: the `gpu` marker, import paths and shared fixtures.

Tests marked `gpu` need a CUDA device and the built library; everything else runs
on the CPU (the oracle, host-side logic, the library's exports and host loading).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "genesis-1.3-version4_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
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
