"""Shared fixtures: the GB300 package (tags_gb300), the CPU oracle, golden data.

Tests marked ``gpu`` need a CUDA device and the built library; everything else
runs on CPU (oracle pins, host logic, library symbol checks).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libtags_gpu.so")


@pytest.fixture(scope="session")
def pkg():
    return entry.load_package()


@pytest.fixture(scope="session")
def orc_mod():
    return entry.load_oracle()


@pytest.fixture(scope="session")
def port(orc_mod):
    return orc_mod.get("port")


@pytest.fixture(scope="session")
def ref(orc_mod):
    if not orc_mod.available("ref"):
        pytest.skip("reference build (oracle/_ref) not present here")
    return orc_mod.get("ref")


@pytest.fixture(scope="session")
def gpu_pkg(pkg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    pkg.build()
    pkg.lib()
    return pkg


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
