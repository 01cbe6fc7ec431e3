"""Test configuration: the `gpu` marker, import paths and shared fixtures.

Tests marked `gpu` need a CUDA device and call the library through its C ABI; the rest run on
the CPU (oracle known answers, host logic, ABI symbol checks, multi-process gloo tests).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library through the C ABI)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    import py_oracle
    py_oracle.load()
    return py_oracle


@pytest.fixture(scope="session")
def pg():
    import prestige_gb300
    prestige_gb300.load()
    return prestige_gb300
