"""Builds tests/cpp/test_host.cpp against the C++ host layer (libprestige_host.so) and runs it.

`cpu` checks need no device (equation front end, GPU plan); `gpu` checks run eq1, an SPH run and
the checkpointed adjoint through the C++ API on the GPU.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def test_binary(tmp_path_factory):
    from prestige_gb300 import build_lib
    build_lib.build()
    out = str(tmp_path_factory.mktemp("cpp") / "test_host")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-o", out, os.path.join(ROOT, "tests", "cpp", "test_host.cpp"),
           "-L", build_lib.OUT_DIR, "-lprestige_host", "-lprestige_gpu", "-Wl,-rpath," + build_lib.OUT_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_host_layer_cpu(test_binary):
    r = subprocess.run([test_binary, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_host_layer_gpu(test_binary):
    r = subprocess.run([test_binary, "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr + r.stdout
