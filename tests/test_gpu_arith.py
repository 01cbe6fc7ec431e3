"""Builds tests/cpp/arith_check.cu with nvcc for sm_103a and runs it: the integer-only
double-to-double-word split (df_split_fast) against the hardware conversions, bit for bit, and the
Sterbenz subtraction (df_sub_close) against the f64 difference."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def test_double_word_helpers(tmp_path):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "arith_check")
    src = os.path.join(ROOT, "tests", "cpp", "arith_check.cu")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", exe, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
