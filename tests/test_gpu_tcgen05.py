"""The tcgen05 building blocks of the warm-start network's convolutions
(ofblend_gb300/csrc/flof_tcgen05.cuh) on the GPU: shared-memory layouts and
descriptors (no swizzle and 128-byte swizzle), the instruction descriptor,
tensor-memory allocation and loads.  tests/tcgen05_layouts.cu multiplies
small-integer BF16 matrices (exact in FP32) for N = 16..128 and compares
every entry."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = os.path.join(tempfile.mkdtemp(prefix="flof_tc_"), "tcgen05_layouts")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
           os.path.join(ROOT, "ofblend_gb300", "csrc"), os.path.join(ROOT, "tests", "tcgen05_layouts.cu"),
           "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


@pytest.mark.parametrize("layout", ["none", "sw128"])
def test_tcgen05_layouts_exact(gpu, exe, layout):
    r = subprocess.run([exe, layout], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK"), r.stdout
