"""The C ABI from plain C: tests/c_client.c compiles against
include/flof_gb300.h with a C99 compiler, links the library, and runs."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_client.c")
LIBDIR = os.path.join(ROOT, "ofblend_gb300")


@pytest.fixture(scope="module")
def client():
    from ofblend_gb300 import build
    build.build()
    out = os.path.join(tempfile.mkdtemp(prefix="flof_c_"), "c_client")
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I",
           os.path.join(ROOT, "include"), SRC, "-L", LIBDIR, "-lflof_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-lm", "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_c_client_reports_missing_device(client):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    r = subprocess.run([client, "0"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "no device" in r.stdout


@pytest.mark.gpu
def test_c_client_solves(client):
    r = subprocess.run([client, "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("err ")
