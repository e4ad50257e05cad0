"""The C ABI library without a GPU: it builds, loads, exports every entry
point include/flof_gb300.h declares, and fails cleanly (status code plus
message, no crash) when no device is present."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "flof_gb300.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"FLOF_API\s+[^;(]*?\b(flof_\w+)\s*\(", text, flags=re.S)))


@pytest.fixture(scope="module")
def lib():
    from ofblend_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header(lib):
    from ofblend_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared()


def test_only_flof_symbols_are_exported():
    out = os.popen(f"nm -D --defined-only {os.path.join(ROOT, 'ofblend_gb300', 'libflof_gb300.so')}").read()
    syms = [ln.split()[-1] for ln in out.splitlines() if " T " in ln]
    assert syms and all(s.startswith("flof_") for s in syms), [s for s in syms if not s.startswith("flof_")]


def test_params_match_reference_defaults(lib):
    from ofblend_gb300._lib import OFParams
    p = OFParams()
    lib.flof_of_params_default(ctypes.byref(p))
    # opticalFlowMultiscale4d defaults, source/plugin/optflow4d.cpp:2182-2189
    assert (p.wSmooth, p.wEnergy, p.level, p.postVelBlur) == (0.0, 0.0, 0, 0.0)
    assert np.float32(p.cgAccuracy) == np.float32(1e-4) and p.blurType == 1 and p.cfl == 999.0
    assert (p.orderTime, p.orderSpace, p.resetBndWidth, p.multiStep) == (1, 1, -1.0, 1)
    assert (p.projSizeThresh, p.minGridSize, p.doFinalProject, p.cgMaxIter) == (9999, 10, 0, 1000)
    lib.flof_of_params_flof(ctypes.byref(p))
    # scenes/flof.py:913-915 with ofsd defaults (:371-388)
    assert np.float32(p.wSmooth) == np.float32(0.001) and np.float32(p.wEnergy) == np.float32(0.0001)
    assert np.float32(p.cgAccuracy) == np.float32(0.01) and p.postVelBlur == 4.0
    assert (p.multiStep, p.minGridSize, p.doFinalProject) == (3, 20, 1)
    assert np.float32(p.resetBndWidth) == np.float32(0.1)


def test_status_strings(lib):
    assert lib.flof_status_string(0) == b"ok"
    assert lib.flof_status_string(1) == b"invalid argument"
    assert lib.flof_version().startswith(b"flof-gb300")


def test_errors_are_status_codes_not_crashes(lib):
    # NULL arguments are rejected before any device work
    assert lib.flof_ctx_create(0, None) == 1
    assert b"NULL" in lib.flof_last_error()
    assert lib.flof_grid_create(None, None, 1, None) == 1
    assert lib.flof_opticalFlowMultiscale4d(None, None, None, None, None, None, None) == 1
    assert lib.flof_loadAdvectTimeSlice_Finish(None, 3) == 1


def test_no_device_fails_loudly_on_cpu_host(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = lib.flof_ctx_create(0, ctypes.byref(h))
    assert st != 0 and not h.value
    assert len(lib.flof_last_error()) > 0
