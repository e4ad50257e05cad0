"""Whole solves bit for bit against the oracle with FLOF_OPT_STRICT.

With the context option FLOF_OPT_STRICT the PCG does the reference's
arithmetic operation for operation (double alpha and beta, addScaled's
double multiply and add rounded once to float, dotProd's serial double sum
in row order; optflow4d.cpp:234-329) and the error metric is summed in
calcLsDiffTempl's loop order (:895-927).  Every other stage already
reproduces the reference's per-cell operations, so a whole multiscale solve,
the final projection included, must equal the oracle's bit for bit: velocity
field, error metric, and the iteration count and residual of every solve.
"""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

FLOF = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=0.01, postVelBlur=4, cfl=999, multiStep=3,
            minGridSize=20, resetBndWidth=0.1)


@pytest.fixture(scope="module")
def sctx(gpu):
    ctx = F.Context(0)
    ctx.set_option(_lib.FLOF_OPT_STRICT, 1)
    yield ctx
    ctx.close()


def _grid(arr, ctx):
    arr = np.ascontiguousarray(arr, np.float32)
    if arr.ndim == 5:
        T, Z, Y, X, _ = arr.shape
        return F.Grid4Vec4(dims=(X, Y, Z, T), ctx=ctx).from_numpy(arr)
    T, Z, Y, X = arr.shape
    return F.Grid4Real(dims=(X, Y, Z, T), ctx=ctx).from_numpy(arr)


def _same_solves(got, want):
    """Per-solve (size, iterations, residual) of the GPU and the oracle."""
    g = [(s[0], s[1], np.float32(s[2])) for s in got]
    w = [(s[0], s[1], np.float32(s[2])) for s in want]
    return g == w, g, w


def test_strict_ls_diff_bitexact(sctx, orc):
    dims = (32, 30, 28, 24)
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    for bnd in (0, 4):
        want = np.float32(orc.calcLsDiff4d(i0, i1, 0.1 / 20, bnd))
        got = np.float32(F.calcLsDiff4d(_grid(i0, sctx), _grid(i1, sctx), None, 0.1 / 20, bnd))
        assert got == want, (bnd, got, want)


def test_strict_single_level_solve_bitexact(sctx, orc):
    dims = (24, 22, 20, 18)
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    want, wit, wres = orc.opticalFlow4d(zv, i0, i1, wSmooth=0.001, wEnergy=0.0001, postVelBlur=4.0,
                                        cgAccuracy=1e-4, resetBndWidth=0.1)
    gv = _grid(zv, sctx)
    it, res = F.opticalFlow4d(gv, _grid(i0, sctx), _grid(i1, sctx), wSmooth=0.001, wEnergy=0.0001,
                              postVelBlur=4.0, cgAccuracy=1e-4, resetBndWidth=0.1)
    assert (it, np.float32(res)) == (wit, np.float32(wres))
    assert np.array_equal(gv.to_numpy(), want)


@pytest.mark.parametrize("project", [False, True])
def test_strict_multiscale_c1_bitexact(sctx, orc, project):
    """The 32^4 one-way workload with flof.py's parameters (flof.py:913-915),
    with and without the final projection."""
    dims = (32, 32, 32, 32)
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    kw = dict(FLOF, doFinalProject=project)
    want, werr, wst = orc.opticalFlowMultiscale4d(zv, i0, i1, **kw)
    gv = _grid(zv, sctx)
    err = F.opticalFlowMultiscale4d(gv, _grid(i0, sctx), _grid(i1, sctx), **kw)
    st = F.last_solve_stats()["solves"]
    same, g, w = _same_solves(st, wst)
    assert same, (g, w)
    got = gv.to_numpy()
    diff = int(np.count_nonzero(got != want))
    assert diff == 0, f"{diff} of {got.size} velocity entries differ"
    assert np.float32(err) == np.float32(werr)
    # and the deformed SDF at alpha = 0.5 with it
    sdf0 = i0 / synth.LS_FACTOR
    a = orc.advect4d(want, sdf0, 0.5)
    gs = _grid(sdf0, sctx)
    F.advect4d(gv, gs, 0.5)
    assert np.array_equal(gs.to_numpy(), a)
