"""The multigrid-preconditioned solve (solver="mg") of the learned solve
mode against the plain Jacobi-PCG.

Both stop on the reference's rule on the same residual (signed max of r at
most cgAccuracy times that of b, optflow4d.cpp:284-315).  At cgAccuracy 1e-4
the plain result itself is only about 1e-3 (relative L2) from the converged
deformation, so the preconditioned result is judged against a tightly
converged plain solve (cgAccuracy 1e-7), with the plain 1e-4 solve's own
distance from it as the bar.
"""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

FLOF = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=1e-4, postVelBlur=4, cfl=999, multiStep=3,
            minGridSize=20, resetBndWidth=0.1)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(gpu):
    dims = (48, 48, 48, 32)
    g0 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(synth.scene_for(0), dims))
    g1 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(synth.scene_for(1), dims))
    return dims, g0, g1


def _solve(case, **kw):
    dims, g0, g1 = case
    v = F.Grid4Vec4(dims=dims)
    err = F.opticalFlowMultiscale4d(v, g0, g1, **kw)
    return v.to_numpy(), err, F.last_solve_stats()["solves"]


def test_mg_fewer_iterations_same_accuracy(case):
    kw = dict(FLOF, doFinalProject=False)
    plain, _, sp = _solve(case, **kw)
    mg, _, sm = _solve(case, solver="mg", **kw)
    tight, _, _ = _solve(case, **dict(kw, cgAccuracy=1e-7))
    # the same solves (levels, multisteps), each converged by the same rule
    assert [s[0] for s in sm] == [s[0] for s in sp]
    assert all(s[3] == 1 and s[2] <= 1e-4 for s in sm), sm
    it_p = sum(s[1] for s in sp if s[0] == 48)
    it_m = sum(s[1] for s in sm if s[0] == 48)
    e_p, e_m = rel_l2(plain, tight), rel_l2(mg, tight)
    print(f"finest-level iterations plain {it_p}, mg {it_m}; rel L2 to the converged solve: "
          f"plain {e_p:.2e}, mg {e_m:.2e}")
    assert it_m * 4 <= it_p
    assert e_m <= 1.5 * e_p


def test_mg_with_projection_converges(case):
    mg, err, sm = _solve(case, solver="mg", **dict(FLOF, doFinalProject=True))
    _, perr, _ = _solve(case, **dict(FLOF, doFinalProject=True))
    assert all(s[3] == 1 for s in sm), sm
    assert np.isfinite(mg).all()
    assert abs(err - perr) <= 0.02 * perr, (err, perr)


def test_mg_repeats_bitwise(case):
    kw = dict(FLOF, doFinalProject=True, solver="mg")
    a, ea, _ = _solve(case, **kw)
    b, eb, _ = _solve(case, **kw)
    assert ea == eb and np.array_equal(a, b)


def test_plain_pcg_finishes_when_mg_stops_early(case):
    """An iteration cap of 2 stops the preconditioned solve before the
    threshold; the plain operator's residual check sees it and the plain
    Jacobi-PCG finishes each solve to the same threshold."""
    ctx = F.context()
    f0 = ctx.mg_fallbacks()
    kw = dict(FLOF, doFinalProject=False)
    tight, _, _ = _solve(case, **dict(kw, cgAccuracy=1e-7))
    plain, _, _ = _solve(case, **kw)
    try:
        ctx.set_mg_params(max_iter=2)
        mg, _, sm = _solve(case, solver="mg", **kw)
    finally:
        ctx.set_mg_params()
    assert ctx.mg_fallbacks() - f0 == len(sm)
    assert all(s[3] == 1 and s[2] <= 1e-4 for s in sm), sm
    assert rel_l2(mg, tight) <= 1.5 * rel_l2(plain, tight)


def test_separable_stencils_match_direct(case):
    """blurType 2 (separable blur and extrapolation box sums) against the
    direct stencils, on the plain and on the preconditioned solve: equal up
    to rounding, which the projection does not amplify here."""
    kw = dict(FLOF, doFinalProject=True)
    for solver in ("pcg", "mg"):
        a, ea, _ = _solve(case, solver=solver, **kw)
        b, eb, _ = _solve(case, solver=solver, blurType=2, **kw)
        print(f"{solver}: blurType 2 vs 1 rel L2 {rel_l2(b, a):.2e}, error metric {eb} vs {ea}")
        assert rel_l2(b, a) < 1e-4
        assert abs(eb - ea) <= 1e-3 * ea


def test_slab_tma_kernels_match_plain_loads(case):
    """The TMA slab kernels (the Vec4 blur and the extrapolation sweeps
    walking t, direct and separable) and their plain-load counterparts take
    the same sums in the same order: whole solves with the final projection
    agree bit for bit, on an x extent that leaves a partial tile."""
    kw = dict(FLOF, doFinalProject=True)
    ctx = F.context()
    for blur in (1, 2):
        a, ea, _ = _solve(case, blurType=blur, **kw)
        ctx.set_option(_lib.FLOF_OPT_SLAB_TMA, 0)
        try:
            b, eb, _ = _solve(case, blurType=blur, **kw)
        finally:
            ctx.set_option(_lib.FLOF_OPT_SLAB_TMA, 1)
        assert np.array_equal(a, b) and ea == eb, (blur, rel_l2(b, a), ea, eb)


def test_slab_tma_kernels_match_plain_loads_odd_extents(gpu):
    """The same on extents that leave partial tiles on every axis: x and y
    tiles, a last z group of one plane, a last keep-mask word of three t
    planes and a partial t walk."""
    dims = (37, 45, 29, 23)
    g0 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(synth.scene_for(0), dims))
    g1 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(synth.scene_for(1), dims))
    kw = dict(FLOF, doFinalProject=True, multiStep=1, minGridSize=100)
    ctx = F.context()
    for blur in (1, 2):
        out = []
        for tma in (1, 0):
            ctx.set_option(_lib.FLOF_OPT_SLAB_TMA, tma)
            try:
                v = F.Grid4Vec4(dims=dims)
                e = F.opticalFlowMultiscale4d(v, g0, g1, blurType=blur, **kw)
                out.append((v.to_numpy(), e))
            finally:
                ctx.set_option(_lib.FLOF_OPT_SLAB_TMA, 1)
        (a, ea), (b, eb) = out
        assert np.array_equal(a, b) and ea == eb, (blur, rel_l2(b, a), ea, eb)


def test_mg_params_are_checked(gpu):
    ctx = F.context()
    with pytest.raises(F.FlofError):
        ctx.set_mg_params(omega0=0.0)
    with pytest.raises(F.FlofError):
        ctx.set_mg_params(lam=1.5)
    with pytest.raises(F.FlofError):
        ctx.set_mg_params(coarse_sweeps=0)
    with pytest.raises(F.FlofError):
        F.opticalFlowMultiscale4d(F.Grid4Vec4(dims=(8,) * 4), F.Grid4Real(dims=(8,) * 4),
                                  F.Grid4Real(dims=(8,) * 4), solver="nope")
