"""Batched solves of uneven sizes and the PCG autotuner.  A batch must give,
solve by solve, exactly what the single call gives on the same grids; tuned
launch shapes change only the grouping of the dot-product partial sums."""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

FLOF = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=0.01, postVelBlur=4, cfl=999, multiStep=2,
            minGridSize=20, resetBndWidth=0.1)
DIMS = [(24, 24, 24, 16), (20, 22, 18, 16), (28, 24, 20, 18), (16, 16, 16, 12), (24, 20, 22, 14),
        (32, 32, 32, 16)]


def pairs():
    out = []
    for k, dims in enumerate(DIMS):
        s0, s1 = synth.random_pair_scenes(500 + k)
        out.append((dims, synth.flow_input(s0, dims), synth.flow_input(s1, dims)))
    return out


def grids(ctx, ps):
    vs, a, b = [], [], []
    for dims, i0, i1 in ps:
        vs.append(F.Grid4Vec4(dims=dims, ctx=ctx))
        a.append(F.Grid4Real(dims=dims, ctx=ctx).from_numpy(i0))
        b.append(F.Grid4Real(dims=dims, ctx=ctx).from_numpy(i1))
    return vs, a, b


def test_batch_equals_single_calls(gpu):
    ps = pairs()
    ctx = F.Context(0)
    vs, a, b = grids(ctx, ps)
    single_err = [F.opticalFlowMultiscale4d(v, x, y, **FLOF) for v, x, y in zip(vs, a, b)]
    single = [v.to_numpy() for v in vs]
    for v in vs:
        v.setConst(0.0)
    errs = F.opticalFlowMultiscale4d_batch(vs, a, b, workers=3, **FLOF)
    for q in range(len(ps)):
        assert np.array_equal(vs[q].to_numpy(), single[q]), q
        assert errs[q] == single_err[q]
    # automatic worker count, a second time on the cached workers
    for v in vs:
        v.setConst(0.0)
    errs2 = F.opticalFlowMultiscale4d_batch(vs, a, b, **FLOF)
    assert errs2 == errs
    ctx.close()


def test_autotuned_solves_agree(gpu):
    ps = pairs()[:3]
    ctx = F.Context(0)
    vs, a, b = grids(ctx, ps)
    base = []
    for v, x, y in zip(vs, a, b):
        F.opticalFlowMultiscale4d(v, x, y, **dict(FLOF, doFinalProject=False))
        base.append(v.to_numpy())
        v.setConst(0.0)
    ctx.set_option(_lib.FLOF_OPT_AUTOTUNE, 1)
    F.opticalFlowMultiscale4d_batch(vs, a, b, workers=2, **dict(FLOF, doFinalProject=False))
    for q, v in enumerate(vs):
        got = v.to_numpy()
        rel = np.linalg.norm(got - base[q]) / np.linalg.norm(base[q])
        assert rel < 1e-4, (q, rel)
    ctx.close()


def test_batch_errors(gpu):
    ctx = F.Context(0)
    v = F.Grid4Vec4(dims=(8, 8, 8, 8), ctx=ctx)
    a = F.Grid4Real(dims=(8, 8, 8, 9), ctx=ctx)
    with pytest.raises(F.FlofError):
        F.opticalFlowMultiscale4d_batch([v], [a], [a], **FLOF)
    assert F.opticalFlowMultiscale4d_batch([], [], [], **FLOF) == []
    ctx.close()


def test_grids_outliving_their_context(gpu):
    """Destroying a context frees its grids' storage; the handles stay safe to
    drop and are rejected by every call."""
    ctx = F.Context(0)
    g = F.Grid4Real(dims=(8, 8, 8, 8), ctx=ctx)
    h = F.Grid4Real(dims=(8, 8, 8, 8), ctx=ctx)
    ctx.close()
    with pytest.raises(F.FlofError):
        g.setConst(1.0)
    del g, h
    ctx2 = F.Context(0)  # no error left behind by the teardown
    F.Grid4Real(dims=(8, 8, 8, 8), ctx=ctx2).setConst(2.0)
    ctx2.close()
