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


def test_fresh_workers_many_streams(gpu):
    """Sixteen fresh worker contexts build their blur tables during the first
    solves while the others already run.  The tables must be on the device
    before the first blur reads them: every result equals the single call's."""
    P = dict(FLOF, cgAccuracy=1e-4, multiStep=3, doFinalProject=True)
    dims = (24, 24, 24, 16)
    ps = []
    for k in range(32):
        s0, s1 = synth.random_pair_scenes(5000 + k)
        ps.append((dims, synth.flow_input(s0, dims), synth.flow_input(s1, dims)))
    ref_ctx = F.Context(0)
    vs, a, b = grids(ref_ctx, ps)
    single = []
    for v, x, y in zip(vs, a, b):
        F.opticalFlowMultiscale4d(v, x, y, **P)
        single.append(v.to_numpy())
    ref_ctx.close()
    for rep in range(3):
        ctx = F.Context(0)  # new context: new workers, empty table caches
        vs, a, b = grids(ctx, ps)
        F.opticalFlowMultiscale4d_batch(vs, a, b, workers=16, **P)
        for q in range(len(ps)):
            assert np.array_equal(vs[q].to_numpy(), single[q]), (rep, q)
        ctx.close()


def test_batch_with_warm_start_equals_single_calls(gpu):
    """With a model attached, warm-started batch solves give the single
    calls' results (they run in turn on the calling context)."""
    ctx = F.Context(0)
    m = F.Model(16, ctx=ctx, seed=11)
    m.attach()
    dims = (32, 32, 32, 32)  # coarsest level 16^4: the model's grid
    ps = []
    for k in range(3):
        s0, s1 = synth.random_pair_scenes(7000 + k)
        ps.append((dims, synth.flow_input(s0, dims), synth.flow_input(s1, dims)))
    vs, a, b = grids(ctx, ps)
    single = []
    flags = []
    for v, x, y in zip(vs, a, b):
        F.opticalFlowMultiscale4d(v, x, y, warmStart=True, **FLOF)
        single.append(v.to_numpy())
        flags.append(F.last_solve_stats()["warm_start"])
        v.setConst(0.0)
    assert all(f in (0, 1) for f in flags)  # the prediction was tried
    F.opticalFlowMultiscale4d_batch(vs, a, b, workers=4, warmStart=True, **FLOF)
    for q in range(len(ps)):
        assert np.array_equal(vs[q].to_numpy(), single[q]), q
    m.detach()
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


# ---------------------------------------------------------------------------
# mixed precision (BF16 gradient, FP64 residuals, iterative refinement)
# ---------------------------------------------------------------------------
def test_mixed_precision_against_fp64_oracle(gpu):
    """The mixed solve's deformation against the FP64 oracle (the reference's
    double build restated), next to the FP32 solve's; both must stay within
    the deformation tolerance of each other's order, and the recorded true
    residual of the FP32 system must be small."""
    import oracle
    o64 = oracle.get(double=True)
    dims = (32, 32, 32, 32)
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    kw = dict(FLOF, cgAccuracy=1e-4, multiStep=1, doFinalProject=False)
    zv = np.zeros(i0.shape + (4,), np.float64)
    want = o64.opticalFlowMultiscale4d(zv, i0.astype(np.float64), i1.astype(np.float64),
                                       **{k: v for k, v in kw.items() if k != "blurType"})[0]
    out = {}
    for prec in ("fp32", "mixed"):
        v = F.Grid4Vec4(dims=dims)
        F.opticalFlowMultiscale4d(v, F.Grid4Real(dims=dims).from_numpy(i0),
                                  F.Grid4Real(dims=dims).from_numpy(i1), precision=prec, **kw)
        out[prec] = (v.to_numpy().astype(np.float64), F.last_solve_stats())
    rel = {p: np.linalg.norm(out[p][0] - want) / np.linalg.norm(want) for p in out}
    print("rel L2 vs FP64 oracle:", rel, "true residual (mixed):", out["mixed"][1]["true_residual"],
          "iterations:", {p: out[p][1]["cg_total_iterations"] for p in out})
    assert rel["fp32"] < 1e-4, rel
    assert rel["mixed"] < 1e-3, rel
    tr = [t for t in out["mixed"][1]["true_residual"] if t >= 0]
    assert tr and max(tr) < 1e-2, out["mixed"][1]
    assert all(t < 0 for t in out["fp32"][1]["true_residual"])
