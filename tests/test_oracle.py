"""The CPU oracle against the reference's own known answers and properties.

Known answers come from the reference's tests:
  tools/tests/test_0032_grid4dop.py  Grid4d arithmetic, closed-form values
  tools/tests/test_0042_interpol4d.py interpolateGrid4d up/down chain
The rest checks properties the reference's algorithm guarantees (PCG
convergence, float/double agreement without the projection step) and that
the oracle still reproduces the committed golden fixtures bit for bit.
"""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "flof_golden.npz")


# ---------------------------------------------------------------------------
# tools/tests/test_0032_grid4dop.py
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("double", [False, True])
def test_grid4dop_known_answers(double):
    import oracle
    o = oracle.get(double)
    shape = (12, 30, 20, 10)  # gs = (10, 20, 30), fourthDim = 12
    z = np.zeros(shape, o.dtype)
    zv = np.zeros(shape + (4,), o.dtype)
    # Real
    rlg1 = o.addConst(o.setConst(z, 1.0), 0.1)
    rlg2 = o.multConst(o.setConst(z, 2.4), 0.5)
    rlg3 = o.addScaled(o.add(rlg1.copy(), rlg2), rlg2, 0.5)
    thr = 1e-14 if double else 1e-07  # threshold / thresholdStrict of the test
    for g, want in ((rlg1, 1.1), (rlg2, 1.2), (rlg3, 2.9)):
        assert np.abs(g.astype(np.float64) - o.dtype(want)).max() <= thr
    # Vec4
    fdg1 = o.addConst(o.setConst(zv, 1.0), 0.2)
    fdg2 = o.multConst(o.setConst(zv, 1.0), 0.5)
    fdg3 = o.addScaled(o.add(fdg1.copy(), fdg2), fdg2, 0.5)
    thr = 1e-14 if double else 5e-07
    for g, want in ((fdg1, 1.2), (fdg2, 0.5), (fdg3, 1.95)):
        # grid4dMaxDiffVec4 sums |diff| over the four components
        assert np.abs(g.astype(np.float64) - o.dtype(want)).sum(axis=-1).max() <= thr
    if not double:
        # getMaxAbsValue values quoted in the test's comments
        assert repr(o.getMaxAbs(fdg1)) == "2.4000000953674316"
        assert o.getMaxAbs(fdg2) == 1.0
        assert repr(o.getMaxAbs(fdg3)) == "3.9000000953674316"


# ---------------------------------------------------------------------------
# tools/tests/test_0042_interpol4d.py (resolution 20 instead of 40)
# ---------------------------------------------------------------------------
def test_interpol4d_chain(orc):
    res, up = 20, 2
    sm, nm, xl = res // up, res, res * up
    rs, re = sm * 0.3, sm * 0.7
    box = np.zeros((sm,) * 4, np.float32)
    idx = np.arange(sm)
    inside = (idx >= rs) & (idx <= re)  # knSetRegion4d keeps start <= p <= end
    box[np.ix_(inside, inside, inside, inside)] = 1.0
    dens = orc.interpolateGrid4d((nm,) * 4, box)
    xld = orc.interpolateGrid4d((xl,) * 4, dens)
    dens2 = orc.interpolateGrid4d((nm,) * 4, xld)
    sm2 = orc.interpolateGrid4d((sm,) * 4, dens2)
    for g in (dens, xld, dens2, sm2):
        assert g.min() >= 0.0 and g.max() <= 1.0
    # the core of the box survives the round trip exactly, far cells stay 0
    c = slice(int(rs) + 2, int(re) - 1)
    assert np.all(sm2[c, c, c, c] == 1.0)
    assert sm2[0, 0, 0, 0] == 0.0 and sm2[-1, -1, -1, -1] == 0.0
    # up- then down-sampling by 2 keeps every cell whose 3^4 neighbourhood
    # is constant
    import itertools
    core = np.ones_like(dens, dtype=bool)
    for off in itertools.product((-1, 0, 1), repeat=4):
        core &= np.roll(dens, off, axis=(0, 1, 2, 3)) == dens
    core[[0, -1], :, :, :] = core[:, [0, -1], :, :] = False
    core[:, :, [0, -1], :] = core[:, :, :, [0, -1]] = False
    assert core.sum() > 0 and np.array_equal(dens2[core], dens[core])
    # Vec4 path equals the Real path per component
    boxv = np.repeat(box[..., None], 4, axis=-1)
    densv = orc.interpolateGrid4d((nm,) * 4, boxv)
    assert np.array_equal(densv[..., 2], dens)


def test_grid_factor(orc):
    fac, off = orc.gridFactor4d((64, 64, 64, 64), (128, 128, 128, 64), (-1,) * 4, (1, 1, 1, 1), (0, 0, 0, 0))
    assert np.allclose(fac, [0.5, 0.5, 0.5, 1.0]) and np.allclose(off, [0.25, 0.25, 0.25, 0.5])
    fac, off = orc.gridFactor4d((40, 40, 40, 60), (32, 32, 32, 48), (-1,) * 4, (0.8,) * 4, (4, 4, 4, 6))
    assert np.allclose(fac, np.float32(40 / 32) / np.float32(0.8))
    assert np.allclose(off, -np.array([4, 4, 4, 6]) * fac + fac * 0.5)


def test_interp4_clamp_semantics(orc):
    g = np.arange(4 * 5 * 6 * 7, dtype=np.float32).reshape(7, 6, 5, 4)
    # cell centres return the cell value exactly
    assert orc.interp4(g, (2.5, 3.5, 1.5, 4.5)) == g[4, 1, 3, 2]
    # below the first centre: clamped to index 0 with weight 1
    assert orc.interp4(g, (-3.0, 0.5, 0.5, 0.5)) == g[0, 0, 0, 0]
    # beyond the last centre: clamped to size-2 with the high weight
    assert orc.interp4(g, (99.0, 0.5, 0.5, 0.5)) == g[0, 0, 0, 3]
    # midpoint between two x cells
    assert orc.interp4(g, (1.0, 0.5, 0.5, 0.5)) == np.float32(0.5) * (g[0, 0, 0, 0] + g[0, 0, 0, 1])


# ---------------------------------------------------------------------------
# algorithmic properties
# ---------------------------------------------------------------------------
def _drop_pair(dims, a=0, b=1):
    from ofblend_gb300 import synth
    return synth.flow_input(synth.scene_for(a), dims), synth.flow_input(synth.scene_for(b), dims)


def test_pcg_meets_its_stop_rule(orc):
    dims = (12, 12, 12, 12)
    i0, i1 = _drop_pair(dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    x, it, res, ok = orc.cgSolve(zv, i0, i1, 0.001, 0.0001, 1e-4)
    assert ok and it > 0 and res <= 1e-4
    rhs, blockd, offd = orc.ofAssemble(zv, i0, i1, 0.001, 0.0001)
    # recompute r = b - A x in double from the assembled matrix
    n = rhs.size
    X, Y, Z, T = dims
    B = blockd.reshape(-1, 4, 4).astype(np.float64)
    xc = x.reshape(-1, 4).astype(np.float64)
    ax = np.einsum("cdm,cm->cd", B, xc).reshape(-1)
    g = x.reshape(T, Z, Y, X, 4).astype(np.float64)
    nb = np.zeros_like(g)
    for axis in range(4):
        nb += np.roll(g, 1, axis=3 - axis) + np.roll(g, -1, axis=3 - axis)
    ax += offd.astype(np.float64) * nb.reshape(-1)
    r = rhs.astype(np.float64) - ax
    assert r.max() <= 1.01e-4 * rhs.max()
    assert n == 4 * X * Y * Z * T


def test_float_and_double_oracles_agree_without_projection(orc, orc64):
    dims = (16, 16, 16, 16)
    i0, i1 = _drop_pair(dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    kw = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=0.01, postVelBlur=4, cfl=999, multiStep=3,
              minGridSize=6, doFinalProject=False, resetBndWidth=0.1)
    v32, e32, _ = orc.opticalFlowMultiscale4d(zv, i0, i1, **kw)
    v64, e64, _ = orc64.opticalFlowMultiscale4d(zv.astype(np.float64), i0.astype(np.float64),
                                                i1.astype(np.float64), **kw)
    rel = np.linalg.norm(v32 - v64) / np.linalg.norm(v64)
    assert rel < 1e-4
    assert abs(e32 - e64) <= 1e-3 * abs(e64)


def test_multistep_stop_rule_and_early_exit(orc):
    g = np.load(GOLDEN)
    it = g["ms_iters"]
    # coarsest level: tiny residual exits before the first iteration
    assert it[0] == 0
    # at most three multistep solves per level
    assert len(it) <= 9


# ---------------------------------------------------------------------------
# golden fixtures (tests/golden/gen_golden.py)
# ---------------------------------------------------------------------------
def test_oracle_reproduces_golden(orc):
    g = np.load(GOLDEN)
    assert np.array_equal(orc.advect4d(g["adv_vel"], g["adv_src"], 0.7), g["adv_out_a07"])
    assert np.array_equal(orc.advect4d(g["adv_vel"], g["adv_srcv"], 1.0), g["adv_outv_a1"])
    assert np.array_equal(orc.interpolateGrid4d((13, 11, 10, 7), g["ip_src"], offset=(1.0, 0.5, 0.0, 2.0),
                                                scale=(0.8, 0.8, 0.8, 1.0)), g["ip_up"])
    assert np.array_equal(orc.interpolGrid((4, 4, 3, 3), g["adv_srcv"]), g["ip_down_v"])
    assert np.array_equal(orc.gaussianBlur4d(g["blur_in"], 2.0), g["blur_s2"])
    assert np.array_equal(orc.gaussianBlur4d(g["blur_in"], 1.125), g["blur_s1125"])
    assert np.float32(orc.calcLsDiff4d(g["ls_a"], g["ls_b"], 0.1 / 20, 2)) == g["ls_val"]
    zv = np.zeros(g["of_i0"].shape + (4,), np.float32)
    v, it, res = orc.opticalFlow4d(zv, g["of_i0"], g["of_i1"], 0.001, 0.0001, 4.0, 1e-4, 0.1)
    assert it == g["of_iters"] and np.array_equal(v, g["of_vel"])
    zv = np.zeros(g["ms_i0"].shape + (4,), np.float32)
    v, err, st = orc.opticalFlowMultiscale4d(zv, g["ms_i0"], g["ms_i1"], wSmooth=0.001, wEnergy=0.0001,
                                             cgAccuracy=0.01, postVelBlur=4, cfl=999, multiStep=3,
                                             minGridSize=5, doFinalProject=True, resetBndWidth=0.1)
    assert np.array_equal(v, g["ms_vel"]) and np.float32(err) == g["ms_err"]
    dst = np.full((23, 22, 24), 7.0, np.float32)
    out = orc.optRunFrame(g["lk_defo"], dst, g["lk_phi"], time=2.5, blendAlpha=0.25,
                          defoFactor=(4.0, 4.0, 4.0, 1.0), overrideSize=(24, 22, 23, 5), bordSkip=2)
    assert np.array_equal(out, g["lk_out"])
