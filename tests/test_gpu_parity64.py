"""Parity at the benchmark's own configuration: 64^4 float32 with flof.py's
parameters (flof.py:913-915) at cgAccuracy 1e-4, the two-way mode-2 apply
on the 64^4 grid and mode-3 frames of a 128^3 x 64 hi-res series.

* The deformation 0 -> 1 without the final projection is compared with the
  oracle's within the tolerances of the parallel PCG: 1e-4 relative L2 for
  the field, 1e-3 cells max-abs for the SDF deformed at alpha = 0.5.
* The per-cell stages after the solve are compared bit for bit on the GPU's
  own deformations of the benchmark (both directions, projection on): the
  oracle applies them with deform4d (flof.py:591-637) and with
  loadAdvectTimeSlice_OptRun (optflow4d.cpp:1951-2105) plus the two-way
  blend (flof.py:750-755).
"""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import synth

pytestmark = pytest.mark.gpu

R, H = 64, 128
FLOF = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=1e-4, postVelBlur=4, cfl=999, multiStep=3,
            minGridSize=20, resetBndWidth=0.1)
REL_L2_DEFO = 1e-4
SDF_CELLS = 1e-3
ALPHAS = (0.25, 0.5, 0.75)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def inputs():
    dims = (R,) * 4
    s0, s1 = synth.scene_for(0), synth.scene_for(1)
    return {"dims": dims, "s0": s0, "s1": s1,
            "i0": synth.flow_input(s0, dims), "i1": synth.flow_input(s1, dims)}


def test_deformation_64_matches_oracle(gpu, orc, inputs):
    i0, i1, dims = inputs["i0"], inputs["i1"], inputs["dims"]
    kw = dict(FLOF, doFinalProject=False)
    zv = np.zeros(i0.shape + (4,), np.float32)
    want, werr, wst = orc.opticalFlowMultiscale4d(zv, i0, i1, **kw)
    gv = F.Grid4Vec4(dims=dims)
    err = F.opticalFlowMultiscale4d(gv, F.Grid4Real(dims=dims).from_numpy(i0),
                                    F.Grid4Real(dims=dims).from_numpy(i1), **kw)
    st = F.last_solve_stats()["solves"]
    got = gv.to_numpy()
    assert [s[0] for s in st] == [s[0] for s in wst]
    rl = rel_l2(got, want)
    sdf0 = i0 / synth.LS_FACTOR
    cells = float(np.abs(orc.advect4d(want, sdf0, 0.5) - orc.advect4d(got, sdf0, 0.5)).max())
    print(f"64^4 deformation vs oracle: rel L2 {rl:.3e}, deformed SDF max-abs {cells:.3e} cells, "
          f"error metric {err:.6f} vs {werr:.6f}, iterations {[s[1] for s in st]} vs "
          f"{[s[1] for s in wst]}")
    assert rl < REL_L2_DEFO
    assert cells <= SDF_CELLS
    assert abs(err - werr) <= 1e-3 * abs(werr)


@pytest.fixture(scope="module")
def bench_fields(gpu, inputs):
    """Both deformations exactly as the benchmark computes them."""
    dims = inputs["dims"]
    g0 = F.Grid4Real(dims=dims).from_numpy(inputs["i0"])
    g1 = F.Grid4Real(dims=dims).from_numpy(inputs["i1"])
    out = {}
    for key, (x, y) in (("01", (g0, g1)), ("10", (g1, g0))):
        v = F.Grid4Vec4(dims=dims)
        F.opticalFlowMultiscale4d(v, x, y, **FLOF, doFinalProject=True)
        out[key] = v
    return out


def test_deform4d_64_bitexact_on_gpu_deformations(orc, inputs, bench_fields):
    dims = inputs["dims"]
    a0, a1 = synth.sdf4d(inputs["s0"], dims), synth.sdf4d(inputs["s1"], dims)
    v01, v10 = bench_fields["01"].to_numpy(), bench_fields["10"].to_numpy()
    gs0, gs1 = F.Grid4Real(dims=dims).from_numpy(a0), F.Grid4Real(dims=dims).from_numpy(a1)
    out = F.Grid4Real(dims=dims)
    for alpha in ALPHAS:
        F.deform4d(out, gs0, gs1, bench_fields["01"], bench_fields["10"], alpha=alpha, twoway=1)
        want = orc.deform4d(v01, v10, a0, a1, np.float32(alpha), twoway=1)
        assert np.array_equal(out.to_numpy(), want), alpha


def test_hires_frames_bitexact_on_gpu_deformations(orc, inputs, bench_fields):
    hd = (H, H, H, R)
    h0, h1 = synth.sdf4d(inputs["s0"], hd), synth.sdf4d(inputs["s1"], hd)
    gh0, gh1 = F.Grid4Real(dims=hd).from_numpy(h0), F.Grid4Real(dims=hd).from_numpy(h1)
    v01, v10 = bench_fields["01"].to_numpy(), bench_fields["10"].to_numpy()
    factor = (H / R, H / R, H / R, 1.0)
    bord = int(H * 0.1)
    kw = dict(loadTimeScale=1.0, defoOffset=(0, 0, 0, 0), defoScale=(1, 1, 1, 1), defoFactor=factor,
              overrideSize=hd, overrideTimeOff=0.0, bordSkip=bord)
    dst = F.RealGrid(dims=(H, H, H, 1))
    box = (slice(bord, H - bord),) * 3
    F.loadAdvectTimeSlice_OptInit(1, bench_fields["01"])
    F.loadAdvectTimeSlice_OptInit(2, bench_fields["10"])
    try:
        for t, alpha in ((5, 0.25), (31, 0.5), (58, 0.75)):
            time = t + 0.5
            ai = np.float32(1.0 - alpha)
            d0 = orc.optRunFrame(v01, np.zeros((H, H, H), np.float32), h0, time=time, blendAlpha=alpha, **kw)
            d1 = orc.optRunFrame(v10, np.zeros((H, H, H), np.float32), h1, time=time, blendAlpha=ai, **kw)
            want = orc.addScaled(orc.multConst(d0[None], ai), d1[None], np.float32(alpha))[0]
            F.loadAdvectTimeSlice_OptRunTwoway(1, 2, dst, gh0, gh1, time, alpha, 1.0, (0, 0, 0, 0),
                                               (1, 1, 1, 1), factor, overrideSize=hd,
                                               overrideTimeOff=0.0, bordSkip=bord)
            got = dst.to_numpy().reshape(H, H, H)
            assert np.array_equal(got[box], want[box]), (t, alpha)
    finally:
        F.loadAdvectTimeSlice_Finish(1)
        F.loadAdvectTimeSlice_Finish(2)
