"""Parity of the steps either side of the solve against the CPU oracle:
input conditioning of the 4D level sets (repeatFrame4d, extrap4dLsSimple,
scenes/flof.py postProcessPhiData) and the 3D output stage of the hi-res
frames (join, setBound, setBoundNeumann, simpleBlurSpecial,
shiftForwGrid4d).  All of it is integer / float work in the reference's
operation order: results are compared bit for bit."""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import scene, synth

pytestmark = pytest.mark.gpu


def grid4(a):
    return (F.Grid4Vec4 if a.ndim == 5 else F.Grid4Real)(dims=synth_dims(a)).from_numpy(a)


def synth_dims(a):
    t, z, y, x = a.shape[:4]
    return (x, y, z, t)


def grid3(a):
    z, y, x = a.shape
    return F.RealGrid(dims=(x, y, z, 1)).from_numpy(a)


def sdf(dims, data_id=0):
    return synth.sdf4d(synth.scene_for(data_id), dims)


# ---------------------------------------------------------------------------
# input conditioning
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("srct,rng,bnd", [(1.0 / 20, 0.0, 0), (3.4, 2.0, 1), (0.2, 5.0, 0),
                                          (13.7, 1.0, 2)])
def test_repeat_frame_bitexact(gpu, orc, srct, rng, bnd):
    dims = (21, 18, 17, 14)
    a = sdf(dims)
    want = orc.repeatFrame4d(a, srct, rng, bnd)
    g = grid4(a)
    F.repeatFrame4d(g, srct, rng, bnd)
    assert np.array_equal(g.to_numpy(), want)


@pytest.mark.parametrize("distance,inside", [(4, False), (4, True), (9, False), (1, True)])
def test_extrap_ls_simple_bitexact(gpu, orc, distance, inside):
    dims = (23, 19, 18, 16)
    a = sdf(dims) * 0.37  # a narrow band so that the sweeps have work to do
    want = orc.extrap4dLsSimple(a, distance, inside)
    g = grid4(a)
    F.extrap4dLsSimple(g, distance, inside)
    assert np.array_equal(g.to_numpy(), want)


def test_post_process_phi_data_bitexact(gpu, orc):
    """postProcessPhiData in level-set mode (flof.py:491-531) on the GPU against
    the same sequence of oracle calls."""
    dims = (24, 22, 20, 18)
    a = sdf(dims, 1)
    ofsd = scene.flof_ofsd(dims[0])
    ofsd["maxDist"] = 6  # flof uses 40; 6 sweeps leave unreached cells at this size
    load_offset = scene.vec4(0.0, 0.0, 0.0, 1.0)
    g = grid4(a)
    scene.postProcessPhiData(g, False, load_offset, ofsd)

    w = orc.repeatFrame4d(a, load_offset.t + 1.0 / float(ofsd["resBackup"]),
                          ofsd["repeatStartDist"], 0)
    if ofsd["isosurfaceOff"] != 0.0:
        w = orc.addConst(w, ofsd["isosurfaceOff"])
    if ofsd["isosurfaceMult"] != 1.0:
        w = orc.multConst(w, ofsd["isosurfaceMult"])
    w = orc.setBound(w, 0.1, ofsd["autoBrdRes"])
    w = orc.extrap4dLsSimple(w, ofsd["maxDist"], False)
    w = orc.extrap4dLsSimple(w, ofsd["maxDist"], True)
    w = orc.multConst(w, ofsd["lsFactor"])
    assert np.array_equal(g.to_numpy(), w)


# ---------------------------------------------------------------------------
# 3D output stage
# ---------------------------------------------------------------------------
def frame3(shape, seed):
    r = np.random.default_rng(seed)
    z, y, x = shape
    zz, yy, xx = np.meshgrid(np.arange(z), np.arange(y), np.arange(x), indexing="ij")
    d = np.sqrt((xx - x / 2) ** 2 + (yy - y / 3) ** 2 + (zz - z / 2) ** 2) - min(shape) / 4
    return (d + 0.3 * r.standard_normal(shape)).astype(np.float32)


@pytest.mark.parametrize("shape", [(18, 20, 24), (1, 21, 19)])
@pytest.mark.parametrize("it,thresh,bord", [(1, 0.0, 0), (2, 0.0, 3), (1, -999.0, 2), (3, 0.5, 1)])
def test_simple_blur_special_bitexact(gpu, orc, shape, it, thresh, bord):
    a = frame3(shape, 5)
    want = orc.simpleBlurSpecial(a, it, thresh, bord)
    g = grid3(a)
    F.simpleBlurSpecial(g, it, thresh, bord)
    assert np.array_equal(g.to_numpy(), want)


def test_join_and_blend_union_bitexact(gpu, orc):
    """The blend-union of two deformed frames (flof.py:739-751): tmp = join(a, b);
    a = a*w0 + tmp*wu + b*w1."""
    a, b = frame3((16, 18, 20), 1), frame3((16, 18, 20), 2)
    w0, wu, w1 = scene.blendW(0.35, 0.1)
    ga, gb = grid3(a), grid3(b)
    tmp = F.RealGrid(dims=ga.dims).copyFrom(ga)
    tmp.join(gb)
    ga.multConst(w0)
    ga.addScaled(tmp, wu)
    ga.addScaled(gb, w1)
    j = orc.join(a, b)
    # 3D arrays as (1, Z, Y, X) 4D grids for the elementwise oracle ops
    w = orc.multConst(a[None], w0)
    w = orc.addScaled(w, j[None], wu)
    w = orc.addScaled(w, b[None], w1)
    assert np.array_equal(tmp.to_numpy(), j)
    assert np.array_equal(ga.to_numpy(), w[0])


@pytest.mark.parametrize("shape", [(14, 16, 18), (1, 12, 15)])
@pytest.mark.parametrize("w", [0, 2])
def test_grid3_bounds_bitexact(gpu, orc, shape, w):
    a = frame3(shape, 3)
    g = grid3(a)
    g.setBound(0.5, w)
    assert np.array_equal(g.to_numpy(), orc.setBound3(a, 0.5, w))
    g = grid3(a)
    g.setBoundNeumann(w)
    assert np.array_equal(g.to_numpy(), orc.setBoundNeumann3(a, w))


def test_output_stage_frame_bitexact(gpu, orc):
    """Time-SDF merge, level-set border and writeResults smoothing of one frame
    (flof.py:818-839, ofHelpers.py:108-113)."""
    cur, prev2 = frame3((20, 22, 24), 7), frame3((20, 22, 24), 8)
    g, gp = grid3(cur), grid3(prev2)
    scene.timeSdfMerge(g, gp)
    g.setBound(0.5, 3)
    scene.sdfSmooth(g, 2, 4)
    w = orc.join(cur, prev2)
    w = orc.simpleBlurSpecial(w, 1, 0.0, 0)
    w = orc.setBound3(w, 0.5, 3)
    w = orc.simpleBlurSpecial(w, 1, 0.0, 3)
    w = orc.simpleBlurSpecial(w, 1, -999.0, 3)
    assert np.array_equal(g.to_numpy(), w)


@pytest.mark.parametrize("good", [1, 5, 9, 12])
def test_shift_forw_grid(gpu, good):
    dims = (9, 8, 7, 13)
    a = np.random.default_rng(good).standard_normal((13, 7, 8, 9)).astype(np.float32)
    g = grid4(a)
    F.shiftForwGrid4d(g, good)
    want = a.copy()
    shift = 13 - good
    s = 0
    while s < good:  # the reference's block copy (optflow4d.cpp:1603-1615)
        n = good - s if s + shift >= good else shift
        want[s:s + n] = want[s + shift:s + shift + n]
        s += shift
    assert np.array_equal(g.to_numpy(), want)


def test_stage_argument_errors(gpu):
    g = F.Grid4Real(dims=(8, 8, 8, 8))
    with pytest.raises(F.FlofError):
        F.shiftForwGrid4d(g, 8)
    with pytest.raises(F.FlofError):
        F.extrap4dLsSimple(F.Grid4Real(dims=(8, 8, 8, 2)), 4)
    with pytest.raises(F.FlofError):
        F.simpleBlurSpecial(g)  # a 4D grid
