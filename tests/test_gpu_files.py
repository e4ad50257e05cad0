"""GPU tests of the file-facing parts of the path: .uni grid files
(fileio.cpp:834-1000) against an independent writer/reader of the layout,
the hi-res 4D assembly loadPlaceGrid4d (optflow4d.cpp:1460-1594) and the
non-optimised loadAdvectTimeSlice (:1671-1760) against the oracle, and
OptInit from a deformation file."""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import synth
import unifmt

pytestmark = pytest.mark.gpu


def dims_of(a):
    t, z, y, x = a.shape[:4]
    return (x, y, z, t)


def rnd(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape).astype(np.float32)


# ---------------------------------------------------------------------------
# .uni files
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("kind", ["real4", "vec4", "real3"])
def test_uni_roundtrip(gpu, tmp_path, kind):
    if kind == "real4":
        a, g = rnd((5, 6, 7, 9), 1), F.Grid4Real(dims=(9, 7, 6, 5))
    elif kind == "vec4":
        a, g = rnd((4, 6, 7, 9, 4), 2), F.Grid4Vec4(dims=(9, 7, 6, 4))
    else:
        a, g = rnd((6, 7, 9), 3), F.RealGrid(dims=(9, 7, 6, 1))
    g.from_numpy(a)
    p = str(tmp_path / "g.uni")
    g.save(p)
    r = unifmt.read(p)
    assert r["tag"] == (b"MNT2" if kind == "real3" else b"M4T2")
    assert r["dims"][:3] == g.dims[:3]
    assert r["bytesPerElement"] == (16 if kind == "vec4" else 4)
    assert np.array_equal(r["data"], a)
    # a file written by the independent writer loads bit for bit
    b = a * 2 + 1
    p2 = str(tmp_path / "h.uni")
    unifmt.write(p2, b, is4d=(kind != "real3"), grid_type=(17 if kind == "real3" else None))
    g.load(p2)
    assert np.array_equal(g.to_numpy(), b)


def test_uni_read_slice_and_errors(gpu, tmp_path):
    a = rnd((6, 5, 4, 3, 4), 4)
    p = str(tmp_path / "defo.uni")
    unifmt.write(p, a, is4d=True)
    s = F.Grid4Vec4(dims=(3, 4, 5, 1))
    for t in (0, 3, 5):
        F.readGrid4dUniSlice(p, t, s)
        assert np.array_equal(s.to_numpy()[0], a[t])
    with pytest.raises(F.FlofError):
        F.readGrid4dUniSlice(p, 6, s)
    with pytest.raises(F.FlofError):
        F.Grid4Vec4(dims=(3, 4, 5, 5)).load(p)       # t extent differs
    with pytest.raises(F.FlofError):
        F.Grid4Real(dims=(3, 4, 5, 6)).load(p)       # element size differs
    with pytest.raises(F.FlofError):
        F.Grid4Vec4(dims=(3, 4, 5, 6)).load(str(tmp_path / "missing.uni"))


# ---------------------------------------------------------------------------
# loadPlaceGrid4d
# ---------------------------------------------------------------------------
def slice_series(n, shape, seed):
    """n hi-res 3D SDF frames of a falling drop (cells, clamped to [-4, 4])."""
    sc = synth.scene_for(seed)
    z, y, x = shape
    return np.stack([synth.sdf_slice(sc, (x, y, z), t, n) for t in range(n)]).astype(np.float32)


PLACE = dict(offset=(2.4, 2.2, 2.0, 3.5), scale=(0.8, 0.8, 0.8, 0.8), fileIdxStart=0, fileIdxEnd=10,
             spread=1.0, overrideSize=(24, 22, 20, 26), overrideTimeOff=0.0, loadTimeScale=1.0,
             rescaleSdfValues=True, sdfIsoOff=-0.5, repeatStartFrame=0.1)


@pytest.mark.parametrize("variant", ["flof", "no_rescale", "partial"])
def test_load_place_grid4d_bitexact(gpu, orc, tmp_path, variant):
    dims = (24, 22, 20, 26)
    sl = slice_series(10, (33, 36, 40), 0)
    kw = dict(PLACE)
    prev = None
    if variant == "no_rescale":
        kw.update(rescaleSdfValues=False, sdfIsoOff=0.0, repeatStartFrame=0.0, spread=1.5)
    if variant == "partial":
        kw.update(overrideGoodRegion=11, overrideTimeOff=-4.0)
        prev = rnd((26, 20, 22, 24), 9)
    want = orc.loadPlaceGrid4d(dims, sl, phi=prev, **kw)
    phi = F.Grid4Real(dims=dims)
    if prev is not None:
        phi.from_numpy(prev)
    grids = [F.RealGrid(dims=(40, 36, 33, 1)).from_numpy(s) for s in sl]
    F.loadPlaceGrid4d(grids, phi, **kw)
    got = phi.to_numpy()
    assert np.array_equal(got, want)
    # the same from files named by a pattern
    for q, s in enumerate(sl):
        unifmt.write(tmp_path / f"slice_{q:04d}.uni", s, is4d=False)
    phi2 = F.Grid4Real(dims=dims)
    if prev is not None:
        phi2.from_numpy(prev)
    F.loadPlaceGrid4d(str(tmp_path / "slice_%04d.uni"), phi2, **kw)
    assert np.array_equal(phi2.to_numpy(), want)


def test_load_place_grid4d_pattern_checked(gpu, tmp_path):
    phi = F.Grid4Real(dims=(8, 8, 8, 8))
    with pytest.raises(F.FlofError):
        F.loadPlaceGrid4d(str(tmp_path / "s_%s.uni"), phi, (0, 0, 0, 0), (1, 1, 1, 1), 0, 4)
    with pytest.raises(F.FlofError):
        F.loadPlaceGrid4d(str(tmp_path / "s_%d_%d.uni"), phi, (0, 0, 0, 0), (1, 1, 1, 1), 0, 4)


# ---------------------------------------------------------------------------
# loadAdvectTimeSlice (non-optimised) and OptInit from a file
# ---------------------------------------------------------------------------
def defo_and_phi():
    r = np.random.default_rng(12)
    defo = (r.standard_normal((16, 12, 12, 12, 4)) * 0.6).astype(np.float32)
    phi = synth.sdf4d(synth.scene_for(1), (30, 30, 30, 16))
    return defo, phi


LATS = dict(loadTimeScale=1.0, defoOffset=(0, 0, 0, 0), defoScale=(1, 1, 1, 1),
            defoFactor=(2.5, 2.5, 2.5, 1.0))


@pytest.mark.parametrize("time,alpha", [(3.0, 0.5), (7.6, 0.25), (15.0, 1.0)])
def test_load_advect_time_slice_bitexact(gpu, orc, tmp_path, time, alpha):
    defo, phi = defo_and_phi()
    d0 = rnd((30, 30, 30), 3)
    want = orc.loadAdvectTimeSlice(defo, d0, phi, time, alpha, overrideSize=-1.0, **LATS)
    gphi = F.Grid4Real(dims=(30, 30, 30, 16)).from_numpy(phi)
    gdefo = F.Grid4Vec4(dims=(12, 12, 12, 16)).from_numpy(defo)
    dst = F.RealGrid(dims=(30, 30, 30, 1)).from_numpy(d0)
    F.loadAdvectTimeSlice(0, gdefo, dst, gphi, time, alpha, **LATS)
    assert np.array_equal(dst.to_numpy(), want)
    p = str(tmp_path / "defo.uni")
    unifmt.write(p, defo, is4d=True)
    dst2 = F.RealGrid(dims=(30, 30, 30, 1)).from_numpy(d0)
    F.loadAdvectTimeSlice(0, p, dst2, gphi, time, alpha, **LATS)
    assert np.array_equal(dst2.to_numpy(), want)


def test_optinit_from_file_matches_grid(gpu, tmp_path):
    defo, phi = defo_and_phi()
    p = str(tmp_path / "defo.uni")
    unifmt.write(p, defo, is4d=True)
    gphi = F.Grid4Real(dims=(30, 30, 30, 16)).from_numpy(phi)
    gdefo = F.Grid4Vec4(dims=(12, 12, 12, 16)).from_numpy(defo)
    outs = []
    for src in (gdefo, p):
        F.loadAdvectTimeSlice_OptInit(7, src)
        dst = F.RealGrid(dims=(30, 30, 30, 1))
        F.loadAdvectTimeSlice_OptRun(7, "", dst, gphi, 5.5, 0.5, bordSkip=2, **LATS)
        outs.append(dst.to_numpy())
        F.loadAdvectTimeSlice_Finish(7)
    assert np.array_equal(outs[0], outs[1])
