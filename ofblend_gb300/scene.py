"""Scene-level helpers of the FlOF driver, on the GPU grids of this package.

These restate the small Python functions that scenes/flof.py and
scenes/ofHelpers.py wrap around the plugins, so that a flof.py-shaped driver
can run on the GPU: grid sizes and load offsets (ofHelpers.py:26-33, 59-83),
the flof parameter set (flof.py:69-84, 123-131, 266, 304-320), the input
conditioning postProcessPhiData (flof.py:491-531), the blend-union weights
blendW (flof.py:576-585), the time-SDF merge (flof.py:818-826) and the
writeResults smoothing (ofHelpers.py:108-113).
"""
from __future__ import annotations

from . import api
from .api import vec3, vec4

__all__ = ["initRes", "initOffsets", "flof_ofsd", "postProcessPhiData", "blendW",
           "timeSdfMerge", "sdfSmooth", "vec3", "vec4"]


def initRes(res, yFactor, fourdFactor, loadTimeScale):
    """(3D grid size as ints, 4D size as floats) for resolution res
    (ofHelpers.py:26-33)."""
    s4 = vec4(res * 1, res * yFactor, res * 1, res * fourdFactor * loadTimeScale)
    s3 = vec3(int(s4.x), int(s4.y), int(s4.z))
    return s3, s4


def initOffsets(gs4d, gs4dDefo, autoBorder, repeatStartDist, loadTimeScale):
    """Load offset/scale of the level-set data and of the deformation, and the
    magnitude factor of a deformation computed at gs4dDefo (ofHelpers.py:59-83).
    Returns (loadOffset, loadScale, defoOffset, defoScale, defoFactor)."""
    loadOffset = vec4(gs4d.x * autoBorder, gs4d.y * autoBorder, gs4d.z * autoBorder,
                      gs4d.t * autoBorder + repeatStartDist)
    inner = 1.0 - 2.0 * autoBorder
    loadScale = vec4(inner, inner, inner, inner * loadTimeScale)
    defoOffset = vec4(0.0)
    defoScale = vec4(1.0, 1.0, 1.0, loadTimeScale)
    defoFactor = vec4(gs4d.x / gs4dDefo.x, gs4d.y / gs4dDefo.y, gs4d.z / gs4dDefo.z,
                      gs4d.t / gs4dDefo.t)
    return loadOffset, loadScale, defoOffset, defoScale, defoFactor


def flof_ofsd(res: int) -> dict:
    """The parameter set flof.py uses for its two-drop setup at resolution res."""
    border = 0.1
    return {
        "postProcMode": 1,             # level-set post-processing
        "isosurfaceOff": 0,
        "isosurfaceMult": 1.0,
        "fourdFactor": 1.5,
        "yFactor": 1.0,
        "autoBorder": border,
        "autoBrdRes": int(res * border),
        "lsFactor": -0.1 / 20.0,
        "maxDist": 40,
        "cgAccuracy": 0.01,
        "resBackup": res,
        "repeatStartDist": float(res) * border,
        "postVelBlur": 4,
        "maxLSPDist": 10,
        "lspBlur": 2.0,
    }


def postProcessPhiData(iTarget, isSlice=False, loadOffset=None, ofsd=None):
    """Conditioning of a loaded 4D level set before the solve (flof.py:491-531):
    repeat the start frame, then in level-set mode offset/scale the values,
    push the border outside, extrapolate outside and inside the surface, and
    scale to the solver's units.  Mode 3 converts a smoke density instead."""
    ofsd = ofsd or {}
    loadOffset = loadOffset if loadOffset is not None else vec4(0.0)
    mode = ofsd["postProcMode"]
    if mode == -1:
        return
    api.repeatFrame4d(iTarget, loadOffset.t + 1.0 / float(ofsd["resBackup"]),
                      ofsd["repeatStartDist"], bnd=0)
    if mode == 1:
        if ofsd["isosurfaceOff"] != 0.0:
            iTarget.addConst(ofsd["isosurfaceOff"])
        if ofsd["isosurfaceMult"] != 1.0:
            iTarget.multConst(ofsd["isosurfaceMult"])
        iTarget.setBound(0.1, ofsd["autoBrdRes"])
        api.extrap4dLsSimple(iTarget, distance=ofsd["maxDist"])
        api.extrap4dLsSimple(iTarget, distance=ofsd["maxDist"], inside=True)
        iTarget.multConst(ofsd["lsFactor"])
    elif mode == 3:
        iTarget.addConst(-0.125)
        iTarget.multConst(-1.0 * ofsd["lsFactor"])
        iTarget.setBound(0.0, ofsd["autoBrdRes"])


def blendW(t, l):
    """Weights (w0, w_union, w1) of the two-way blend with union at alpha t and
    overlap l (flof.py:576-585)."""
    w0 = min(max((1.0 + l - 2.0 * t) / (1.0 + l), 0.0), 1.0)
    w1 = min(max((-1.0 + l + 2.0 * t) / (1.0 + l), 0.0), 1.0)
    return w0, 1.0 - w0 - w1, w1


def timeSdfMerge(dst, dstPrev2):
    """Temporal merge of one output frame with the frame two steps back
    (flof.py:818-826): union, then one smoothing pass of the positive side."""
    dst.join(dstPrev2)
    api.simpleBlurSpecial(dst, 1, 0.0)


def sdfSmooth(grid, sdfSmooth, sdfSmoothBord):
    """writeResults output smoothing (ofHelpers.py:108-113): one pass over the
    positive side, then one over every cell, both inside sdfSmoothBord-1."""
    if sdfSmooth > 0:
        api.simpleBlurSpecial(grid, 1, 0.0, sdfSmoothBord - 1)
        api.simpleBlurSpecial(grid, 1, -999.0, sdfSmoothBord - 1)
