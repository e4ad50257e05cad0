"""Generates tests/golden/flof_golden.npz: small input/output fixtures of the
CPU oracle (oracle/flof_oracle.c, float build) on seeded inputs.

The fixtures freeze the oracle's results so that (a) a change of the oracle
shows up in the CPU suite and (b) the GPU tests can compare against stored
vectors as well as against the live oracle.  Regenerate with
`python tests/golden/gen_golden.py` after an intended oracle change.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ofblend_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "flof_golden.npz")


def cases() -> dict:
    o = oracle.get(False)
    g = {}
    rng = np.random.default_rng(1234)

    # advect4d, Real and Vec4, non-cubic grid
    dims = (9, 8, 7, 6)
    X, Y, Z, T = dims
    vel = rng.uniform(-2.5, 2.5, size=(T, Z, Y, X, 4)).astype(np.float32)
    src = rng.standard_normal((T, Z, Y, X)).astype(np.float32)
    srcv = rng.standard_normal((T, Z, Y, X, 4)).astype(np.float32)
    g["adv_vel"], g["adv_src"], g["adv_srcv"] = vel, src, srcv
    g["adv_out_a07"] = o.advect4d(vel, src, 0.7)
    g["adv_outv_a1"] = o.advect4d(vel, srcv, 1.0)

    # interpolateGrid4d with offset/scale, up and down
    g["ip_src"] = src
    g["ip_up"] = o.interpolateGrid4d((13, 11, 10, 7), src, offset=(1.0, 0.5, 0.0, 2.0),
                                     scale=(0.8, 0.8, 0.8, 1.0))
    g["ip_down_v"] = o.interpolGrid((4, 4, 3, 3), srcv)

    # Gaussian blur sigma 2 (radius 2) and 1.125 (radius 1)
    g["blur_in"] = srcv
    g["blur_s2"] = o.gaussianBlur4d(srcv, 2.0)
    g["blur_s1125"] = o.gaussianBlur4d(srcv, 1.125)

    # calcLsDiff
    a = rng.standard_normal((T, Z, Y, X)).astype(np.float32) * 0.01
    b = rng.standard_normal((T, Z, Y, X)).astype(np.float32) * 0.01
    g["ls_a"], g["ls_b"] = a, b
    g["ls_val"] = np.float32(o.calcLsDiff4d(a, b, 0.1 / 20, 2))

    # one-level solve with blur and border reset on drop data
    dims = (12, 11, 10, 9)
    i0 = synth.flow_input(synth.make_scene(11, ndrops=1, radius_range=(3.0, 4.0)), dims)
    i1 = synth.flow_input(synth.make_scene(12, ndrops=1, radius_range=(3.0, 4.0)), dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    g["of_i0"], g["of_i1"] = i0, i1
    v, it, res = o.opticalFlow4d(zv, i0, i1, 0.001, 0.0001, 4.0, 1e-4, 0.1)
    g["of_vel"], g["of_iters"], g["of_res"] = v, np.int32(it), np.float32(res)

    # multiscale, flof parameters, two levels (minGridSize 5)
    dims = (12, 12, 12, 10)
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    zv = np.zeros(i0.shape + (4,), np.float32)
    v, err, st = o.opticalFlowMultiscale4d(zv, i0, i1, wSmooth=0.001, wEnergy=0.0001, cgAccuracy=0.01,
                                           postVelBlur=4, cfl=999, multiStep=3, minGridSize=5,
                                           doFinalProject=True, resetBndWidth=0.1)
    g["ms_i0"], g["ms_i1"], g["ms_vel"], g["ms_err"] = i0, i1, v, np.float32(err)
    g["ms_iters"] = np.array([s[1] for s in st], np.int32)

    # mode-3 frame lookup
    defo = rng.uniform(-1.5, 1.5, size=(5, 6, 6, 6, 4)).astype(np.float32)
    phi = rng.standard_normal((5, 23, 22, 24)).astype(np.float32)
    dst = np.full((23, 22, 24), 7.0, np.float32)
    g["lk_defo"], g["lk_phi"] = defo, phi
    g["lk_out"] = o.optRunFrame(defo, dst, phi, time=2.5, blendAlpha=0.25,
                                defoFactor=(4.0, 4.0, 4.0, 1.0), overrideSize=(24, 22, 23, 5), bordSkip=2)
    return g


if __name__ == "__main__":
    g = cases()
    np.savez_compressed(OUT, **g)
    print(OUT, os.path.getsize(OUT), "bytes")
