"""CPU checks of the oracle's conditioning / output-stage functions against
independent numpy restatements, and of the scene helpers' formulas.  The
reference's own tests do not cover these functions, so this is the oracle's
cross-check: two restatements written differently (loops in C, array
expressions here) must agree bit for bit."""
import numpy as np
import pytest

from ofblend_gb300 import scene, synth


def np_extrap(phi, distance, inside):
    """extrap4dLsSimple (optflow4d.cpp:1332-1406) with numpy shifts."""
    a = phi.astype(np.float32).copy()
    tmp = np.zeros(a.shape, np.int32)
    inner = (slice(1, -1),) * 4
    core = a[inner]
    tmp[inner] = ((core > 0) if inside else (core < 0)).astype(np.int32)

    def nb(arr):
        # neighbour views in nbs4d order: -x,+x,-y,+y,-z,+z,-t,+t (axes reversed)
        out = []
        for ax in (3, 2, 1, 0):
            for s in (-1, 1):
                sl = [slice(1, -1)] * 4
                sl[ax] = slice(1 + s, arr.shape[ax] - 1 + s)
                out.append(arr[tuple(sl)])
        return out

    t0 = tmp[inner].copy()
    hit = np.zeros(t0.shape, bool)
    for v in nb(tmp):
        hit |= v == 1
    t0[(t0 == 0) & hit] = 2
    tmp[inner] = t0
    direction = np.float32(-1.0 if inside else 1.0)
    for d in range(2, distance + 1):
        cur = tmp[inner]
        avg = np.zeros(cur.shape, np.float32)
        cnt = np.zeros(cur.shape, np.int32)
        for tv, pv in zip(nb(tmp), nb(a)):
            m = tv == d
            avg = np.where(m, avg + pv, avg).astype(np.float32)
            cnt += m
        upd = (cur == 0) & (cnt > 0)
        val = (avg / cnt.clip(1).astype(np.float32) + direction).astype(np.float32)
        sub = a[inner]
        sub[upd] = val[upd]
        a[inner] = sub
        cur = cur.copy()
        cur[upd] = d + 1
        tmp[inner] = cur
    sub = a[inner]
    sub[tmp[inner] == 0] = np.float32(direction * (distance + 2))
    a[inner] = sub
    return a


@pytest.mark.parametrize("distance,inside", [(4, False), (6, True), (1, False)])
def test_oracle_extrap_matches_numpy(orc, distance, inside):
    a = synth.sdf4d(synth.scene_for(2), (14, 13, 12, 11)) * 0.4
    assert np.array_equal(orc.extrap4dLsSimple(a, distance, inside), np_extrap(a, distance, inside))


def np_simple_blur(a, it, thresh, bord):
    """knSimpleBlurSpecial (test.cpp:94-131) on a (Z, Y, X) array, Z > 1."""
    a = a.astype(np.float32)
    tmp = np.zeros_like(a)
    cur, nxt = a.copy(), tmp
    Z, Y, X = a.shape
    for _ in range(it):
        c = cur[1:-1, 1:-1, 1:-1]
        s = (cur[1:-1, 1:-1, 2:] + cur[1:-1, 1:-1, :-2]).astype(np.float32)
        s = (s + cur[1:-1, 2:, 1:-1]).astype(np.float32)
        s = (s + cur[1:-1, :-2, 1:-1]).astype(np.float32)
        s = (s + (cur[2:, 1:-1, 1:-1] + cur[:-2, 1:-1, 1:-1]).astype(np.float32)).astype(np.float32)
        s = (s.astype(np.float64) * (1.0 / 6.0)).astype(np.float32)
        k, j, i = np.meshgrid(np.arange(1, Z - 1), np.arange(1, Y - 1), np.arange(1, X - 1),
                              indexing="ij")
        inb = (i >= bord) & (j >= bord) & (k >= bord) & (i < X - bord) & (j < Y - bord) & (k < Z - bord)
        keep = ~inb | (c < np.float32(thresh))
        nxt[1:-1, 1:-1, 1:-1] = np.where(keep, c, s)
        cur, nxt = nxt, cur
    return cur


@pytest.mark.parametrize("it,thresh,bord", [(1, 0.0, 0), (2, -999.0, 2), (3, 0.25, 1)])
def test_oracle_simple_blur_matches_numpy(orc, it, thresh, bord):
    a = np.random.default_rng(4).standard_normal((9, 11, 13)).astype(np.float32)
    assert np.array_equal(orc.simpleBlurSpecial(a, it, thresh, bord), np_simple_blur(a, it, thresh, bord))


def test_oracle_join_and_bounds(orc):
    r = np.random.default_rng(5)
    a, b = r.standard_normal((2, 7, 8, 9)).astype(np.float32)
    assert np.array_equal(orc.join(a, b), np.minimum(a, b))
    w = 1
    want = a.copy()
    want[:w + 1], want[-w - 1:] = 0.5, 0.5
    want[:, :w + 1], want[:, -w - 1:] = 0.5, 0.5
    want[:, :, :w + 1], want[:, :, -w - 1:] = 0.5, 0.5
    assert np.array_equal(orc.setBound3(a, 0.5, w), want)
    # a 2D grid ignores z
    a2 = a[:1]
    want2 = a2.copy()
    want2[:, :w + 1], want2[:, -w - 1:] = 0.5, 0.5
    want2[:, :, :w + 1], want2[:, :, -w - 1:] = 0.5, 0.5
    assert np.array_equal(orc.setBound3(a2, 0.5, w), want2)


def test_oracle_repeat_frame_is_time_lerp(orc):
    """At cell centres in x, y, z the interpolation is a lerp in t between the
    slices around srct."""
    a = np.random.default_rng(6).standard_normal((9, 6, 7, 8)).astype(np.float32)
    srct = np.float32(2.25)
    out = orc.repeatFrame4d(a, srct, 2.0, 0)
    w1 = np.float32(srct - np.float32(2.0))
    w0 = np.float32(1.0 - w1)
    lerp = (a[2] * w0 + a[3] * w1).astype(np.float32)
    for t in (0, 1, 2):
        assert np.allclose(out[t], lerp, rtol=0, atol=1e-6)
    assert np.array_equal(out[3:], a[3:])


def test_scene_helpers():
    s3, s4 = scene.initRes(64, 1.0, 1.5, 1.0)
    assert (s3.x, s3.y, s3.z) == (64, 64, 64) and s4.t == 96.0
    lo, ls, do, ds, df = scene.initOffsets(s4, scene.vec4(32, 32, 32, 48), 0.1, 6.4, 1.0)
    assert (lo.x, lo.t) == (pytest.approx(6.4), pytest.approx(9.6 + 6.4))
    assert ls.x == pytest.approx(0.8) and ds.t == 1.0 and df.x == 2.0 and df.t == 2.0
    assert scene.blendW(0.0, 0.1) == (1.0, 0.0, 0.0)
    w0, wu, w1 = scene.blendW(0.5, 0.1)
    assert w0 == pytest.approx(0.1 / 1.1) and w1 == pytest.approx(0.1 / 1.1)
    assert wu == pytest.approx(1 - 0.2 / 1.1)
    o = scene.flof_ofsd(64)
    assert o["autoBrdRes"] == 6 and o["repeatStartDist"] == pytest.approx(6.4)
