"""The seeded drop/pool input generator."""
import numpy as np

from ofblend_gb300 import synth


def test_reproducible_and_seed_dependent():
    a = synth.sdf4d(synth.scene_for(0), (16, 16, 16, 8))
    b = synth.sdf4d(synth.scene_for(0), (16, 16, 16, 8))
    c = synth.sdf4d(synth.scene_for(1), (16, 16, 16, 8))
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_range_layout_and_scaling():
    s = synth.scene_for(0)
    a = synth.sdf4d(s, (32, 32, 32, 32))
    assert a.shape == (32, 32, 32, 32) and a.dtype == np.float32
    assert a.min() == -4.0 and a.max() == 4.0
    # liquid below the pool surface, air at the top
    assert a[0, 16, 0, 16] < 0 and a[0, 16, -1, 16] > 0
    # the same scene at twice the resolution: values are in target cells
    b = synth.sdf4d(s, (64, 64, 64, 32))
    assert np.allclose(b[:, ::2, ::2, ::2].mean(), a.mean(), atol=0.3)


def test_drop_falls():
    s = synth.make_scene(5)
    d = s.drops[0]
    a = synth.sdf4d(s, (32, 32, 32, 32))
    ix, iz = int(d.x0), int(d.z0)
    col0 = a[0, iz, :, ix]
    col1 = a[20, iz, :, ix]
    # the drop's lowest inside cell moves down over time
    assert np.argmax(col0[10:] < 0) > np.argmax(col1[10:] < 0) or col1[10:].min() >= 0


def test_ellipsoid_and_flow_input():
    s = synth.scene_for(2)
    assert s.drops[0].axes is not None and all(4 <= a <= 10 for a in s.drops[0].axes)
    i = synth.flow_input(s, (8, 8, 8, 4))
    assert np.allclose(i, synth.sdf4d(s, (8, 8, 8, 4)) * np.float32(-0.005))
