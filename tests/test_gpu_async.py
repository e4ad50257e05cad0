"""Asynchronous host transfers on the context's copy stream: each copy is
ordered after the work queued when it was issued, and copy_wait orders later
work after the copy."""
import numpy as np
import pytest

import ofblend_gb300 as F

pytestmark = pytest.mark.gpu


def pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


def test_upload_then_use(gpu):
    dims = (33, 20, 17, 9)
    r = np.random.default_rng(1)
    a = r.standard_normal((dims[3], dims[2], dims[1], dims[0])).astype(np.float32)
    host = pinned(a.shape)
    host[...] = a
    g = F.Grid4Real(dims=dims)
    g.upload_async(host).copy_wait()
    g.multConst(2.0)
    assert np.array_equal(g.to_numpy(), a * np.float32(2.0))


def test_download_sees_queued_work_and_not_later_work(gpu):
    dims = (24, 16, 12, 8)
    g = F.Grid4Vec4(dims=dims)
    g.setConst([1.0, 2.0, 3.0, 4.0])
    out = pinned(g.to_numpy().shape)
    g.download_async(out)          # after setConst
    g.copy_wait()                  # the overwrite below waits for the copy
    g.setConst([9.0, 9.0, 9.0, 9.0])
    F.context().copies_sync()
    assert np.all(out == np.array([1, 2, 3, 4], np.float32))
    assert np.all(g.to_numpy() == 9.0)


def test_many_grids_interleaved(gpu):
    dims = (40, 24, 16, 12)
    shape = (dims[3], dims[2], dims[1], dims[0])
    gs = [F.Grid4Real(dims=dims) for _ in range(6)]
    ins = [pinned(shape) for _ in gs]
    outs = [pinned(shape) for _ in gs]
    for k, (g, h) in enumerate(zip(gs, ins)):
        h[...] = k + 0.5
        g.upload_async(h)
    for k, (g, o) in enumerate(zip(gs, outs)):
        g.copy_wait()
        g.addConst(float(k))
        g.download_async(o)
    F.context().synchronize()  # both streams
    for k, o in enumerate(outs):
        assert np.all(o == np.float32(2 * k + 0.5)), k


def test_rejects_wrong_buffers(gpu):
    g = F.Grid4Real(dims=(8, 8, 8, 8))
    with pytest.raises(F.FlofError):
        g.download_async(np.zeros(10, np.float32))
    with pytest.raises(F.FlofError):
        g.upload_async(np.zeros((8, 8, 8, 8), np.float64))
