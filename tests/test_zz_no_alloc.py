"""flof_calcLsDiff4d_noalloc, the entry point for callers that cannot
allocate device memory (fixed device-memory budgets, loops that cannot
afford the device synchronisation an allocation may cost).

It is called through the C ABI on buffers the caller allocated (torch
tensors here) and must give what the context-based flof_calcLsDiff4d gives,
on two calls in a row: its scratch array is shared and keeps the previous
call's contents, so the second call checks that the call clears what must
start at zero.  Collected last, so that a failure here leaves every other
test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_calc_ls_diff_noalloc_matches_context_entry_point():
    import torch

    import ofblend_gb300 as F
    from ofblend_gb300 import _lib, synth

    lib = _lib.lib()
    dims = (40, 36, 32, 24)
    X, Y, Z, T = dims
    i0 = synth.flow_input(synth.scene_for(0), dims)
    i1 = synth.flow_input(synth.scene_for(1), dims)
    corr, bnd = 0.1 / 20, 4

    g0 = F.Grid4Real(dims=dims).from_numpy(i0)
    g1 = F.Grid4Real(dims=dims).from_numpy(i1)
    gout = F.Grid4Real(dims=dims)
    want = np.float32(F.calcLsDiff4d(g0, g1, gout, corr, bnd))
    want_out = gout.to_numpy()
    assert want > 0

    t0 = torch.from_numpy(i0).cuda()
    t1 = torch.from_numpy(i1).cuda()
    tout = torch.empty_like(t0)
    tres = torch.empty(1, dtype=torch.float32, device="cuda")
    cd = (ctypes.c_int * 4)(*dims)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    inner = (slice(bnd, T - bnd), slice(bnd, Z - bnd), slice(bnd, Y - bnd), slice(bnd, X - bnd))
    for call in range(2):
        tout.fill_(-7.0)
        tres.fill_(-1.0)
        st = lib.flof_calcLsDiff4d_noalloc(_ptr(t0), _ptr(t1), _ptr(tout), cd, corr, bnd, _ptr(tres), stream)
        assert st == 0, lib.flof_last_error()
        torch.cuda.synchronize()
        got = np.float32(tres.item())
        # same tolerance as the context entry point's own parity test
        assert abs(got - want) <= np.spacing(want), (call, got, want)
        assert np.array_equal(tout.cpu().numpy()[inner], want_out[inner])
        assert (tout.cpu().numpy()[0] == -7.0).all()  # cells outside the box untouched

    # without the per-cell output
    st = lib.flof_calcLsDiff4d_noalloc(_ptr(t0), _ptr(t1), None, cd, corr, bnd, _ptr(tres), stream)
    assert st == 0
    torch.cuda.synchronize()
    assert abs(np.float32(tres.item()) - want) <= np.spacing(want)

    # a bnd that leaves no cells: the reference's 0 * (1 / count), here
    # count 0 (NaN), as the context entry point gives
    st = lib.flof_calcLsDiff4d_noalloc(_ptr(t0), _ptr(t1), None, cd, corr, 20, _ptr(tres), stream)
    assert st == 0, lib.flof_last_error()
    torch.cuda.synchronize()
    assert np.isnan(tres.item()) and np.isnan(F.calcLsDiff4d(g0, g1, None, corr, 20))
    # sizes beyond what the entry point handles are rejected with a message
    st = lib.flof_calcLsDiff4d_noalloc(_ptr(t0), _ptr(t1), None, cd, corr, -1, _ptr(tres), stream)
    assert st == 1 and b"bnd" in lib.flof_last_error()
    big = (ctypes.c_int * 4)(2048, 2048, 1024, 2)
    st = lib.flof_calcLsDiff4d_noalloc(_ptr(t0), _ptr(t1), None, big, corr, 0, _ptr(tres), stream)
    assert st == 1 and b"2^31" in lib.flof_last_error()
