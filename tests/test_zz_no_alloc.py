"""The allocation-free orientation average (dpx_mc_average_noalloc).

It serves callers that cannot call cudaMalloc/cudaFree — applications whose
device memory is pre-reserved by their own pool, or serving loops where a
device-synchronizing cudaFree would stall other streams.  Called through the
C-ABI with caller-owned device buffers, its I(q) must equal the regular entry
point's (dpx_orientation_average) within the parity tolerances used elsewhere,
on two calls in a row (the shared static scratch keeps the previous call's
contents).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import dpx
from dpx import _lib
from dpx import models as M
from helpers import globule, rel

pytestmark = pytest.mark.gpu


def _regular(ctx, grid, Q, dirs, eps):
    res = np.zeros(len(Q))
    h = (C.c_void_p * 1)(grid.handle.value)
    _lib.check(dpx.lib().dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, len(Q),
                                                 _lib.dptr(Q), dirs.ctypes.data_as(C.c_void_p), 0, 0, len(dirs), eps,
                                                 _lib.dptr(res)))
    return res


@pytest.mark.parametrize("prec,tol", [(M.FP64, 1e-10), (M.FP32, 1e-4)])
def test_noalloc_matches_regular_entry_point(ctx, prec, tol):
    import torch
    amp = globule(500, 1.5, seed=77)
    gs, qmax = 40, 5.0
    grid = amp.calculateGrid(ctx, qmax, gs, prec)
    ctx.synchronize()
    stream = torch.cuda.Stream()
    cases = [(np.linspace(0, qmax, 150), M.mc_directions(5, 3000), 0.0),
             (np.linspace(0.2, 4.7, 61), M.mc_directions(6, 2500), 1e-3)]
    for Q, dirs, eps in cases:  # two calls in a row through the shared scratch
        Q = np.ascontiguousarray(Q)
        d_dirs = torch.from_numpy(np.ascontiguousarray(dirs)).cuda()
        d_res = torch.full((len(Q),), float("nan"), dtype=torch.float64, device="cuda")
        rc = dpx.lib().dpx_mc_average_noalloc(C.c_void_p(grid.device_ptr), gs, qmax, prec, len(Q), _lib.dptr(Q),
                                              C.c_void_p(d_dirs.data_ptr()), len(dirs), eps,
                                              C.c_void_p(d_res.data_ptr()), C.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        stream.synchronize()
        got = d_res.cpu().numpy()
        want = _regular(ctx, grid, Q, dirs, eps)
        assert np.all(np.isfinite(got))
        assert rel(got, want) <= tol


def test_noalloc_rejects_requests_beyond_its_scratch(ctx):
    import torch
    amp = globule(100, 0.8, seed=78)
    grid = amp.calculateGrid(ctx, 4.0, 40, M.FP32)
    # few samples but 400,000 q values over 20 brackets: about 42 MB of partial
    # sums, above the static limit.  Every buffer is backed in full, so even a
    # request that slipped past the check would read and write valid memory.
    Q = np.linspace(0, 4.0, 400_000)
    n = 1000
    d_dirs = torch.from_numpy(M.mc_directions(9, n)).cuda()
    d_res = torch.zeros(len(Q), dtype=torch.float64, device="cuda")
    rc = dpx.lib().dpx_mc_average_noalloc(C.c_void_p(grid.device_ptr), 40, 4.0, M.FP32, len(Q), _lib.dptr(Q),
                                          C.c_void_p(d_dirs.data_ptr()), n, 0.0, C.c_void_p(d_res.data_ptr()), None)
    assert rc == -1
    assert b"static limit" in dpx.lib().dpx_last_error()
