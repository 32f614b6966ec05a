"""Serving engine (dpx_server) on the GPU: each request's I(q) is the same
alone and in the mix, grids are reused by placement-only repeats, the memory
budget admits and evicts, and requests that cannot fit fail cleanly."""
import numpy as np
import pytest

from dpx import _lib
from dpx import models as M
from dpx.serve import Server
from helpers import LAYER, SOLVENT, VACUUM, fill_method, globule

pytestmark = pytest.mark.gpu


def _mix():
    """(amps, grid_size, qmax, Q, precision) per request; leaves shared by repeats."""
    a = globule(500, 1.5, seed=101, extra=SOLVENT)
    b = globule(300, 1.2, seed=102, extra=VACUUM)
    c = globule(800, 1.9, seed=103, extra=LAYER)
    d = globule(200, 1.0, seed=104, extra=VACUUM)
    b2 = globule(300, 1.2, seed=102, extra=VACUUM)  # same content as b: same cache key
    b2.location = (0.4, -0.2, 0.1, 0.3, 0.2, 0.1)
    rows = [[0, 0, 0, 0, 0, 0], [3.0, 0, 0, 0, 0, 90], [0, 3.0, 0.5, 45, 30, 10], [-2.0, 1.0, 0, 45, 30, 10],
            [1.0, 1.0, 2.0, 10, 20, 30]]
    sym = M.ManualSymmetry(d, rows, scale=0.8, use_grid=False)
    rows2 = [[r[0] + 0.3, r[1], r[2], r[3] + 5, r[4], r[5]] for r in rows]  # repeat: new R_k / t_k only
    sym2 = M.ManualSymmetry(d, rows2, scale=0.8, use_grid=False)
    reqs = [
        ([a], 24, 4.0, np.linspace(0, 4.0, 37), M.FP32),
        ([b], 20, 3.0, np.linspace(0.2, 3.0, 25), M.FP32),
        ([c, b], 28, 5.0, np.linspace(0, 5.0, 41), M.FP32),
        ([sym], 24, 4.0, np.linspace(0, 4.0, 30), M.FP32),
        ([b2], 20, 3.0, np.linspace(0.2, 3.0, 25), M.FP32),   # repeat of b, moved
        ([sym2], 24, 4.0, np.linspace(0, 4.0, 30), M.FP32),  # repeat of sym, new copies
        ([a], 24, 4.0, np.linspace(0, 4.0, 37), M.FP64),
        ([d], 16, 2.5, np.linspace(0, 2.5, 20), M.FP64),
    ]
    return reqs


def _direct(ctx, req, dirs, method):
    """One DomainModel solve, filled with the fill method the server uses."""
    amps, gs, qmax, Q, prec = req
    for a in amps:
        for leaf in (a, getattr(a, "child", None)):
            if leaf is not None:
                leaf._grid = None
    with fill_method(ctx, method):
        return M.DomainModel(amps, gs, qmax, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)


@pytest.fixture(params=[_lib.DPX_FILL_HARMONIC, _lib.DPX_FILL_DIRECT], ids=["harmonic", "direct"])
def method(request, ctx):
    """The server fills with the context's FP32 fill method."""
    with fill_method(ctx, request.param):
        yield request.param


def test_server_same_alone_and_in_the_mix(ctx, method):
    dirs = M.mc_directions(13, 640)
    reqs = _mix()
    direct = [_direct(ctx, r, dirs, method) for r in reqs]
    # alone: one request at a time through a fresh server
    alone = []
    for r in reqs:
        srv = Server(ctx, dirs, max_inflight=4, n_streams=3)
        t = srv.submit_models(r[0], r[1], r[2], r[3], precision=r[4])
        alone.append(srv.wait(t)[0])
        srv.close()
    # in the mix: everything submitted at once
    srv = Server(ctx, dirs, max_inflight=4, n_streams=3)
    tickets = [srv.submit_models(r[0], r[1], r[2], r[3], precision=r[4]) for r in reqs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    for k, (x, y, (z, lat)) in enumerate(zip(direct, alone, mixed)):
        assert np.allclose(y, x, rtol=1e-12, atol=0), k
        assert np.allclose(z, x, rtol=1e-12, atol=0), k
        assert lat > 0
    assert st["completed"] == len(reqs) and st["failed"] == 0
    # b2 and sym2 change placements only: their grids are found resident (or
    # filled once within the same turn); no (leaf, grid) is filled twice:
    # FP32 a@24, b@20, c@28, b@28, d@24 and FP64 a@24, d@16
    assert st["grid_fills"] == 7
    if method == _lib.DPX_FILL_DIRECT:  # one batched launch per turn, FP64 one per grid
        assert st["fill_launches"] <= st["grid_fills"]


def test_server_budget_evicts_and_rejects(ctx, method):
    dirs = M.mc_directions(14, 256)
    reqs = _mix()[:4]
    direct = [_direct(ctx, r, dirs, method) for r in reqs]
    import dpx
    g28 = dpx.lib().dpx_grid_bytes(28, M.FP32)
    # room for about two grids: later requests evict earlier, unpinned grids
    srv = Server(ctx, dirs, hbm_budget_bytes=int(2.5 * g28), max_inflight=2, n_streams=2)
    outs = [srv.wait(srv.submit_models(r[0], r[1], r[2], r[3], precision=r[4]))[0] for r in reqs]
    st = srv.stats()
    for x, y in zip(outs, direct):
        assert np.allclose(x, y, rtol=1e-12, atol=0)
    assert st["evictions"] >= 1
    assert st["bytes_peak"] <= st["budget"]
    # a request larger than the whole budget fails with DPX_ERR_OOM, the server keeps serving
    big = globule(100, 1.0, seed=105)
    t = srv.submit_models([big], 120, 5.0, np.linspace(0, 5, 10))
    with pytest.raises(dpx.DpxError) as e:
        srv.wait(t)
    assert e.value.code == -3
    x = srv.wait(srv.submit_models(reqs[1][0], reqs[1][1], reqs[1][2], reqs[1][3]))[0]
    assert np.allclose(x, direct[1], rtol=1e-12, atol=0)
    srv.close()
