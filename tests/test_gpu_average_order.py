"""The orientation average takes a shared direction set in an angular order
when eps = 0 (the mean is the same; only the order of the sums changes).
Against the same directions given per layer (a layer stride: taken as given)."""
import ctypes as C

import numpy as np
import pytest

from dpx import _lib
from dpx import models as M
from helpers import SOLVENT, globule, rel

pytestmark = pytest.mark.gpu


def _average(ctx, grid, Q, dirs, stride, n):
    res = np.zeros(len(Q))
    h = (C.c_void_p * 1)(grid.handle.value)
    d = np.ascontiguousarray(dirs)
    _lib.check(_lib.lib().dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, len(Q),
                                                  _lib.dptr(Q), d.ctypes.data_as(C.c_void_p), 0, stride, n, 0.0,
                                                  _lib.dptr(res)))
    return res


@pytest.mark.parametrize("prec,tol", [(M.FP64, 1e-12), (M.FP32, 1e-5)])
def test_angular_order_keeps_the_mean(ctx, prec, tol):
    amp = globule(600, 1.5, seed=91, extra=SOLVENT)
    gs, qmax = 40, 5.0
    grid = amp.calculateGrid(ctx, qmax, gs, prec)
    Q = np.ascontiguousarray(np.linspace(0.0, qmax, 80))
    dirs = M.mc_directions(7, 4000)
    ordered = _average(ctx, grid, Q, dirs, 0, len(dirs))
    per_layer = np.tile(dirs, (gs // 2, 1))  # the same set for every layer
    given = _average(ctx, grid, Q, per_layer, len(dirs), len(dirs))
    assert np.all(np.isfinite(ordered))
    assert rel(ordered, given) <= tol
