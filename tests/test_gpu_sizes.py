"""Parity at the workloads' own sizes, and against the FP64 direct sum.

* The 2,000-atom vacuum globule (r = 2.5 nm) on a 60-layer grid, qmax 5,
  200 q in [0, 5], Monte Carlo over 1e5 seeded directions shared by every
  bracket: the plain FP64 path within 1e-10 of the FP64 oracle's
  IntegrateLayersTogether, the FP32-bulk path within 1e-4.
* dpx_direct_intensity (the FP64 direct sum every grid result reports its
  error against) within 1e-10 of the oracle's direct sum, with solvent boxes
  and docked copies.
* The 20,000-atom subunit with its 0.3 nm solvation layer on the 200-layer
  grid (qmax 7.5): the FP32 harmonic grid's I(q) against the FP64 direct sum
  at 20 q x 2,000 directions.  The grid method itself errs against the direct
  sum (interpolation); the FP32 bulk precision must add nothing visible to
  that: FP32 and plain FP64 grids err alike against the direct sum.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import dpx
from dpx import _lib
from dpx import models as M
from helpers import LAYER, SOLVENT, VACUUM, globule, rel

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


def _average(ctx, grid, Q, dirs, n=None):
    """dpx_orientation_average of one grid at identity placement."""
    res = np.zeros(len(Q))
    h = (C.c_void_p * 1)(grid.handle.value)
    d = np.ascontiguousarray(dirs)
    _lib.check(dpx.lib().dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, len(Q),
                                                 _lib.dptr(Q), d.ctypes.data_as(C.c_void_p), 0, 0,
                                                 len(d) if n is None else n, 0.0, _lib.dptr(res)))
    return res


def _direct(ctx, amp, Q, dirs, copy_rot=None, copy_tr=None):
    descs, keep = M.pdb_descs([amp])
    descs[0].center = None  # the frame as given: the direct sum does not centre
    res = np.zeros(len(Q))
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    nc = 0 if copy_rot is None else len(copy_rot)
    cr = None if copy_rot is None else np.ascontiguousarray(copy_rot, dtype=np.float64)
    ct = None if copy_tr is None else np.ascontiguousarray(copy_tr, dtype=np.float64)
    _lib.check(dpx.lib().dpx_direct_intensity(ctx.handle, descs, nc, _lib.dptr(cr), _lib.dptr(ct), len(Q),
                                              _lib.dptr(Q), len(d), _lib.dptr(d), _lib.dptr(res)))
    del keep
    return res


def test_config0_full_size_matches_oracle(ctx):
    """2,000 atoms, L = 60 (1,548,289 cells), 200 q, 1e5 shared directions."""
    amp = globule(2000, 2.5, seed=20250, extra=VACUUM)
    gs, qmax = 120, 5.0
    Q = np.linspace(0.0, qmax, 200)
    dirs = M.mc_directions(1234, 100_000)
    s = O.Struct.from_pdb(amp)
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 0.0)
    for prec, tol in ((M.FP64, TOL64), (M.FP32, TOL32)):
        I = M.DomainModel([amp], gs, qmax, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
        err = rel(I, ref)
        print(f"config-0 full size: precision {'FP64' if prec == M.FP64 else 'FP32'} max rel err {err:.3e}")
        assert err <= tol


def test_direct_sum_matches_oracle(ctx):
    amp = globule(400, 1.4, seed=31, extra=LAYER)
    Q = np.array([0.0, 0.4, 1.3, 2.9, 4.4, 6.0])
    dirs = M.mc_directions(8, 64)
    s = O.Struct.from_pdb(amp)
    assert s.boxes is not None and len(s.boxes) > 10
    got = _direct(ctx, amp, Q, dirs)
    want = O.direct_intensity(s, Q, dirs)
    assert rel(got, want) <= TOL64
    rng = np.random.default_rng(5)
    crot = rng.uniform(-np.pi, np.pi, (7, 3))
    ctr = rng.uniform(-4, 4, (7, 3))
    got = _direct(ctx, amp, Q, dirs, crot, ctr)
    want = O.direct_intensity(s, Q, dirs, crot, ctr)
    assert rel(got, want) <= TOL64


def test_config1_subunit_against_direct_sum(ctx):
    """The bench's 20k-atom subunit (r = 5 nm, 333 e/nm^3 dummy atoms, 0.3 nm
    layer at 400 e/nm^3), 200 layers, qmax 7.5: grid I(q) (FP32 harmonic and
    plain FP64) against the FP64 direct sum at every 25th of the 500 q and the
    first 2,000 of the 1e5 directions; the direct sum itself against the
    oracle's on 3 q x 24 directions."""
    amp = globule(20000, 5.0, seed=20251, extra=LAYER)
    gs, qmax = 400, 7.5
    Qall = np.linspace(0.0, qmax, 500)
    Q = np.ascontiguousarray(Qall[12::25])
    dirs = np.ascontiguousarray(M.mc_directions(1234, 100_000)[:2000])
    s = O.Struct.from_pdb(amp)
    small = _direct(ctx, amp, Q[[0, 9, 19]], dirs[:24])
    assert rel(small, O.direct_intensity(s, Q[[0, 9, 19]], dirs[:24])) <= TOL64
    direct = _direct(ctx, amp, Q, dirs)
    errs = {}
    for prec in (M.FP32, M.FP64):
        grid = amp.calculateGrid(ctx, qmax, gs, prec)
        errs[prec] = rel(_average(ctx, grid, Q, dirs), direct)
        amp._grid = None
        grid.close()
    print(f"config-1 vs FP64 direct sum: FP32 harmonic grid {errs[M.FP32]:.3e}, plain FP64 grid {errs[M.FP64]:.3e}")
    # the grid method's own error, the same with FP32 bulk arithmetic
    assert errs[M.FP64] <= 5e-2
    assert abs(errs[M.FP32] - errs[M.FP64]) <= TOL32 + 0.05 * errs[M.FP64]
