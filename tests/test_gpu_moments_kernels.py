"""The harmonic fill's other moments kernels against the FP64 oracle's direct
sum and against the default mma.sync TF32 kernel, through the C-ABI
(dpx_set_moments_kernel): the mma.sync FP16 kernel (m16n8k16, operands split
into value and remainder) and the fifth-generation tensor-core kernel
(tcgen05.mma, FP16 split operands, accumulators in tensor memory).

The leaves reach high orders (a 3 nm globule at q_max 12 with the solvation
layer: radial bins up to l_b of about 60), so a unit's (l, m) steps span
several CTAs and slots start inside an octet of orders (the silent warm-up).

Tolerances: grid amplitudes within 2e-6 of the largest amplitude (the FP32
bound of the direct fill); the kernels within 1e-6 of each other; I(q) within
1e-4 of the plain FP64 path.
"""
import ctypes as C
from contextlib import contextmanager

import numpy as np
import pytest

import oracle as O
from dpx import _lib
from dpx import models as M
from helpers import LAYER, SOLVENT, globule, rel, rel_to_max

pytestmark = pytest.mark.gpu


@contextmanager
def moments_kernel(kind):
    L = _lib.lib()
    before = L.dpx_get_moments_kernel()
    _lib.check(L.dpx_set_moments_kernel(kind))
    try:
        yield
    finally:
        _lib.check(L.dpx_set_moments_kernel(before))


def device_faults():
    f = C.c_uint(0)
    _lib.check(_lib.lib().dpx_take_device_faults(C.byref(f)))
    return f.value


@pytest.fixture
def harmonic(ctx):
    before = ctx.fill_method()
    ctx.set_fill_method(_lib.DPX_FILL_HARMONIC)
    device_faults()
    yield ctx
    ctx.set_fill_method(before)
    assert device_faults() == 0


def _fill(ctx, amp, qmax, gs, kind):
    amp._grid = None
    with moments_kernel(kind):
        g = amp.calculateGrid(ctx, qmax, gs, M.FP32)
        v, d = g.read(True, True)
    amp._grid = None
    return v, d


KINDS = pytest.mark.parametrize("kind", [_lib.DPX_MOMENTS_MMA_F16, _lib.DPX_MOMENTS_TCGEN05], ids=["f16", "tcgen05"])


@KINDS
@pytest.mark.parametrize("extra,qmax,gs", [(LAYER, 12.0, 36), (SOLVENT, 9.0, 30), (LAYER, 5.0, 40)])
def test_moments_kernel_grid_matches_oracle(harmonic, kind, extra, qmax, gs):
    amp = globule(1500, 3.0, seed=171, extra=extra)
    amp.xyz = amp.xyz + np.array([0.4, -0.3, 0.2])
    v, _ = _fill(harmonic, amp, qmax, gs, kind)
    ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)
    assert rel_to_max(v, ref) <= 2e-6


@KINDS
@pytest.mark.parametrize("extra,qmax,gs", [(LAYER, 12.0, 36), (LAYER, 4.0, 24), (SOLVENT, 15.0, 40)])
def test_moments_kernel_agrees_with_tf32(harmonic, kind, extra, qmax, gs):
    amp = globule(2000, 2.8, seed=172, extra=extra)
    tc, dtc = _fill(harmonic, amp, qmax, gs, kind)
    mm, dmm = _fill(harmonic, amp, qmax, gs, _lib.DPX_MOMENTS_MMA_SYNC)
    assert rel_to_max(tc, mm) <= 1e-6
    assert rel_to_max(dtc, dmm) <= 1e-5


@KINDS
def test_moments_kernel_intensity_matches_fp64(harmonic, kind):
    amp = globule(2500, 3.0, seed=173, extra=LAYER)
    gs, qmax = 50, 10.0
    Q = np.linspace(0.0, qmax, 51)
    dirs = M.mc_directions(174, 3000)
    I = {}
    with moments_kernel(kind):
        for prec in (M.FP32, M.FP64):
            amp._grid = None
            I[prec] = M.DomainModel([amp], gs, qmax, prec).CalculateIntensityVector(harmonic, Q, 0.0, len(dirs), dirs)
    amp._grid = None
    assert rel(I[M.FP32], I[M.FP64]) <= 1e-4


@KINDS
def test_moments_kernel_in_a_batch_equals_single_fills(harmonic, kind):
    """A batch of leaves of different sizes and orders: one moments launch over
    the job table gives each leaf the grid its own fill gives, bit for bit."""
    leaves = [globule(700, 2.4, seed=175, extra=LAYER), globule(300, 1.0, seed=176, extra=SOLVENT),
              globule(1100, 3.1, seed=177, extra=LAYER)]
    qmax, gs = 8.0, 28
    with moments_kernel(kind):
        for a in leaves:
            a._grid = None
        batch = [g.read(True, True) for g in M.calculate_grids(harmonic, leaves, qmax, gs, M.FP32)]
        single = []
        for a in leaves:
            a._grid = None
            single.append(a.calculateGrid(harmonic, qmax, gs, M.FP32).read(True, True))
            a._grid = None
    for (bv, bd), (sv, sd) in zip(batch, single):
        assert np.array_equal(bv, sv) and np.array_equal(bd, sd)


def test_tcgen05_issue_calibration(ctx):
    """dpx_measure_tcgen05_issue: 32 MMAs (M = 128) from one thread take longer
    at N = 256 than at N = 16, and neither is free (the N = 256 MMA carries 16x
    the work; the small one is bound by its issue)."""
    c = np.zeros(2)
    _lib.check(_lib.lib().dpx_measure_tcgen05_issue(ctx.handle, _lib.dptr(c)))
    assert 1.0 < c[0] <= c[1] < 1e5
