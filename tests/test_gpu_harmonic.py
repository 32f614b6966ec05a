"""GPU parity of the harmonic (multipole) FP32 fill against the FP64 oracle's
direct sum, through the C-ABI (dpx_ctx_set_fill_method).

Tolerances: grid amplitudes within 2e-6 of the largest amplitude (the FP32
bound of the direct fill); I(q) within 1e-4 of the plain FP64 path.
"""
import numpy as np
import pytest

import oracle as O
from dpx import _lib
from dpx import models as M
from helpers import LAYER, SOLVENT, VACUUM, globule, rel, rel_to_max

pytestmark = pytest.mark.gpu
TOL32 = 1e-4


@pytest.fixture
def harmonic(ctx):
    before = ctx.fill_method()
    ctx.set_fill_method(_lib.DPX_FILL_HARMONIC)
    yield ctx
    ctx.set_fill_method(before)


@pytest.mark.parametrize("extra,centered", [(VACUUM, False), (SOLVENT, True), (SOLVENT, False), (LAYER, False)])
def test_harmonic_grid_matches_oracle(harmonic, extra, centered):
    amp = globule(1200, 2.0, seed=141, extra=extra, centered=centered)
    if not centered:
        amp.xyz = amp.xyz + np.array([0.7, -1.1, 2.3])  # off-centre leaf: the centring phase is exercised
    gs, qmax = 40, 5.0
    g = amp.calculateGrid(harmonic, qmax, gs, M.FP32)
    v, _ = g.read(True, False)
    ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)
    assert rel_to_max(v, ref) <= 2e-6


@pytest.mark.parametrize("extra", [SOLVENT, LAYER])
def test_harmonic_intensity_matches_fp64(harmonic, extra):
    amp = globule(2500, 2.6, seed=142, extra=extra)
    gs, qmax = 60, 6.0
    Q = np.linspace(0.0, qmax, 61)
    dirs = M.mc_directions(143, 3000)
    I = {}
    for prec in (M.FP32, M.FP64):
        amp._grid = None
        I[prec] = M.DomainModel([amp], gs, qmax, prec).CalculateIntensityVector(harmonic, Q, 0.0, len(dirs), dirs)
    amp._grid = None
    assert rel(I[M.FP32], I[M.FP64]) <= TOL32


def test_harmonic_and_direct_fill_agree_in_a_batch(ctx):
    """A batch mixing leaves (one with solvent boxes, two grid sizes): the
    harmonic grids equal the direct FP32 grids within the FP32 bound."""
    leaves = [globule(900, 1.7, seed=144, extra=LAYER), globule(300, 1.0, seed=145, extra=VACUUM)]
    qmax = 4.0
    got = {}
    before = ctx.fill_method()
    for method in (_lib.DPX_FILL_DIRECT, _lib.DPX_FILL_HARMONIC):
        ctx.set_fill_method(method)
        for a in leaves:
            a._grid = None
        got[method] = [g.read(True, False)[0] for g in M.calculate_grids(ctx, leaves, qmax, 30, M.FP32)]
    ctx.set_fill_method(before)
    for x, y in zip(got[_lib.DPX_FILL_DIRECT], got[_lib.DPX_FILL_HARMONIC]):
        assert rel_to_max(y, x) <= 2e-6


@pytest.mark.parametrize("extra,gs", [(LAYER, 40), (SOLVENT, 12)])
def test_harmonic_fill_writes_the_spline_pass_derivatives(harmonic, extra, gs):
    """The synthesis writes each row's phi-spline derivatives with its values
    (and their conjugates on the Friedel mirror row): bit for bit those of the
    spline pass, long rows and the short rows of the exact periodic kernel
    (grid_size 12: shells 1-5 have rows of 30 cells or fewer)."""
    amp = globule(800, 1.6, seed=146, extra=extra)
    amp.xyz = amp.xyz + np.array([0.3, -0.2, 0.5])
    g = amp.calculateGrid(harmonic, 4.0, gs, M.FP32)
    g.compute_splines()  # a no-op: the fill wrote them
    v0, d0 = g.read(True, True)
    _ = g.device_ptr  # handing out the pointer clears the flag: the pass recomputes
    g.compute_splines()
    v1, d1 = g.read(True, True)
    assert np.array_equal(v0, v1)
    assert np.array_equal(d0, d1)
    assert np.abs(d0).max() > 0


def test_grid_write_clears_the_fill_derivatives(harmonic):
    """A write after a harmonic fill: compute_splines derives the new values."""
    amp = globule(500, 1.4, seed=147, extra=VACUUM)
    g = amp.calculateGrid(harmonic, 4.0, 30, M.FP32)
    v, _ = g.read(True, False)
    g.write(2.0 * v)
    g.compute_splines()
    _, d2 = g.read(False, True)
    ref = M.Grid(harmonic, 30, 4.0, M.FP32)
    ref.write(2.0 * v)
    ref.compute_splines()
    _, dr = ref.read(False, True)
    assert np.array_equal(d2, dr)


def _leaf(grid, desc):
    import ctypes as C
    import dpx
    h = C.c_void_p()
    _lib.check(dpx.lib().dpx_leaf_create(grid.handle, desc, C.byref(h)))
    return h


@pytest.mark.parametrize("method,prec", [(_lib.DPX_FILL_HARMONIC, M.FP32), (_lib.DPX_FILL_DIRECT, M.FP32),
                                         (_lib.DPX_FILL_HARMONIC, M.FP64)])
@pytest.mark.parametrize("extra", [LAYER, SOLVENT])
def test_prepared_leaf_fill_equals_batch_fill(ctx, method, prec, extra):
    """dpx_leaf_fill (planned once, queue-only fills) writes the same bits as
    dpx_grid_fill_pdb_batch, for host atoms and for centred device atoms, and
    again on a second fill."""
    import ctypes as C
    import dpx
    import torch
    L = dpx.lib()
    amp = globule(900, 1.7, seed=148, extra=extra)
    gs, qmax = 30, 4.0
    before = ctx.fill_method()
    ctx.set_fill_method(method)
    try:
        ref = M.Grid(ctx, gs, qmax, prec)
        descs, keep = M.pdb_descs([amp])
        _lib.check(L.dpx_grid_fill_pdb_batch(1, (C.c_void_p * 1)(ref.handle.value), descs))
        ref.compute_splines()
        v0, d0 = ref.read(True, True)
        g = M.Grid(ctx, gs, qmax, prec)
        leaf = _leaf(g, descs)
        for _ in range(2):
            _lib.check(L.dpx_leaf_fill(leaf))
            g.compute_splines()
            v, d = g.read(True, True)
            assert np.array_equal(v, v0) and np.array_equal(d, d0)
        harm = C.c_int()
        _lib.check(L.dpx_leaf_info(leaf, C.byref(harm), None, None))
        assert harm.value == (1 if method == _lib.DPX_FILL_HARMONIC and prec == M.FP32 else 0)
        _lib.check(L.dpx_leaf_destroy(leaf))
        if prec == M.FP32:  # device atoms, centred by the caller
            cen = amp.xyz.mean(0)
            at = amp.atoms_float4()
            at[:, :3] = (amp.xyz - cen).astype(np.float32)
            d_at = torch.from_numpy(at).cuda()
            c = np.ascontiguousarray(cen)
            descs[0].atoms, descs[0].atoms_on_device, descs[0].center = d_at.data_ptr(), 1, _lib.dptr(c)
            _lib.check(L.dpx_grid_fill_pdb_batch(1, (C.c_void_p * 1)(ref.handle.value), descs))
            ref.compute_splines()
            v1, _ = ref.read(True, False)
            leaf = _leaf(g, descs)
            _lib.check(L.dpx_leaf_fill(leaf))
            v2, _ = g.read(True, False)
            assert np.array_equal(v1, v2)
            assert rel_to_max(v2, v0) <= 2e-6
            _lib.check(L.dpx_leaf_destroy(leaf))
        del keep
    finally:
        ctx.set_fill_method(before)


def test_prepared_leaf_fill_replays_in_a_cuda_graph(harmonic):
    """A stream capture records dpx_leaf_fill (side stream joined back by
    events); replaying the graph refills the grid with the same bits."""
    import ctypes as C
    import dpx
    import torch
    L = dpx.lib()
    amp = globule(700, 1.6, seed=149, extra=LAYER)
    g = M.Grid(harmonic, 30, 4.0, M.FP32)
    descs, keep = M.pdb_descs([amp])
    leaf = _leaf(g, descs)
    _lib.check(L.dpx_leaf_fill(leaf))
    harmonic.synchronize()
    v0, d0 = g.read(True, True)
    s = torch.cuda.Stream()
    old = C.c_void_p(L.dpx_ctx_get_stream(harmonic.handle))
    harmonic.set_stream(s.cuda_stream)
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            _lib.check(L.dpx_leaf_fill(leaf))
        g.write(np.zeros_like(v0))  # the replay must write every cell again
        graph.replay()
        torch.cuda.synchronize()
    finally:
        harmonic.set_stream(old.value)
    v1, d1 = g.read(True, True)
    assert np.array_equal(v1, v0) and np.array_equal(d1, d0)
    _lib.check(L.dpx_leaf_destroy(leaf))
    del keep


def test_pipe_calibration_is_plausible(ctx):
    """dpx_measure_pipe_peaks: the FP32 FMA pipe (scalar and f32x2) within a
    factor of two of 152 SMs x 128 lanes x 2 flops at 1.0-2.1 GHz, and the TF32
    and FP16 mma.sync paths measured."""
    import dpx
    p = np.zeros(4)
    _lib.check(dpx.lib().dpx_measure_pipe_peaks(ctx.handle, _lib.dptr(p)))
    nominal_lo, nominal_hi = 152 * 128 * 2 * 1.0e9, 152 * 128 * 2 * 2.1e9
    for v in p[:2]:
        assert nominal_lo / 2 <= v <= nominal_hi * 2
    assert p[2] > 1e12 and p[3] > 1e12
