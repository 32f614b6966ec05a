"""GPU parity: libdpx kernels (through the C-ABI) against the CPU oracle.

Tolerances (stated per test):
* plain FP64 path           <= 1e-10 relative to the FP64 oracle
* FP32-bulk path            <= 1e-4 relative I(q) error against the FP64 oracle
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle as O
import dpx
from dpx import _lib
from dpx import models as M
from helpers import BOXES5, LAYER, SOLVENT, VACUUM, fill_method, globule, oracle_grid, rel, rel_to_max

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")

TOL64 = 1e-10
TOL32 = 1e-4


@pytest.mark.parametrize("extra", [VACUUM, SOLVENT])
def test_grid_fill_fp64_matches_oracle(ctx, extra):
    amp = globule(300, 1.2, seed=1, extra=extra)
    gs, qmax = 24, 6.0
    g = M.Grid(ctx, gs, qmax, M.FP64)
    a = amp.atoms_float4()
    _lib.check(dpx.lib().dpx_grid_fill_pdb(g.handle, len(a), a.ctypes.data_as(C.c_void_p), 0, len(amp.unique),
                                           _lib.iptr(amp.atoms_per_ion), _lib.dptr(amp.coeffs),
                                           _lib.dptr(amp.ion_rads), amp.flags, amp.solventED, amp.c1, amp.scale,
                                           None))
    v, _ = g.read(True, False)
    ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)
    assert rel_to_max(v, ref) <= TOL64


@pytest.mark.parametrize("extra", [VACUUM, SOLVENT])
def test_grid_fill_fp32_matches_oracle(ctx, extra):
    amp = globule(2000, 2.5, seed=2, extra=extra)
    gs, qmax = 40, 5.0
    g = amp.calculateGrid(ctx, qmax, gs, M.FP32)
    v, _ = g.read(True, False)
    ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)
    # amplitude error relative to the grid's largest amplitude
    assert rel_to_max(v, ref) <= 2e-6


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, 2e-6)])
def test_splines_match_oracle(ctx, prec, tol):
    amp = globule(200, 1.0, seed=3)
    gs, qmax = 60, 5.0
    ref_v, _ = oracle_grid(amp, gs, qmax)
    g = M.Grid(ctx, gs, qmax, prec)
    g.write(ref_v)
    g.compute_splines()
    v, d = g.read()
    ref_d = O.grid_splines(gs, v, O.FP64)
    # derivatives enter the Hermite interpolation next to the values: bound the
    # error on the amplitude scale (FP32 storage rounds y at 6e-8 |y|)
    assert np.max(np.abs(d - ref_d)) <= tol * np.max(np.abs(v))


def _avg(ctx, amp, gs, qmax, Q, dirs, prec, eps=0.0, stride=0, n=None):
    dom = M.DomainModel([amp], gs, qmax, prec)
    return dom.CalculateIntensityVector(ctx, Q, eps, n or (len(dirs) if stride == 0 else stride), dirs, stride)


@pytest.mark.parametrize("Q", [np.linspace(0, 5, 200), np.linspace(0.37, 4.9, 57)])
def test_intensity_fp64_matches_oracle(ctx, Q):
    """Config-0 shape in miniature: grid fill + splines + MC between layers."""
    amp = globule(400, 1.5, seed=4)
    gs, qmax = 40, 5.0
    dirs = M.mc_directions(17, 700)
    I = _avg(ctx, amp, gs, qmax, Q, dirs, M.FP64)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 0.0)
    assert rel(I, ref) <= TOL64


def test_intensity_fp32_matches_fp64_oracle(ctx):
    amp = globule(2000, 2.5, seed=5)
    gs, qmax = 120, 5.0
    Q = np.linspace(0, 5, 200)
    dirs = M.mc_directions(19, 2000)
    I = _avg(ctx, amp, gs, qmax, Q, dirs, M.FP32)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 0.0)
    assert rel(I, ref) <= TOL32


def test_per_layer_direction_streams(ctx):
    """Each bracket draws its own mt19937 stream from the injected master seed."""
    amp = globule(150, 1.0, seed=6)
    gs, qmax = 20, 4.0
    Q = np.linspace(0, 4, 50)
    D = 300
    dirs = M.layer_directions(2024, len(Q), gs // 2, D)
    I = _avg(ctx, amp, gs, qmax, Q, dirs.reshape(-1, 2), M.FP64, stride=D)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs.reshape(-1, 2), D, D, 0.0)
    assert rel(I, ref) <= TOL64


def test_convergence_rule_matches_oracle(ctx):
    amp = globule(100, 0.8, seed=7)
    gs, qmax = 20, 4.0
    Q = np.linspace(0, 4, 60)
    dirs = M.mc_directions(23, 5000)
    I = _avg(ctx, amp, gs, qmax, Q, dirs, M.FP64, eps=1e-3)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 1e-3)
    assert rel(I, ref) <= TOL64


def test_placed_leaf_rotation_translation(ctx):
    amp = globule(200, 1.0, seed=8)
    amp.location = (0.5, -1.0, 2.0, 0.3, -0.7, 1.9)
    gs, qmax = 30, 5.0
    Q = np.linspace(0, 5, 80)
    dirs = M.mc_directions(29, 500)
    I = _avg(ctx, amp, gs, qmax, Q, dirs, M.FP64)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co, rot=amp.location[3:], tr=amp.location[:3])], Q, dirs,
                             0, len(dirs), 0.0)
    assert rel(I, ref) <= TOL64


@pytest.mark.parametrize("dpt", [1, 2])
def test_fp32_slide_average_matches_oracle(ctx, dpt):
    """The FP32 average of one undocked leaf over a shared direction set (the
    plane window with the radial weight table), at one and two directions per
    thread: a plain leaf with an odd chunk count (the two-direction blocks'
    last chunk runs past the samples), a placed leaf, q sets whose brackets
    skip one and two planes (the window's shifts by 2 and 3), and eps > 0
    (chunks of 100 samples)."""
    amp = globule(600, 1.6, seed=81, extra=SOLVENT)
    gs, qmax = 48, 5.0
    data, co = oracle_grid(amp, gs, qmax)
    dirs = M.mc_directions(83, 128 * 7 + 45)
    cases = [(np.linspace(0, qmax, 157), None, 0.0),
             (np.linspace(0.05, 4.9, 61), (0.4, -0.8, 1.5, 0.3, -0.7, 1.9), 0.0),
             (np.linspace(0.02, 4.95, 13), None, 0.0),
             (np.concatenate([np.linspace(0.1, 1.0, 4), np.linspace(1.3, 4.8, 7)]), None, 0.0),
             (np.linspace(0.1, 4.9, 90), None, 2e-3)]
    try:
        M.set_average_shape(dpt)
        for Q, loc, eps in cases:
            amp.location = loc or (0, 0, 0, 0, 0, 0)
            I = _avg(ctx, amp, gs, qmax, Q, dirs, M.FP32, eps=eps)
            leaf = O.make_leaf(data, co) if loc is None else O.make_leaf(data, co, rot=loc[3:], tr=loc[:3])
            ref = O.integrate_layers(gs, qmax, [leaf], Q, dirs, 0, len(dirs), eps)
            assert rel(I, ref) <= TOL32, (len(Q), loc, eps)
    finally:
        M.set_average_shape(1)
        amp.location = (0, 0, 0, 0, 0, 0)


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, TOL32)])
def test_docked_sum_matches_oracle(ctx, prec, tol):
    """ManualSymmetry docked copies (hybrid per-orientation sum), incl. two
    copies sharing a rotation."""
    amp = globule(300, 1.2, seed=9)
    rows = [[0, 0, 0, 0, 0, 0], [3.0, 0, 0, 0, 0, 90], [0, 4.0, 1.0, 45, 30, 10], [-2.0, 1.0, 0, 45, 30, 10],
            [5.0, 5.0, 5.0, 120, -60, 33]]
    sym = M.ManualSymmetry(amp, rows, scale=0.7)
    gs, qmax = 40, 4.0
    Q = np.linspace(0, 4, 90)
    dirs = M.mc_directions(31, 800)
    dom = M.DomainModel([sym], gs, qmax, prec)
    I = dom.CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    data, co = oracle_grid(amp, gs, qmax)
    keep = []
    leaf = O.make_leaf(data, co, copy_rot=sym.rot, copy_tr=sym.trans, sym_scale=0.7, keep=keep)
    ref = O.integrate_layers(gs, qmax, [leaf], Q, dirs, 0, len(dirs), 0.0)
    assert rel(I, ref) <= tol


def test_two_leaves_sum(ctx):
    a = globule(150, 1.0, seed=10)
    b = globule(120, 0.9, seed=11, extra=VACUUM)
    b.location = (2.0, 0.0, -1.0, 0.0, 0.5, 0.0)
    gs, qmax = 24, 4.0
    Q = np.linspace(0, 4, 40)
    dirs = M.mc_directions(37, 400)
    dom = M.DomainModel([a, b], gs, qmax, M.FP64)
    I = dom.CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    da, ca = oracle_grid(a, gs, qmax)
    db, cb = oracle_grid(b, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(da, ca), O.make_leaf(db, cb, rot=b.location[3:],
                                                                         tr=b.location[:3])], Q, dirs, 0,
                             len(dirs), 0.0)
    assert rel(I, ref) <= TOL64


@pytest.mark.parametrize("idx", [0, 2, 8, 20])
def test_single_atom_fixtures_on_gpu(ctx, idx):
    with open(os.path.join(GOLD, "single_atom.json")) as f:
        fx = json.load(f)["fixtures"][idx]
    amp = M.PDBAmplitude([fx["ion"]], [[0.1, 0.2, 0.3]], fx["extra"], centered=fx["centered"])
    dirs = M.mc_directions(41, 600)
    ref = np.array(fx["I"])
    for prec in (M.FP64, M.FP32):
        I = _avg(ctx, amp, fx["gridSize"], fx["qMax"], fx["q"], dirs, prec, eps=fx["convergence"], n=600)
        assert np.max(np.abs(np.sqrt(I) - np.sqrt(ref))) <= 2e-6 * np.sqrt(ref.max()), fx["name"]


def test_drop_in_grid_amplitude_entry(ctx):
    """dpx_pdb_jacobian_grid_amplitude with the reference's argument meaning."""
    amp = globule(250, 1.1, seed=12)
    gs, qmax = 20, 5.0
    P = dpx.lib().dpx_grid_cells(gs)
    out = np.zeros(2 * P)
    a = amp.atoms_float4()
    cf = amp.coeffs.astype(np.float32)
    rf = amp.ion_rads.astype(np.float32)
    rc = dpx.lib().dpx_pdb_jacobian_grid_amplitude(P, 3, 6, qmax / (gs // 2), _lib.dptr(out), _lib.fptr(a), len(a),
                                                   len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(cf),
                                                   _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, None, None, 0,
                                                   0.0, None, None, 0, 0.0, amp.scale, M.FP64, None)
    _lib.check(rc)
    s = O.Struct(amp.xyz, amp.atoms_per_ion, cf.astype(np.float64), rf.astype(np.float64), amp.flags,
                 amp.solventED, amp.c1, amp.scale)
    assert rel_to_max(out, O.grid_fill(s, gs, qmax, O.FP64)) <= TOL64
    stop = C.c_int(1)
    assert dpx.lib().dpx_pdb_jacobian_grid_amplitude(P, 3, 6, qmax / (gs // 2), _lib.dptr(out), _lib.fptr(a), len(a),
                                                     len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(cf),
                                                     _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, None, None,
                                                     0, 0.0, None, None, 0, 0.0, amp.scale, M.FP64,
                                                     C.byref(stop)) == -4
    assert dpx.lib().dpx_pdb_jacobian_grid_amplitude(P + 1, 3, 6, 0.5, _lib.dptr(out), _lib.fptr(a), len(a),
                                                     len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(cf),
                                                     _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, None, None,
                                                     0, 0.0, None, None, 0, 0.0, amp.scale, M.FP64, None) == -1


def test_drop_in_mcoa_entry(ctx):
    amp = globule(200, 1.0, seed=13)
    gs, qmax = 20, 4.0
    data, co = oracle_grid(amp, gs, qmax)
    Q = np.linspace(0, 4, 33)
    dirs = M.mc_directions(43, 400)
    out = np.zeros(len(Q))
    P = dpx.lib().dpx_grid_cells(gs)
    _lib.check(dpx.lib().dpx_calc_mcoa_jacob_sphr(P, 3, 6, qmax / (gs // 2), _lib.dptr(data), _lib.dptr(co),
                                                  _lib.dptr(Q), _lib.dptr(out), len(Q), len(dirs), 0.0,
                                                  _lib.dptr(dirs), 0, M.FP64, None))
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 0.0)
    assert rel(out, ref) <= TOL64


def test_errors_are_statuses(ctx):
    amp = globule(50, 0.6, seed=14)
    g = amp.calculateGrid(ctx, 3.0, 10, M.FP32)
    res = np.zeros(3)
    Q = np.array([0.0, 1.0, 5.0])  # beyond qmax
    dirs = M.mc_directions(1, 10)
    h = (C.c_void_p * 1)(g.handle.value)
    rc = dpx.lib().dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, 3, _lib.dptr(Q),
                                           dirs.ctypes.data_as(C.c_void_p), 0, 0, 10, 0.0, _lib.dptr(res))
    assert rc == -1 and b"beyond" in dpx.lib().dpx_last_error()
    Q = np.array([1.0, 0.5])  # not ascending
    rc = dpx.lib().dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, 2, _lib.dptr(Q),
                                           dirs.ctypes.data_as(C.c_void_p), 0, 0, 10, 0.0, _lib.dptr(res))
    assert rc == -1


def test_grid_reuse_is_device_resident(ctx):
    amp = globule(100, 0.8, seed=15)
    g1 = amp.calculateGrid(ctx, 3.0, 12, M.FP32)
    g2 = amp.calculateGrid(ctx, 3.0, 12, M.FP32)
    assert g1 is g2
    amp.set_extra([2, 333, 1, 0.05, 0.14, 0.28, 0, 0, 0, 4])
    g3 = amp.calculateGrid(ctx, 3.0, 12, M.FP32)
    assert g3 is not g1


@pytest.mark.parametrize("prec,tol,docked", [(M.FP64, TOL64, False), (M.FP32, TOL32, False), (M.FP64, TOL64, True),
                                             (M.FP32, TOL32, True)])
def test_vegas_matches_oracle(ctx, prec, tol, docked):
    """VEGAS: same points (keyed counter stream), same bin refinement carried
    across brackets, same running mean and convergence test as the restatement."""
    amp = globule(250, 1.1, seed=21)
    gs, qmax = 24, 4.0
    Q = np.linspace(0, 4, 37)
    if docked:
        rows = [[0, 0, 0, 0, 0, 0], [2.5, 0, 0, 0, 0, 90], [0, 3.0, 1.0, 45, 30, 10]]
        model = M.ManualSymmetry(amp, rows, scale=1.3)
    else:
        model = amp
    dom = M.DomainModel([model], gs, qmax, prec)
    I = dom.CalculateIntensityVector(ctx, Q, 1e-3, 6 * 2048, method="VEGAS", seed=99, points_per_iter=2048)
    data, co = oracle_grid(amp, gs, qmax)
    keep = []
    if docked:
        leaf = O.make_leaf(data, co, copy_rot=model.rot, copy_tr=model.trans, sym_scale=1.3, keep=keep)
    else:
        leaf = O.make_leaf(data, co)
    ref = O.vegas_intensity(gs, qmax, [leaf], Q, 99, 2048, 6 * 2048, 1e-3)
    assert rel(I, ref) <= tol


@pytest.mark.parametrize("prec,tol,docked", [(M.FP64, TOL64, False), (M.FP32, TOL32, False), (M.FP64, TOL64, True)])
def test_gauss_kronrod_matches_oracle(ctx, prec, tol, docked):
    """Adaptive GK 7/15: same rule, same acceptance test and depth budget as the
    recursion of DomainModel::GaussLegTheta / GaussLegPhi."""
    amp = globule(150, 0.9, seed=23)
    amp.location = (0.3, -0.2, 0.5, 0.2, 0.4, -0.3)
    gs, qmax = 20, 4.0
    Q = np.array([0.0, 0.45, 1.3, 2.2, 3.9])
    if docked:
        model = M.ManualSymmetry(amp, [[0, 0, 0, 0, 0, 0], [2.0, 0.5, 0, 30, 0, 60]], scale=0.8)
    else:
        model = amp
    dom = M.DomainModel([model], gs, qmax, prec)
    I = dom.CalculateIntensityVector(ctx, Q, 1e-3, 6, method="GK")
    data, co = oracle_grid(amp, gs, qmax)
    keep = []
    kw = dict(rot=amp.location[3:], tr=amp.location[:3], keep=keep)
    leaf = O.make_leaf(data, co, copy_rot=model.rot, copy_tr=model.trans, sym_scale=0.8, **kw) if docked \
        else O.make_leaf(data, co, **kw)
    ref = np.array([O.gk_intensity(gs, qmax, [leaf], q, 1e-3, 6) for q in Q])
    assert rel(I, ref) <= tol


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, 2e-6)])
def test_assembly_grid_matches_oracle(ctx, prec, tol):
    """Grid-path ManualSymmetry: the assembled grid cell by cell (tolerance on the
    amplitude scale), then its MC average."""
    amp = globule(200, 1.0, seed=24)
    amp.location = (0.2, 0.1, -0.3, 0.1, 0.2, 0.3)
    rows = [[0, 0, 0, 0, 0, 0], [2.0, 0, 0, 0, 0, 90], [0, 2.5, 0.5, 45, 30, 10], [-1.5, 1.0, 0, 45, 30, 10]]
    sym = M.ManualSymmetry(amp, rows, scale=0.9, use_grid=True)
    gs, qmax = 24, 4.0
    g = sym.calculateGrid(ctx, qmax, gs, prec)
    v, _ = g.read(True, False)
    data, co = oracle_grid(amp, gs, qmax)
    keep = []
    leaf = O.make_leaf(data, co, rot=amp.location[3:], tr=amp.location[:3], copy_rot=sym.rot, copy_tr=sym.trans,
                       sym_scale=0.9, keep=keep)
    ref = O.assemble_grid(gs, qmax, [leaf])
    assert np.max(np.abs(v - ref)) <= tol * np.max(np.abs(ref))
    if prec == M.FP64:
        Q = np.linspace(0, 4, 41)
        dirs = M.mc_directions(51, 400)
        I = M.DomainModel([sym], gs, qmax, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
        rco = O.grid_splines(gs, ref, O.FP64)
        refI = O.integrate_layers(gs, qmax, [O.make_leaf(ref, rco)], Q, dirs, 0, len(dirs), 0.0)
        assert rel(I, refI) <= TOL64


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, 2e-6)])
def test_space_filling_grid_matches_oracle(ctx, prec, tol):
    amp = globule(120, 0.8, seed=25)
    sf = M.SpaceFillingSymmetry([amp], 3.0, 3.5, 4.0, 90, 80, 100, 3, 2, 4, scale=0.5)
    gs, qmax = 20, 3.0
    g = sf.calculateGrid(ctx, qmax, gs, prec)
    v, _ = g.read(True, False)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.assemble_grid(gs, qmax, [O.make_leaf(data, co)], lattice=sf.lattice, scale=0.5)
    assert np.max(np.abs(v - ref)) <= tol * np.max(np.abs(ref))


def test_vegas_rejects_bad_point_counts(ctx):
    amp = globule(50, 0.6, seed=22)
    dom = M.DomainModel([amp], 10, 3.0, M.FP32)
    with pytest.raises(dpx.DpxError):
        dom.CalculateIntensityVector(ctx, np.linspace(0, 3, 5), 0.0, 5000, method="VEGAS", points_per_iter=1000)


def test_batched_fill_equals_single_fills(ctx):
    """dpx_grid_fill_pdb_batch: one persistent FP32 launch over several leaves
    gives bit-identical cells to one call per leaf; FP64 leaves in the same
    batch match the oracle."""
    gs, qmax = 30, 5.0
    leaves = [globule(900, 2.0, seed=41, extra=VACUUM), globule(150, 1.0, seed=42, extra=SOLVENT),
              globule(2500, 2.6, seed=43, extra=SOLVENT), globule(300, 1.2, seed=44, extra=VACUUM)]
    precs = [M.FP32, M.FP32, M.FP32, M.FP64]
    singles = []
    for amp, p in zip(leaves, precs):
        g = M.Grid(ctx, gs, qmax, p)
        a = amp.atoms_float4()
        _lib.check(dpx.lib().dpx_grid_fill_pdb(g.handle, len(a), a.ctypes.data_as(C.c_void_p), 0, len(amp.unique),
                                               _lib.iptr(amp.atoms_per_ion), _lib.dptr(amp.coeffs),
                                               _lib.dptr(amp.ion_rads), amp.flags, amp.solventED, amp.c1,
                                               amp.scale, None))
        singles.append(g.read(True, False)[0])
    grids = [M.Grid(ctx, gs, qmax, p) for p in precs]
    descs = (_lib.PdbDesc * len(leaves))()
    keep = []
    for d, amp in zip(descs, leaves):
        a = amp.atoms_float4()
        keep.append(a)
        d.n_atoms, d.atoms, d.atoms_on_device, d.n_ions = len(a), a.ctypes.data, 0, len(amp.unique)
        d.atoms_per_ion, d.coeffs, d.ion_rads = _lib.iptr(amp.atoms_per_ion), _lib.dptr(amp.coeffs), \
            _lib.dptr(amp.ion_rads)
        d.flags, d.solvent_ed, d.c1, d.scale, d.center = amp.flags, amp.solventED, amp.c1, amp.scale, None
    handles = (C.c_void_p * len(grids))(*[g.handle.value for g in grids])
    _lib.check(dpx.lib().dpx_grid_fill_pdb_batch(len(grids), handles, descs))
    for g, ref in zip(grids, singles):
        assert np.array_equal(g.read(True, False)[0], ref)
    ref64 = O.grid_fill(O.Struct.from_pdb(leaves[3]), gs, qmax, O.FP64)
    assert rel_to_max(singles[3], ref64) <= TOL64
    # the same grid twice in one batch is refused
    dup = (C.c_void_p * 2)(grids[0].handle.value, grids[0].handle.value)
    assert dpx.lib().dpx_grid_fill_pdb_batch(2, dup, descs) == -1


def test_domain_model_batches_leaf_fills(ctx):
    """DomainModel fills all missing leaf grids in one batch; I(q) equals the
    one-leaf-at-a-time result exactly."""
    gs, qmax = 24, 4.0
    Q = np.linspace(0.1, 3.9, 40)
    dirs = M.mc_directions(5, 300)
    def mk():
        a, b = globule(400, 1.4, seed=51, extra=VACUUM), globule(250, 1.1, seed=52, extra=SOLVENT)
        a.location, b.location = (0.5, 0, 0, 0.2, 0, 0), (-0.5, 0.3, 0, 0, 0.4, 0.1)
        return [a, b]
    a1 = mk()
    for a in a1:  # one fill per leaf
        a.calculateGrid(ctx, qmax, gs, M.FP32)
    I1 = M.DomainModel(a1, gs, qmax, M.FP32).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    a2 = mk()
    I2 = M.DomainModel(a2, gs, qmax, M.FP32).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    assert np.array_equal(I1, I2)


def _cell_qvectors(gs, qmax):
    """q vectors of every cell in grid-index order (Grid.cpp:169-200 layout)."""
    Lp, step = gs // 2 + 3, qmax / (gs // 2)
    out = [np.zeros((1, 3))]
    for i in range(1, Lp + 1):
        t, p = np.meshgrid(np.arange(3 * i + 1), np.arange(6 * i), indexing="ij")
        th, ph = np.pi * t / (3 * i), np.pi * p / (3 * i)
        q = i * step
        out.append(np.stack([q * np.sin(th) * np.cos(ph), q * np.sin(th) * np.sin(ph), q * np.cos(th)],
                            -1).reshape(-1, 3))
    return np.concatenate(out)


def test_dropin_manual_symmetry_grid(ctx):
    """dpx_calc_man_sym_jacob_sphr: host buffers, loc arrays with the inner
    placement at entry 0, outData accumulated."""
    amp = globule(150, 0.9, seed=61)
    gs, qmax = 20, 3.0
    data, co = oracle_grid(amp, gs, qmax)
    P = len(data) // 2
    rng = np.random.default_rng(3)
    loc = rng.uniform(-1.5, 1.5, (6, 4))  # x, y, z, a, b, c; 1 inner + 3 copies
    loc[3:] = rng.uniform(0, 2 * np.pi, (3, 4))
    loc[3:, 3] = loc[3:, 2]  # two copies share a rotation
    out = rng.normal(size=2 * P)
    out0 = out.copy()
    rc = dpx.lib().dpx_calc_man_sym_jacob_sphr(P, 3, 6, 3, qmax / (gs // 2), _lib.dptr(data), _lib.dptr(out),
                                               _lib.dptr(co), *[_lib.dptr(np.ascontiguousarray(r)) for r in loc],
                                               0.8, M.FP64, None)
    _lib.check(rc)
    keep = []
    leaf = O.make_leaf(data, co, rot=loc[3:, 0], tr=loc[:3, 0], copy_rot=loc[3:, 1:].T.copy(),
                       copy_tr=loc[:3, 1:].T.copy(), sym_scale=0.8, keep=keep)
    ref = O.assemble_grid(gs, qmax, [leaf])
    assert np.max(np.abs(out - out0 - ref)) <= TOL64 * np.max(np.abs(ref))


def test_dropin_space_filling_grid(ctx):
    """dpx_calc_spc_fill_sym_jacob_sphr reproduces SymmetryGenJacob.cu's lattice
    sum sin(N x/2)/sin(x/2) e^{-i (N-1) x/2} (restated here in numpy)."""
    amp = globule(120, 0.8, seed=62)
    gs, qmax = 18, 3.0
    data, co = oracle_grid(amp, gs, qmax)
    P = len(data) // 2
    vm = np.array([3.0, 0.0, 0.0, 0.4, 3.5, 0.0, 0.2, -0.3, 4.0])
    reps = np.array([3.0, 2.0, 4.0])
    irot, itr = np.array([0.3, -0.2, 0.5]), np.array([0.4, 0.1, -0.2])
    out = np.random.default_rng(4).normal(size=2 * P)
    out0 = out.copy()
    _lib.check(dpx.lib().dpx_calc_spc_fill_sym_jacob_sphr(P, 3, 6, qmax / (gs // 2), _lib.dptr(data),
                                                          _lib.dptr(out), _lib.dptr(co), _lib.dptr(vm),
                                                          _lib.dptr(reps), _lib.dptr(irot), _lib.dptr(itr), 0.6,
                                                          M.FP64, None))
    child = O.assemble_grid(gs, qmax, [O.make_leaf(data, co, rot=irot, tr=itr)])
    A = child[0::2] + 1j * child[1::2]
    qv = _cell_qvectors(gs, qmax)
    for k in range(3):
        x, N = qv @ vm[3 * k:3 * k + 3], reps[k]
        small = np.abs(x) < 100 * np.finfo(float).eps
        xs = np.where(small, 1.0, x)
        S = np.sin(N * xs / 2) / np.sin(xs / 2) * np.exp(-0.5j * (N - 1) * xs)
        A = A * np.where(small | (N == 1), N, S)
    got = (out - out0)[0::2] + 1j * (out - out0)[1::2]
    assert np.max(np.abs(got - 0.6 * A)) <= 1e-9 * np.max(np.abs(A))


def test_dropin_sum_grids(ctx):
    """dpx_sum_grids_jacob_sphr overwrites its output with the sum of the placed grids."""
    gs, qmax = 18, 3.0
    a, b = globule(100, 0.8, seed=63), globule(140, 0.9, seed=64)
    (da, ca), (db, cb) = oracle_grid(a, gs, qmax), oracle_grid(b, gs, qmax)
    P = len(da) // 2
    trans = np.array([0.5, 0.0, 0.2, -0.4, 0.3, 0.0])
    rots = np.array([0.1, 0.2, 0.3, 1.0, -0.5, 2.0])
    out = np.full(2 * P, 7.0)
    amps = (_lib._D * 2)(_lib.dptr(da), _lib.dptr(db))
    ders = (_lib._D * 2)(_lib.dptr(ca), _lib.dptr(cb))
    _lib.check(dpx.lib().dpx_sum_grids_jacob_sphr(P, 3, 6, qmax / (gs // 2), amps, ders, _lib.dptr(trans),
                                                  _lib.dptr(rots), 2, _lib.dptr(out), M.FP64, None))
    keep = []
    ref = O.assemble_grid(gs, qmax, [O.make_leaf(da, ca, rot=rots[:3], tr=trans[:3], keep=keep),
                                     O.make_leaf(db, cb, rot=rots[3:], tr=trans[3:], keep=keep)])
    assert np.max(np.abs(out - ref)) <= TOL64 * np.max(np.abs(ref))


def test_fill_schedules_and_autotuner(ctx):
    """Direct sum: flat and persistent FP32 fills give identical cells for every
    shape; the autotuner keeps one of the swept shapes (or the harmonic method)."""
    ctx.set_fill_method(_lib.DPX_FILL_DIRECT)
    gs, qmax = 26, 4.0
    leaves = [globule(700, 1.8, seed=71, extra=SOLVENT), globule(90, 0.7, seed=72, extra=VACUUM)]
    for cpt, th in [(2, 256), (4, 128), (8, 128), (8, 256)]:
        ctx.set_fill_shape(cpt, th)
        got = []
        for persistent in (False, True):
            ctx.set_fill_schedule(persistent)
            for a in leaves:
                a._grid = None
            got.append([g.read(True, False)[0] for g in M.calculate_grids(ctx, leaves, qmax, gs, M.FP32)])
        for x, y in zip(*got):
            assert np.array_equal(x, y)
    # FMA-pipe columns: flat and persistent identical as well
    for kp in (1, 2, 3):
        ctx.set_fill_shape(8, 128, kp)
        got = []
        for persistent in (False, True):
            ctx.set_fill_schedule(persistent)
            for a in leaves:
                a._grid = None
            got.append([g.read(True, False)[0] for g in M.calculate_grids(ctx, leaves, qmax, gs, M.FP32)])
        for x, y in zip(*got):
            assert np.array_equal(x, y)
    ctx.set_fill_schedule(False)
    best, table = M.autotune_fill(ctx, leaves, qmax, gs, repeats=1)
    assert best in table and len(table) == dpx.lib().dpx_fill_shapes(None)
    assert {(8, 128, 0, k) for k in range(4)} <= set(table) and (0, 0, 0, 0) in table
    if best == (0, 0, 0, 0):
        assert ctx.fill_method() == _lib.DPX_FILL_HARMONIC
    else:
        assert ctx.fill_method() == _lib.DPX_FILL_DIRECT and ctx.fill_shape() == best
    assert all(t > 0 for t in table.values())
    ctx.set_fill_shape(8, 128)
    ctx.set_fill_schedule(False)
    ctx.set_fill_method(_lib.DPX_FILL_HARMONIC)


@pytest.mark.parametrize("kp", [1, 2, 3])
@pytest.mark.parametrize("extra", [SOLVENT, LAYER])
def test_fill_fma_pipe_columns_match_oracle(ctx, kp, extra):
    """Phi columns whose sin/cos run as FMA-pipe polynomials: the grid within
    the FP32 amplitude bound of the FP64 oracle (atoms, and atoms with the
    voxelized layer), and I(q) within 1e-4 of the plain FP64 path."""
    amp = globule(1500, 2.2, seed=90 + kp, extra=extra)
    gs, qmax = 40, 5.0
    ctx.set_fill_method(_lib.DPX_FILL_DIRECT)
    ctx.set_fill_shape(8, 128, kp)
    try:
        g = amp.calculateGrid(ctx, qmax, gs, M.FP32)
        v, _ = g.read(True, False)
        ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)  # atoms and boxes
        assert rel_to_max(v, ref) <= 2e-6
        Q = np.linspace(0.0, qmax, 41)
        dirs = M.mc_directions(91, 2000)
        I = {}
        for prec in (M.FP32, M.FP64):
            amp._grid = None
            I[prec] = M.DomainModel([amp], gs, qmax, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
        assert rel(I[M.FP32], I[M.FP64]) <= TOL32
    finally:
        ctx.set_fill_shape(8, 128, 0)
        ctx.set_fill_method(_lib.DPX_FILL_HARMONIC)
        amp._grid = None


def _batch_case(seed0=80):
    rng = np.random.default_rng(seed0)
    leaves, gss, qms, Qs = [], [], [], []
    for k in range(5):
        n = int(rng.integers(60, 900))
        extra = LAYER if k == 3 else (SOLVENT if k % 2 else VACUUM)
        leaves.append(globule(n, 0.5 + 0.02 * n ** (1 / 3) * 3, seed=seed0 + k, extra=extra))
        gss.append(int(rng.integers(6, 16)) * 2)
        qms.append(float(rng.uniform(2.0, 6.0)))
        lo = 0.0 if k % 2 == 0 else 0.3
        Qs.append(np.linspace(lo, qms[-1], int(rng.integers(20, 60))))
    return leaves, gss, qms, Qs


@pytest.mark.parametrize("prec,method", [(M.FP32, _lib.DPX_FILL_HARMONIC), (M.FP32, _lib.DPX_FILL_DIRECT),
                                         (M.FP64, _lib.DPX_FILL_HARMONIC)])
def test_solve_batch_equals_single_solves(ctx, prec, method):
    """dpx_batch (one graph per wave: the harmonic fills planned at creation,
    or one direct-sum launch per wave) gives the same I(q) as one DomainModel
    solve per structure with the same fill method, also when the grid budget
    splits the batch into several waves; replaying the graphs is stable."""
    leaves, gss, qms, Qs = _batch_case()
    dirs = M.mc_directions(9, 500)
    with fill_method(ctx, method):
        singles = [M.DomainModel([a], gs, qm, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
                   for a, gs, qm, Q in zip(leaves, gss, qms, Qs)]
        for budget in (0, 1):  # 1 byte: every structure is its own wave
            b = M.SolveBatch(ctx, leaves, gss, qms, Qs, dirs, precision=prec, grid_budget_bytes=budget)
            waves, launches, _ = b.info()
            assert waves == (5 if budget == 1 else 1)
            assert launches > 0
            for _ in range(2):
                b.run()
                for r, s in zip(b.results(), singles):
                    assert np.allclose(r, s, rtol=1e-12, atol=0)
            b.close()
    if prec == M.FP64:  # pin one structure to the oracle
        data, co = oracle_grid(leaves[0], gss[0], qms[0])
        ref = O.integrate_layers(gss[0], qms[0], [O.make_leaf(data, co)], Qs[0], dirs, 0, len(dirs), 0.0)
        assert rel(singles[0], ref) <= TOL64


@pytest.mark.parametrize("extra", [LAYER, BOXES5])
@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, 2e-5)])
def test_grid_fill_voxel_solvent_matches_oracle(ctx, extra, prec, tol):
    """Atoms plus voxelized-solvent boxes (solvation layer; excluded volume for
    radius type 5), fused into the fill, against the oracle's FP64 box sum.
    FP32 bound on the amplitude scale: the box terms use the SFU sine and
    divide; the I(q) bar (1e-4) is checked in the next test."""
    amp = globule(250, 1.1, seed=91, extra=extra)
    assert amp.solvent_boxes() is not None and len(amp.solvent_boxes()) > 100
    gs, qmax = 24, 5.0
    g = amp.calculateGrid(ctx, qmax, gs, prec)
    v, _ = g.read(True, False)
    ref = O.grid_fill(O.Struct.from_pdb(amp), gs, qmax, O.FP64)
    assert rel_to_max(v, ref) <= tol


def test_intensity_with_solvation_layer(ctx):
    """I(q) of a leaf with the voxelized layer: FP32 bulk within 1e-4 of the
    FP64 oracle, and the layer changes I(q) by far more than that."""
    amp = globule(300, 1.2, seed=92, extra=LAYER)
    bare = globule(300, 1.2, seed=92, extra=SOLVENT)
    gs, qmax = 30, 4.0
    Q = np.linspace(0.05, 4.0, 60)
    dirs = M.mc_directions(93, 500)
    I = M.DomainModel([amp], gs, qmax, M.FP32).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    I0 = M.DomainModel([bare], gs, qmax, M.FP32).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    data, co = oracle_grid(amp, gs, qmax)
    ref = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, len(dirs), 0.0)
    assert rel(I, ref) <= TOL32
    assert rel(I, I0) > 1e-3


def test_layer_fp32_error_with_many_boxes(ctx):
    """Tens of thousands of solvent boxes add in phase near q = 0: the FP32
    fill keeps per-tile partial sums, so I(q) stays within 1e-4 of the plain
    FP64 path at every q including 0."""
    amp = globule(3000, 2.6, seed=95, extra=LAYER)
    assert len(amp.solvent_boxes()) > 10000
    gs, qmax = 30, 6.0
    Q = np.linspace(0.0, 6.0, 61)
    dirs = M.mc_directions(96, 300)
    I32 = M.DomainModel([amp], gs, qmax, M.FP32).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    amp._grid = None
    I64 = M.DomainModel([amp], gs, qmax, M.FP64).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    assert rel(I32, I64) <= TOL32


def test_drop_in_grid_fill_with_voxel_boxes(ctx):
    """The grid-fill drop-in with the reference's float4 / int4 voxel arrays
    gives the grid of the Python leaf with the same boxes (solvation layer)."""
    amp = globule(250, 1.1, seed=97, extra=LAYER)
    gs, qmax = 22, 4.5
    P = dpx.lib().dpx_grid_cells(gs)
    ec, ed, lc, ld = amp.voxel_boxes()
    com4 = np.zeros((len(lc), 4), dtype=np.float32)
    com4[:, :3] = lc
    dim4 = np.zeros((len(ld), 4), dtype=np.int32)
    dim4[:, :3] = ld
    a = amp.atoms_float4()
    cf = amp.coeffs.astype(np.float32)
    rf = amp.ion_rads.astype(np.float32)
    out = np.zeros(2 * P)
    _lib.check(dpx.lib().dpx_pdb_jacobian_grid_amplitude(P, 3, 6, qmax / (gs // 2), _lib.dptr(out), _lib.fptr(a),
                                                         len(a), len(amp.unique), _lib.iptr(amp.atoms_per_ion),
                                                         _lib.fptr(cf), _lib.fptr(rf), amp.flags, amp.solventED,
                                                         amp.c1, None, None, 0, amp.voxelStep, _lib.fptr(com4),
                                                         _lib.iptr(dim4), len(lc), amp.outerSolventED, amp.scale,
                                                         M.FP64, None))
    s = O.Struct(amp.xyz, amp.atoms_per_ion, cf.astype(np.float64), rf.astype(np.float64), amp.flags,
                 amp.solventED, amp.c1, amp.scale, amp.solvent_boxes())
    assert rel_to_max(out, O.grid_fill(s, gs, qmax, O.FP64)) <= TOL64


def test_helical_assembly_closed_form_phase_sums(ctx):
    """Screw-symmetric helix (13 rotation groups, each an arithmetic
    progression of translations): the FP32 average sums each group's phases in
    closed form and stays within 1e-4 of the plain FP64 path (direct sums);
    a copy list with one translation moved off the progression takes the
    direct FP32 sum and agrees as well."""
    from dpx import workloads as W
    amp = globule(150, 0.9, seed=98, extra=VACUUM)
    rot, trn = W.helix_copies(260, 6.0, 13, 4.0, seed=5)
    rows = np.concatenate([trn, np.degrees(rot)], axis=1)
    gs, qmax = 20, 3.0
    Q = np.linspace(0.0, 3.0, 49)
    dirs = M.mc_directions(99, 400)
    for rr in (rows, rows.copy()):
        if rr is not rows:
            rr[13 * 7, 2] += 1e-3  # breaks the progression of one group
        I = {}
        for prec in (M.FP32, M.FP64):
            sym = M.ManualSymmetry(amp, rr, scale=1.0, use_grid=False)
            I[prec] = M.DomainModel([sym], gs, qmax, prec).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
            amp._grid = None
        assert rel(I[M.FP32], I[M.FP64]) <= TOL32
        assert abs(I[M.FP32][0] / I[M.FP64][0] - 1) < 1e-6  # q = 0: every copy in phase


@pytest.mark.parametrize("ext", [".amp", ".ampj"])
def test_amp_file_round_trip_as_a_leaf(ctx, tmp_path, ext):
    """A grid saved as a D+ amplitude file and loaded as AmpGridAmplitude gives
    the same I(q) as the leaf it came from; its scale multiplies the amplitude;
    the same file read into an FP32 grid stays within the FP32 bound."""
    amp = globule(300, 1.2, seed=111, extra=SOLVENT)
    gs, qmax = 24, 4.0
    Q = np.linspace(0, 4.0, 33)
    dirs = M.mc_directions(112, 300)
    g = amp.calculateGrid(ctx, qmax, gs, M.FP64)
    p = str(tmp_path / ("leaf" + ext))
    if ext == ".amp":
        g.save_amp(p, "dpx test grid")
    else:
        g.save_ampj(p, params=[1, 333], header="dpx test grid")
    I0 = M.DomainModel([amp], gs, qmax, M.FP64).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    leaf = M.AmpGridAmplitude(p)
    assert leaf.header == "dpx test grid"
    I1 = M.DomainModel([leaf], gs, qmax, M.FP64).CalculateIntensityVector(ctx, Q, 0.0, len(dirs), dirs)
    assert rel(I1, I0) <= 1e-12
    I2 = M.DomainModel([M.AmpGridAmplitude(p, scale=2.0)], gs, qmax, M.FP64).CalculateIntensityVector(
        ctx, Q, 0.0, len(dirs), dirs)
    assert rel(I2, 4.0 * I0) <= 1e-12
    I3 = M.DomainModel([M.AmpGridAmplitude(p)], gs, qmax, M.FP32).CalculateIntensityVector(
        ctx, Q, 0.0, len(dirs), dirs)
    assert rel(I3, I0) <= TOL32
    with pytest.raises(ValueError):
        M.DomainModel([M.AmpGridAmplitude(p)], gs + 2, qmax, M.FP64).CalculateIntensityVector(
            ctx, Q, 0.0, len(dirs), dirs)


def test_json_state_runs_end_to_end(ctx, tmp_path):
    """A D+ JSON state (two populations, a manual symmetry of a PDB file, an
    amplitude-file leaf) decoded and run: Scale * sum_p w_p I_p + Constant of
    the same models built by hand."""
    import json
    from dpx import state as S
    amp = globule(120, 0.8, seed=121, extra=VACUUM)
    pdb = tmp_path / "sub.pdb"
    with open(pdb, "w") as f:
        for k, (sym, p) in enumerate(zip(amp.symbols, amp.xyz * 10.0)):
            f.write("ATOM  %5d  %-3s ALA A   1    %8.3f%8.3f%8.3f  1.00  0.00          %2s\n"
                    % (k + 1, sym, p[0], p[1], p[2], sym))
    gs, qmax = 20, 3.0
    g = amp.calculateGrid(ctx, qmax, gs, M.FP64)
    g.save_amp(str(tmp_path / "leaf.amp"))
    loc = {"x": 0, "y": 0, "z": 0, "alpha": 0, "beta": 0, "gamma": 0}
    leaf = {"Type": "PDB", "Filename": "C:\\\\data\\\\sub.pdb", "Centered": False, "Location": loc,
            "ExtraParameters": [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0], "Use_Grid": True}
    rows = [[0, 0, 0, 0, 0, 0], [2.5, 0, 0, 0, 0, 60], [0, 2.5, 1, 30, 20, 10]]
    sym = {"Type": ",26", "Location": loc, "Parameters": rows, "ExtraParameters": [0.8], "Children": [leaf],
           "Use_Grid": False}
    ampnode = {"Type": "AMP", "Filename": "leaf.amp", "Location": dict(loc, x=1.0), "ExtraParameters": [1.5]}
    state = {"DomainPreferences": {"GridSize": gs, "qMax": qmax, "OrientationMethod": "Monte Carlo (Mersenne Twister)",
                                   "OrientationIterations": 300, "Convergence": 0.0, "UseGrid": False},
             "Domain": {"Scale": 2.0, "Constant": 0.25,
                        "Populations": [{"PopulationSize": 1.0, "Models": [sym]},
                                        {"PopulationSize": 0.5, "Models": [ampnode]}]}}
    job = S.decode(json.dumps(state), base_dir=str(tmp_path))
    Q = np.linspace(0, 3.0, 31)
    dirs = M.mc_directions(122, 300)
    I = job.intensity(ctx, Q, dirs, precision=M.FP64)
    syms, xyz = S.read_pdb(str(pdb))  # the coordinates as the PDB file rounds them
    same = M.PDBAmplitude(syms, xyz, [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
    by_hand1 = M.DomainModel([M.ManualSymmetry(same, rows, scale=0.8, use_grid=False)], gs, qmax, M.FP64)
    by_hand2 = M.DomainModel([M.AmpGridAmplitude(str(tmp_path / "leaf.amp"), scale=1.5,
                                                 location=(1.0, 0, 0, 0, 0, 0))], gs, qmax, M.FP64)
    ref = 2.0 * (by_hand1.CalculateIntensityVector(ctx, Q, 0.0, 300, dirs)
                 + 0.5 * by_hand2.CalculateIntensityVector(ctx, Q, 0.0, 300, dirs)) + 0.25
    assert rel(I, ref) <= 1e-9


@pytest.mark.parametrize("idx", [0, 5, 9, 13, 21])
def test_single_atom_states_through_the_decoder(ctx, idx):
    """The reference's single-atom state documents decoded by dpx.state and run
    through the Job: I(q) equals the reference's within its printed digits
    (amplitudes within 2e-6 of the largest), FP64 and FP32 bulk."""
    from dpx import state as S
    with open(os.path.join(GOLD, "single_atom.json")) as f:
        fx = json.load(f)["fixtures"][idx]
    job = S.decode(fx["state"], files={fx["pdb_name"]: fx["pdb_lines"]})
    dirs = M.mc_directions(42, 600)
    ref = np.array(fx["I"])
    for prec in (M.FP64, M.FP32):
        I = job.intensity(ctx, np.array(fx["q"]), dirs=dirs, precision=prec, iterations=600)
        assert np.max(np.abs(np.sqrt(I) - np.sqrt(ref))) <= 2e-6 * np.sqrt(ref.max()), fx["name"]


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, TOL32)])
def test_hybrid_calculator_matches_oracle(ctx, prec, tol):
    """The IGPUGridCalculator drop-in (dpx_hybrid_*): one PDB child with three
    rotations of two translations each, Monte Carlo with the reference GPU
    averages' convergence test, against the oracle's docked sum of the same
    copies over the same seeded directions."""
    amp = globule(300, 1.2, seed=61, extra=SOLVENT)
    gs, qmax = 24, 4.0
    L = dpx.lib()
    P = L.dpx_grid_cells(gs)
    Q = (np.arange(1, 49) / 12.0).astype(np.float32)  # exact in float
    h = C.c_void_p()
    _lib.check(L.dpx_hybrid_create(ctx.handle, len(Q), _lib.fptr(Q), 2 * P, 3, 6, gs // 2 + 4, qmax, qmax / (gs // 2),
                                   prec, C.byref(h)))
    _lib.check(L.dpx_hybrid_set_num_children(h, 1))
    descs, keep = M.pdb_descs([amp])
    _lib.check(L.dpx_hybrid_child_pdb(h, 0, descs))
    rots = np.array([[0.0, 0.0, 0.0, 1.0], [0.3, -0.4, 1.1, 1.0], [1.2, 0.2, -0.7, 1.0]], dtype=np.float32)
    _lib.check(L.dpx_hybrid_add_rotations(h, 0, 3, _lib.fptr(rots)))
    trans = [np.array([[0, 0, 0, 0], [2.5, 0, 0, 0]], dtype=np.float32),
             np.array([[0, 1.5, 0.5, 0], [-1, -1, 2, 0]], dtype=np.float32),
             np.array([[0.5, 0.5, -2, 0], [3, 0, 1, 0]], dtype=np.float32)]
    for r, t in enumerate(trans):
        _lib.check(L.dpx_hybrid_add_translations(h, 0, r, 2, _lib.fptr(t)))
    seed, iters, eps = 77, 40_000, 2e-3
    out = np.zeros(len(Q))
    _lib.check(L.dpx_hybrid_compute_intensity(h, _lib.DPX_OA_MC, _lib.dptr(out), eps, iters, seed, None))
    _lib.check(L.dpx_hybrid_destroy(h))
    crot = np.repeat(rots[:, :3].astype(np.float64), 2, axis=0)
    ctr = np.concatenate([t[:, :3] for t in trans]).astype(np.float64)
    data, co = oracle_grid(amp, gs, qmax)
    kp = []
    leaf = O.make_leaf(data, co, copy_rot=crot, copy_tr=ctr, keep=kp)
    dirs = O.mc_directions(seed, iters)
    ref = O.integrate_layers_gpu_rule(gs, qmax, [leaf], Q.astype(np.float64), dirs, 0, iters, eps, 4096)
    assert rel(out, ref) <= tol
    del keep


def test_grid_amplitude_with_tabulated_form_factors(ctx):
    """dpx_pdb_jacobian_grid_amplitude_aff takes the form factors as the
    reference's atomicFFCalculator::GetQMajorAFFMatrix tabulates them ([U][nq],
    q fastest, dummy-atom solvent folded in): the FP64 grid equals the
    coefficient entry's within the table's float rounding."""
    amp = globule(250, 1.1, seed=62, extra=SOLVENT)
    gs, qmax = 20, 5.0
    L = dpx.lib()
    P = L.dpx_grid_cells(gs)
    step = qmax / (gs // 2)
    nq = gs // 2 + 4
    s = O.Struct.from_pdb(amp)
    aff = O.aff_table(s, nq, 0.0, step, O.FP64)  # [nq, U]
    tab = np.ascontiguousarray(aff.T.astype(np.float32))  # [U][nq]
    a = amp.atoms_float4()
    out = np.zeros(2 * P)
    _lib.check(L.dpx_pdb_jacobian_grid_amplitude_aff(P, 3, 6, step, _lib.dptr(out), _lib.fptr(a), len(a),
                                                     len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(tab),
                                                     nq, amp.flags, amp.solventED, None, None, 0, 0.0, None, None, 0,
                                                     0.0, amp.scale, M.FP64, None))
    assert rel_to_max(out, O.grid_fill(s, gs, qmax, O.FP64)) <= 2e-7
    assert L.dpx_pdb_jacobian_grid_amplitude_aff(P, 3, 6, step, _lib.dptr(out), _lib.fptr(a), len(a),
                                                 len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(tab),
                                                 nq - 1, amp.flags, amp.solventED, None, None, 0, 0.0, None, None, 0,
                                                 0.0, amp.scale, M.FP64, None) == -1
