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
from helpers import SOLVENT, VACUUM, globule, oracle_grid, rel, rel_to_max

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
                                                   _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, amp.scale,
                                                   M.FP64, None)
    _lib.check(rc)
    s = O.Struct(amp.xyz, amp.atoms_per_ion, cf.astype(np.float64), rf.astype(np.float64), amp.flags,
                 amp.solventED, amp.c1, amp.scale)
    assert rel_to_max(out, O.grid_fill(s, gs, qmax, O.FP64)) <= TOL64
    stop = C.c_int(1)
    assert dpx.lib().dpx_pdb_jacobian_grid_amplitude(P, 3, 6, qmax / (gs // 2), _lib.dptr(out), _lib.fptr(a), len(a),
                                                     len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(cf),
                                                     _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, amp.scale,
                                                     M.FP64, C.byref(stop)) == -4
    assert dpx.lib().dpx_pdb_jacobian_grid_amplitude(P + 1, 3, 6, 0.5, _lib.dptr(out), _lib.fptr(a), len(a),
                                                     len(amp.unique), _lib.iptr(amp.atoms_per_ion), _lib.fptr(cf),
                                                     _lib.fptr(rf), amp.flags, amp.solventED, amp.c1, amp.scale,
                                                     M.FP64, None) == -1


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
