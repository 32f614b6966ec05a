"""CPU tests: the oracle against the reference's golden vectors and known answers.

Golden data (tests/golden/, made by tests/golden/make_golden.py from the
reference checkout):
* grid_index.json  — the reference's Python Grid index maps (Amplitudes.py:48-200)
* single_atom.json — the reference's deterministic single-atom I(q) fixtures
* points.json      — the six-atom statistical fixture
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from dpx import models as M
from dpx.elements import IONS
from helpers import VACUUM, SOLVENT, rel

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_grid_cell_count():
    # P = 6 L'(L'+1)^2 + 1 (Grid.cpp:184-186); 1,548,289 cells for 60 layers
    assert O.grid_cells(120) == 1548289
    assert O.grid_cells(400) == 50688289
    assert O.grid_cells(300) == 21771289


@pytest.mark.parametrize("key", ["8_50.0", "20_7.5"])
def test_grid_index_maps_match_reference(key):
    import ctypes as C
    cells = _load("grid_index.json")[key]
    L = O.lib()
    qi, ti, pi = C.c_int(), C.c_int64(), C.c_int64()
    gs, qmax = key.split("_")
    step = float(qmax) / (int(gs) // 2)
    for m, i, j, k, q, th, ph in cells:
        L.orc_indices_from_index(m, C.byref(qi), C.byref(ti), C.byref(pi))
        assert (qi.value, ti.value, pi.value) == (i, j, k)
        assert L.orc_index_from_indices(i, j, k) == m
        if i:
            assert abs(i * step - q) <= 1e-12 * max(1, q)
            assert abs(np.pi * j / (3 * i) - th) <= 1e-12
            assert abs(np.pi * k / (3 * i) - ph) <= 1e-12


def test_element_table_matches_reference_rows():
    ions = _load("single_atom.json")["ions"]
    for sym, row in ions.items():
        assert tuple(row["coeffs"]) == IONS[sym].coeffs, sym
        assert row["dummy_radius"] == IONS[sym].dummy_radius, sym


def _single_atom_intensity(f):
    amp = M.PDBAmplitude([f["ion"]], [[0.037, -1.1639, 3.8862]], f["extra"], centered=f["centered"])
    s = O.Struct.from_pdb(amp)
    gs, qmax = f["gridSize"], f["qMax"]
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    dirs = O.mc_directions(7, 600)
    return O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], f["q"], dirs, 0, 600, f["convergence"])


@pytest.mark.parametrize("idx", range(22))
def test_single_atom_known_answers(idx):
    """I(q) = |f(q) - dummy(q)|^2 through grid fill, splines and interpolation.
    The reference evaluates the form factors in float, so the bound is at the
    amplitude level: |sqrt(I) - sqrt(I_ref)| <= 2e-6 sqrt(max I_ref)."""
    f = _load("single_atom.json")["fixtures"][idx]
    I = _single_atom_intensity(f)
    ref = np.array(f["I"])
    assert np.max(np.abs(np.sqrt(I) - np.sqrt(ref))) <= 2e-6 * np.sqrt(ref.max()), f["name"]
    assert np.max(np.abs(I - ref)) <= 2e-6 * ref.max(), f["name"]


@pytest.mark.parametrize("idx", [0, 1])
def test_points_fixture_statistical(idx):
    """Six-atom fixture (orientation dependent): the reference's acceptance is
    statistical (test_generate_results.py:99-199); require the oracle's MC mean
    within 3 sigma-equivalents on >= 90 % of the points."""
    f = _load("points.json")[idx]
    sym = [a[0] for a in f["atoms"]]
    xyz = [a[1:] for a in f["atoms"]]
    amp = M.PDBAmplitude(sym, xyz, f["extra"], centered=f["centered"])
    s = O.Struct.from_pdb(amp)
    gs, qmax = f["gridSize"], f["qMax"]
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    q = np.array(f["q"])[::8]
    ref = np.array(f["I"])[::8]
    sig = np.array(f["sigma"])[::8]
    dirs = O.mc_directions(3, 20000)
    I = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], q, dirs, 0, 20000, 0.0)
    # sigma of a 10-run mean is tiny where the MC converged; allow a 1e-3 relative floor
    tol = 3 * sig + 1e-3 * np.abs(ref)
    assert np.mean(np.abs(I - ref) <= tol) >= 0.9


def test_directions_reproduce_mt19937_stream():
    d = O.mc_directions(5489, 3)
    # std::mt19937 default seed 5489; first outputs are 3499211612, 581869302, ...
    # generate_canonical<double,53> combines two 32-bit draws: (a + b 2^32) / 2^64
    a, b = 3499211612, 581869302
    u2 = 2.0 * (a + b * 2.0 ** 32) / 2.0 ** 64
    assert abs(d[0, 1] - np.pi * u2) < 1e-15
    assert np.all((d[:, 0] >= 0) & (d[:, 0] <= np.pi)) and np.all((d[:, 1] >= 0) & (d[:, 1] < 2 * np.pi))


def test_q_brackets_cover_every_q():
    Q = np.linspace(0, 5, 200)
    b = O.q_brackets(120, 5.0, Q)
    assert b[0] == -1 and np.all(b[1:] >= 0)
    step = 5.0 / 60
    for q, l in zip(Q[1:], b[1:]):
        assert l * step < q <= (l + 1) * step + 1e-12


def test_oracle_modes_agree_to_float_precision():
    amp = M.PDBAmplitude(["C", "N", "O", "S", "C"], np.random.default_rng(0).normal(size=(5, 3)), VACUUM)
    s = O.Struct.from_pdb(amp)
    a = O.grid_fill(s, 16, 4.0, O.FP64)
    b = O.grid_fill(s, 16, 4.0, O.REFEXACT)
    assert np.max(np.abs(a - b)) / np.max(np.abs(a)) < 2e-6


@pytest.mark.skipif(not O.have_ref(), reason="reference checkout not built here")
def test_oracle_pinned_to_reference_build():
    """The restatement against the reference's own Grid.cpp / Atomic Form Factor.cpp."""
    import ctypes as C
    rng = np.random.default_rng(1)
    sym = list(rng.choice(["C", "N", "O", "S"], 25))
    amp = M.PDBAmplitude(sym, rng.normal(size=(25, 3)) * 0.8, SOLVENT)
    s = O.Struct.from_pdb(amp)
    gs, qmax = 64, 5.0  # the reference's OpenMP chunking needs >= 32 shells on 8 cores
    P = O.grid_cells(gs)
    rd, rc = np.zeros(2 * P), np.zeros(2 * P)
    xf = amp.xyz.astype(np.float32).ravel().copy()
    cf = amp.coeffs.astype(np.float32)
    rf = amp.ion_rads.astype(np.float32)
    fp = C.POINTER(C.c_float)
    dp = C.POINTER(C.c_double)
    O.ref().ref_grid_fill(gs, qmax, len(sym), xf.ctypes.data_as(fp), len(amp.atoms_per_ion),
                          amp.atoms_per_ion.ctypes.data_as(C.POINTER(C.c_int)), cf.ctypes.data_as(fp),
                          rf.ctypes.data_as(fp), amp.flags, amp.solventED, amp.c1, amp.scale, rd.ctypes.data_as(dp),
                          rc.ctypes.data_as(dp))
    d64 = O.grid_fill(s, gs, qmax, O.FP64)
    assert np.max(np.abs(d64 - rd)) / np.max(np.abs(rd)) < 1e-6  # reference computes phases in float
    c64 = O.grid_splines(gs, rd, O.FP64)
    assert np.max(np.abs(c64 - rc)) / np.max(np.abs(rc)) < 1e-6  # reference keeps the diagonal in float
    out = np.zeros(2)
    for th, ph in [(0.3, 1.1), (3.0, 6.1), (0.01, 0.0), (np.pi, 3.3)]:
        for q in (0.05, 0.41, 2.2, 5.0):
            mine = O.amplitudes_at_points(gs, qmax, rd, rc, [q], th, ph)[0]
            O.ref().ref_grid_amplitudes_at_points(gs, qmax, rd.ctypes.data_as(dp), rc.ctypes.data_as(dp), 1,
                                                  np.array([q]).ctypes.data_as(dp), th, ph, out.ctypes.data_as(dp))
            r = out[0] + 1j * out[1]
            assert abs(mine - r) <= 1e-14 * abs(r)  # same arithmetic up to FMA contraction


@pytest.mark.parametrize("idx", [0, 9, 21])
def test_single_atom_known_answers_vegas(idx):
    """VEGAS (restated from the reference's GPU-only code) on an orientation-
    independent amplitude returns sum(bin volume x mean) = |f - dummy|^2."""
    f = _load("single_atom.json")["fixtures"][idx]
    amp = M.PDBAmplitude([f["ion"]], [[0.037, -1.1639, 3.8862]], f["extra"], centered=f["centered"])
    s = O.Struct.from_pdb(amp)
    gs, qmax = f["gridSize"], f["qMax"]
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    q = np.array(f["q"])[::10]
    ref = np.array(f["I"])[::10]
    I = O.vegas_intensity(gs, qmax, [O.make_leaf(data, co)], q, 7, 1024, 4096, f["convergence"])
    assert np.max(np.abs(np.sqrt(I) - np.sqrt(ref))) <= 2e-6 * np.sqrt(ref.max())


@pytest.mark.parametrize("idx", [1, 12])
def test_single_atom_known_answers_gauss_kronrod(idx):
    """Adaptive GK on an orientation-independent amplitude: G7 and K15 agree on
    the first level and the integral / 2 pi is |f - dummy|^2."""
    f = _load("single_atom.json")["fixtures"][idx]
    amp = M.PDBAmplitude([f["ion"]], [[0.037, -1.1639, 3.8862]], f["extra"], centered=f["centered"])
    s = O.Struct.from_pdb(amp)
    gs, qmax = f["gridSize"], f["qMax"]
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    q = np.array(f["q"])[::40]
    ref = np.array(f["I"])[::40]
    I = np.array([O.gk_intensity(gs, qmax, [O.make_leaf(data, co)], x, 1e-5, 8) for x in q])
    assert np.max(np.abs(np.sqrt(I) - np.sqrt(ref))) <= 2e-6 * np.sqrt(ref.max())


def test_vegas_refines_bins_toward_variance():
    """The bin refinement moves boundaries: a strongly anisotropic model gets a
    different estimate sequence than a fixed grid would, and converges."""
    rng = np.random.default_rng(4)
    amp = M.PDBAmplitude(list(rng.choice(["C", "O"], 40)), rng.normal(size=(40, 3)) * [0.2, 0.2, 1.5], VACUUM)
    s = O.Struct.from_pdb(amp)
    gs, qmax = 20, 4.0
    data = O.grid_fill(s, gs, qmax, O.FP64)
    co = O.grid_splines(gs, data, O.FP64)
    Q = np.linspace(0, 4, 21)
    a = O.vegas_intensity(gs, qmax, [O.make_leaf(data, co)], Q, 3, 1024, 8 * 1024, 0.0)
    dirs = O.mc_directions(3, 200000)
    mc = O.integrate_layers(gs, qmax, [O.make_leaf(data, co)], Q, dirs, 0, 200000, 0.0)
    assert np.all(np.isfinite(a))
    assert np.max(np.abs(a - mc) / mc) < 0.05  # same integral, independent estimators
