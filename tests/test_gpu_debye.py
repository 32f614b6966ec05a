"""GPU Debye sum (dpx_debye_intensity, dpx_calc_debye_v2) against the oracle
and the reference's own lysozyme output; and the grid path's orientation
average against the Debye sum, an independent check that needs no grid.

Tolerances: FP64 <= 1e-10 relative to the FP64 oracle; FP32 <= 1e-4 relative
I(q); lysozyme against the reference's 6-digit output <= 6e-6 (FP64) and
2e-5 (FP32); Gauss-Kronrod over a 80-layer FP64 grid against Debye <= 1e-4.
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
from dpx import pdb as P
from helpers import LAYER, SOLVENT, VACUUM, globule, rel

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "lysozyme.json")
TOL64, TOL32 = 1e-10, 1e-4
FP = C.POINTER(C.c_float)


def _with_extras(amp, seed, dw, anom):
    rng = np.random.default_rng(seed)
    amp.bfactors = rng.uniform(2.0, 40.0, len(amp.xyz)) if dw else None
    a = rng.normal(scale=[0.5, 0.3], size=(len(amp.xyz), 2)).astype(np.float32) if anom else None
    return a


def _oracle(amp, Q, p, anom):
    flags = _lib.DPX_CALC_ATOMIC_FORMFACTORS | (_lib.DPX_CALC_DUMMY_SOLVENT if p[0] != 0 else 0)
    s = O.Struct(amp.xyz, amp.atoms_per_ion, amp.coeffs, amp.ion_rads, flags, p[0], p[2])
    bf = np.asarray(amp.bfactors, dtype=np.float32).astype(np.float64) if p[1] > 0.1 else None
    an = None if anom is None else anom.astype(np.float64)
    return O.debye(s, Q, bfactor=bf, anom=an, mode=O.FP64)


@pytest.mark.parametrize("sol", [0.0, 333.0])
@pytest.mark.parametrize("dw", [False, True])
@pytest.mark.parametrize("anom", [False, True])
def test_debye_matches_oracle(ctx, sol, dw, anom):
    """300 atoms (a ragged last tile) and 37 q (a ragged last q block)."""
    amp = globule(300, 1.5, seed=41, extra=VACUUM)
    an = _with_extras(amp, 42, dw, anom)
    Q = np.linspace(0.0, 8.0, 37)
    p = [sol, 1.0 if dw else 0.0, 1.03]
    ref = _oracle(amp, Q, p, an)
    t = M.DebyeCalTester(amp, an)
    assert rel(t.CalculateVector(ctx, Q, p, M.FP64), ref) <= TOL64
    assert rel(t.CalculateVector(ctx, Q, p, M.FP32), ref) <= TOL32


@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 1000])
def test_debye_sizes(ctx, n):
    """Tile edges; q = 0 gives (sum f)^2, one atom gives f^2 at every q."""
    amp = globule(n, 0.4 + 0.002 * n, seed=n, extra=VACUUM)
    Q = np.array([0.0, 0.01, 0.7, 3.3, 9.5])
    ref = _oracle(amp, Q, [0, 0, 1], None)
    t = M.DebyeCalTester(amp)
    for prec, tol in ((M.FP64, TOL64), (M.FP32, TOL32)):
        I = t.CalculateVector(ctx, Q, (0, 0, 1), prec)
        assert rel(I, ref) <= tol
    f0 = sum(c * np.sum([u.coeffs[2 * k] for k in range(4)]) + c * u.coeffs[8]
             for c, u in zip(amp.atoms_per_ion, amp.unique))
    assert abs(t.CalculateVector(ctx, [0.0], (0, 0, 1), M.FP64)[0] / f0 ** 2 - 1) <= 1e-12
    one = t.CalculateVector(ctx, [2.0], (0, 0, 1), M.FP64)[0]
    assert one > 0


def test_debye_lysozyme_matches_reference_output(ctx):
    """1lyz (1102 atoms, implicit hydrogens) against the reference's
    DebyeCalculator output, at the q grid it computed on."""
    with open(GOLD) as f:
        g = json.load(f)
    a = P.read_pdb(g["pdb_lines"])
    amp = M.PDBAmplitude(a.symbols, a.xyz, VACUUM, bfactors=a.bfactor)
    d = g["debye"]
    Q = d["qmin"] + (d["qmax"] - d["qmin"]) * np.arange(d["n"]) / (d["n"] - 1)
    ref = np.array(d["I"])
    t = M.DebyeCalTester(amp)
    assert rel(t.CalculateVector(ctx, Q, (0, 0, 1), M.FP64), ref) <= 6e-6
    assert rel(t.CalculateVector(ctx, Q, (0, 0, 1), M.FP32), ref) <= 2e-5


@pytest.mark.parametrize("prec,tol", [(M.FP64, TOL64), (M.FP32, TOL32)])
def test_drop_in_debye_v2(ctx, prec, tol):
    """GPUCalcDebyeV2's interface: float q grid, float4 atoms, radius table
    indexed by atmInd, B factors and anomalous factors."""
    amp = globule(400, 1.6, seed=44, extra=VACUUM)
    an = _with_extras(amp, 45, True, True)
    n, U = len(amp.xyz), len(amp.unique)
    loc = amp.atoms_float4()
    # a radius table with the ions' radii at made-up atom indices
    atm_rad = np.zeros(16, dtype=np.float32)
    atm_ind = np.zeros(n, dtype=np.int8)
    off = 0
    for u, c in enumerate(amp.atoms_per_ion):
        atm_rad[3 + u] = amp.ion_rads[u]
        atm_ind[off:off + c] = 3 + u
        off += c
    coeffs = amp.coeffs.astype(np.float32)
    bf = np.asarray(amp.bfactors, dtype=np.float32)
    nq, qmin, qmax = 50, 0.1, 6.0
    out = np.zeros(nq)
    api = np.ascontiguousarray(np.concatenate([amp.atoms_per_ion, [0]]), dtype=np.int32)
    _lib.check(dpx.lib().dpx_calc_debye_v2(nq, qmin, qmax, _lib.dptr(out), n, _lib.iptr(api),
                                           loc.ctypes.data_as(FP), None, an.ctypes.data_as(FP), 1,
                                           bf.ctypes.data_as(FP), coeffs.ctypes.data_as(FP), 1, 0,
                                           atm_ind.ctypes.data_as(C.POINTER(C.c_char)),
                                           atm_rad.ctypes.data_as(FP), 333.0, 1.0, prec, None))
    step = np.float32((np.float32(qmax) - np.float32(qmin)) / np.float32(nq - 1))
    Q = np.array([np.float32(np.float32(qmin) + step * np.float32(k)) for k in range(nq)], dtype=np.float64)
    s = O.Struct(amp.xyz, amp.atoms_per_ion, coeffs.astype(np.float64), atm_rad[3:3 + U].astype(np.float64), 3,
                 np.float32(333.0), 1.0)
    ref = O.debye(s, Q, bfactor=bf.astype(np.float64), anom=an.astype(np.float64), mode=O.FP64)
    assert rel(out, ref) <= tol


def test_debye_rejects_boxes_and_bad_q(ctx):
    amp = globule(50, 0.8, seed=46, extra=LAYER)
    descs, keep = M.pdb_descs([amp])
    assert descs[0].n_boxes > 0
    out = np.zeros(2)
    Q = np.array([0.0, 1.0])
    assert dpx.lib().dpx_debye_intensity(ctx.handle, descs, None, None, 2, _lib.dptr(Q), M.FP32,
                                         _lib.dptr(out)) == -1
    descs[0].n_boxes, descs[0].boxes = 0, None
    Q[1] = -1.0
    assert dpx.lib().dpx_debye_intensity(ctx.handle, descs, None, None, 2, _lib.dptr(Q), M.FP32,
                                         _lib.dptr(out)) == -1
    Q[1] = 1.0
    assert dpx.lib().dpx_debye_intensity(ctx.handle, descs, None, None, 2, _lib.dptr(Q), M.FP32,
                                         _lib.dptr(out)) == 0
    del keep


@pytest.mark.parametrize("prec", [M.FP64, M.FP32])
def test_grid_orientation_average_converges_to_debye(ctx, prec):
    """The grid path (fill, splines, adaptive Gauss-Kronrod) against the exact
    orientation average: 200 atoms with dummy-atom solvent, 80 layers."""
    amp = globule(200, 1.0, seed=7, extra=SOLVENT)
    Q = np.array([0.0, 0.5, 1.0, 2.0, 3.0, 3.9])
    deb = M.DebyeCalTester(amp).CalculateVector(ctx, Q, (amp.solventED, 0, amp.c1), M.FP64)
    gk = M.DomainModel([amp], 80, 4.0, prec).CalculateIntensityVector(ctx, Q, 1e-6, 20, method="GK")
    assert rel(gk, deb) <= 1e-4
