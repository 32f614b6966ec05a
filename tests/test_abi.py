"""CPU tests of the C-ABI boundary: libdpx loads, exports every entry point
include/dpx.h declares, and its host-only helpers agree with the oracle.
No kernel runs here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
import dpx
from dpx import _lib
from dpx import models as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "dpx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dpx_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol():
    L = C.CDLL(_lib.LIB_PATH)
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_no_device_is_a_status_not_a_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    rc = dpx.lib().dpx_ctx_create(0, C.byref(h))
    assert rc == -5 and b"no CUDA device" in dpx.lib().dpx_last_error()


def test_directions_match_oracle():
    a = M.mc_directions(1234, 1000)
    b = O.mc_directions(1234, 1000)
    assert np.array_equal(a, b)


def test_layer_seeds_match_oracle():
    assert np.array_equal(M.layer_seeds(99, 200, 60), O.layer_seeds(99, 200, 60))


@pytest.mark.parametrize("gs,qmax,nq,q0", [(120, 5.0, 200, 0.0), (30, 15.0, 801, 0.0), (400, 7.5, 500, 0.0),
                                           (40, 3.0, 37, 0.4), (20, 2.0, 3, 0.0)])
def test_brackets_match_oracle(gs, qmax, nq, q0):
    Q = np.linspace(q0, qmax, nq)
    out = np.zeros(nq, dtype=np.int32)
    _lib.check(dpx.lib().dpx_q_brackets(gs, qmax, nq, _lib.dptr(Q), _lib.iptr(out)))
    assert np.array_equal(out, O.q_brackets(gs, qmax, Q))


@pytest.mark.parametrize("seed", range(6))
def test_brackets_match_oracle_ragged(seed):
    """Clustered, repeated, grid-aligned and unsorted q lists (the reference's
    bracket scan has no sortedness requirement) give the oracle's layers."""
    rng = np.random.default_rng(seed)
    gs, qmax = int(rng.integers(4, 120)), float(rng.uniform(1.0, 8.0))
    step = 2 * qmax / gs
    nq = int(rng.integers(1, 300))
    Q = np.sort(rng.uniform(0, qmax, nq))
    if seed % 3 == 1:  # repeats and exact layer boundaries
        Q = np.sort(np.concatenate([Q[: nq // 2], Q[: nq // 4], step * rng.integers(0, gs // 2, nq // 4 + 1)]))
    elif seed % 3 == 2:
        Q = rng.permutation(Q)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    out = np.zeros(len(Q), dtype=np.int32)
    _lib.check(dpx.lib().dpx_q_brackets(gs, qmax, len(Q), _lib.dptr(Q), _lib.iptr(out)))
    assert np.array_equal(out, O.q_brackets(gs, qmax, Q))


def test_grid_geometry():
    assert dpx.lib().dpx_grid_cells(120) == 1548289
    assert dpx.lib().dpx_grid_bytes(400, M.FP32) == 50688289 * 16
    assert dpx.lib().dpx_grid_bytes(400, M.FP64) == 50688289 * 32
    assert dpx.lib().dpx_grid_cells(1) == -1


def test_globule_generator():
    sym, xyz = M.make_globule(3000, 2.5, seed=3)
    assert len(sym) == 3000
    r = np.linalg.norm(xyz, axis=1)
    assert r.max() <= 2.5 + 1e-6
    d = np.linalg.norm(np.diff(xyz, axis=0), axis=1)
    assert np.mean(np.abs(d - 0.15) < 1e-5) > 0.95  # chain steps of 0.15 nm (restarts aside)
    frac = {e: sym.count(e) / 3000 for e in "CNOS"}
    assert abs(frac["C"] - 0.63) < 0.03 and abs(frac["O"] - 0.19) < 0.03
    sym2, xyz2 = M.make_globule(3000, 2.5, seed=3)
    assert sym == sym2 and np.array_equal(xyz, xyz2)


def test_bad_arguments_are_rejected():
    out = np.zeros(4, dtype=np.int32)
    assert dpx.lib().dpx_q_brackets(1, 1.0, 4, None, _lib.iptr(out)) == -1
    assert dpx.lib().dpx_make_globule(0, 1.0, 1, None, None) == -1
    with pytest.raises(NotImplementedError):  # voxel solvent with the van der Waals radius table
        M.PDBAmplitude(["C"], [[0, 0, 0]], [1, 333, 1, 0.05, 0.14, 0.28, 0, 0, 0, 1])
    assert dpx.lib().dpx_voxel_solvent(0, None, None, 0.05, 0.14, 0.28, 0, None) == -1


def test_pdb_amplitude_mirrors_precalculate():
    amp = M.PDBAmplitude(["O", "C", "N", "C", "S"], np.eye(5, 3), [2, 333, 1, 0.05, 0.14, 0.28, 0, 0, 0, 4])
    assert amp.symbols == ["C", "C", "N", "O", "S"]
    assert list(amp.atoms_per_ion) == [2, 1, 1, 1]
    assert amp.flags == 3 and amp.scale == 2.0
    U = 4
    assert amp.coeffs[0 + 8 * U] == 0.2156  # c of carbon, sortedCoeffs layout coeffs[u + k U]
