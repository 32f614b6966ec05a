"""Voxelized solvent on the CPU: the library's C++ voxelizer against the
numpy/scipy restatement in the oracle, box for box, and physical checks of the
solvation layer (its volume against the analytic shell)."""
import math
import sys
import os

import numpy as np
import pytest

from dpx import models as M

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import voxel as OV  # noqa: E402

pytest.importorskip("scipy")


def _leaf(n, r, seed, extra):
    sym, xyz = M.make_globule(n, r, seed)
    return M.PDBAmplitude(sym, xyz, extra)


CASES = [
    # scale, solventED, c1, voxelStep, probe, thickness, outerED, fillHoles, solventOnly, radType
    (60, 0.7, 1, [1, 333, 1, 0.05, 0.14, 0.28, 400, 0, 0, 4]),
    (120, 0.9, 2, [1, 333, 1, 0.05, 0.14, 0.3, 400, 1, 0, 4]),
    (80, 0.8, 3, [1, 333, 1, 0.06, 0.2, 0.1, 380, 1, 0, 4]),    # thickness below the probe
    (90, 0.8, 4, [1, 334, 1, 0.05, 0.14, 0.28, 364, 1, 0, 5]),  # excluded-volume boxes too
]


@pytest.mark.parametrize("n,r,seed,extra", CASES)
def test_voxelizer_matches_oracle(n, r, seed, extra):
    a = _leaf(n, r, seed, extra)
    ec, ed, lc, ld = a.voxel_boxes()
    oec, oed, olc, old, _ = OV.voxel_solvent(a.xyz, a.atom_radii(), a.voxelStep, a.solventRad,
                                             a.solvationThickness, a.fillHoles)
    assert len(ed) > 0 and (len(ld) > 0 or a.solvationThickness < a.solventRad)
    assert np.array_equal(ed, oed) and np.array_equal(ec, oec)
    assert np.array_equal(ld, old) and np.array_equal(lc, olc)


def test_solvent_boxes_weights():
    a = _leaf(90, 0.8, 4, [1, 334, 1, 0.05, 0.14, 0.28, 364, 1, 0, 5])
    b = a.solvent_boxes()
    ec, ed, lc, ld = a.voxel_boxes()
    assert len(b) == len(ec) + len(lc)
    assert np.all(b[:len(ec), 3] == np.float32(-334)) and np.all(b[len(ec):, 3] == np.float32(30))
    assert np.allclose(b[:len(ec), 4:7], 0.05 * ed)
    d4 = _leaf(90, 0.8, 4, [1, 334, 1, 0.05, 0.14, 0.28, 364, 1, 0, 4]).solvent_boxes()
    assert np.all(d4[:, 3] == np.float32(30))  # radius type 4: the layer only
    assert _leaf(50, 0.6, 5, [1, 334, 1, 0.05, 0.14, 0.28, 0, 1, 0, 4]).solvent_boxes() is None


def test_single_atom_layer_volume():
    """A lone carbon: the layer is the shell between the probe-grown surface
    and thickness beyond it; its voxel volume tracks the analytic shell."""
    a = M.PDBAmplitude(["C"], np.zeros((1, 3)), [1, 333, 1, 0.02, 0.14, 0.3, 400, 0, 0, 4])
    ec, ed, lc, ld = a.voxel_boxes()
    vol = float(np.sum(np.prod(ld.astype(np.float64), axis=1))) * 0.02 ** 3
    r = a.atom_radii()[0]
    # voxels within r + probe are the probe shell; the layer adds `thickness`
    # beyond the probe surface and excludes the atom itself
    r_in, r_out = r, r + 0.14 + (0.3 - 0.14)
    shell = 4.0 / 3.0 * math.pi * (r_out ** 3 - r_in ** 3)
    assert 0.7 * shell < vol < 1.3 * shell
