"""The reference's own docked-sum goldens, decoded from its JSON states.

Each case of tests/golden/mansymm.json.gz (made by make_mansymm.py from the
reference's generate/gpu/short/Man_Symm_Impl_No_Charges_* fixtures) is a
two-level ManualSymmetry of the 3J6F tubulin dimer (18 docked copies, 6,763
atoms with implicit hydrogens, dummy-atom solvent, with or without a
voxelized hydration layer) averaged by Monte Carlo, VEGAS or Gauss-Kronrod on
the grid or by the hybrid per-orientation docked sum.  The state document goes
through dpx.state.decode (this package's JSON state reader) and the PDB
records through dpx.pdb.read_pdb; the I(q) of the FP32-bulk path must pass
the reference's acceptance of its generate tests
(PythonInterface/tests/reviewer_tests/test_generate/test_generate_results.py:
99-199): chi-square within one or two sigma of the standard's, or the point
test (fewer than half of the points outside one sigma and under 30 % outside
two), or the normalised residuals below 1e-8, or no point below 0.999999 of
the standard.  The standards are the mean of 10 runs of the reference's GPU
path, with their spread as sigma.
"""
import gzip
import json
import math
import os
import struct

import numpy as np
import pytest

from dpx import models as M
from dpx import state as S

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "mansymm.json.gz")


def _load():
    with gzip.open(GOLD, "rt") as f:
        return json.load(f)


DATA = _load()
CASES = sorted(DATA["cases"])


# ---- the reference's acceptance (test_generate_results.py:99-199), restated ----
def chi_a_sq(calc, exp, sig):
    tot = 0.0
    for c, e, s in zip(calc, exp, sig):
        tot += (e - c) ** 2 if s < 10e-4 else ((e - c) / s) ** 2
    return tot / len(exp)


def points_test(calc, exp, sig):
    failed = {1: 0, 2: 0}
    for c, e, s in zip(calc, exp, sig):
        for j in (1, 2):
            inside = e - j * s <= c <= e + j * s
            ulps = struct.unpack("<qq", struct.pack("<dd", c, e))
            if not inside and abs(ulps[1] - ulps[0]) > 256:
                failed[j] += 1
    n = len(exp)
    return failed[1] / n < 0.5 and failed[2] / n < 0.3


def normalized_rqi(calc, exp):
    r = [abs((c - e) / max(c, e)) if max(c, e) != 0 else 0.0 for c, e in zip(calc, exp)]
    return max(r) < 1e-8 and float(np.mean(r)) < 1e-8


def div_test(calc, exp):
    return all(abs(c / e) >= 0.999999 for c, e in zip(calc, exp))


@pytest.mark.parametrize("name", CASES)
def test_reference_docked_sum_golden(ctx, name):
    case = DATA["cases"][name]
    std = case["standard"]
    job = S.decode(case["state"], files={DATA["pdb_name"]: DATA["pdb_lines"]})
    Q = np.asarray(std["q"])
    exp, sig = np.asarray(std["I"]), np.asarray(std["sigma"])
    dirs = M.mc_directions(20260, 1_000_000) if job.method == "MC" else None
    I = job.intensity(ctx, Q, dirs=dirs, precision=M.FP32, seed=11)
    chi = chi_a_sq(I, exp, sig)
    a = chi < std["chi_square"] + std["sigma_chi_square"]
    b = chi < std["chi_square"] + 2 * std["sigma_chi_square"]
    c = points_test(I, exp, sig)
    d = normalized_rqi(I, exp)
    e = div_test(I, exp)
    rel = np.abs(I - exp) / exp
    print(f"{name}: method {job.method}, chi_a^2 {chi:.4g} (standard {std['chi_square']:.4g} +- "
          f"{std['sigma_chi_square']:.3g}), chi1 {a} chi2 {b} points {c} rqi {d} div {e}; "
          f"max rel diff {rel.max():.3e}, median {np.median(rel):.3e}")
    assert math.isfinite(chi)
    assert a or b or c or d or e
