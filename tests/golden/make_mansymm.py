"""Regenerate tests/golden/mansymm.json.gz from the reference's docked-sum goldens.

Run in a container that holds the reference checkout, given as the first
argument (or DPX_REF_ROOT); the GPU machine and the tests only read the committed
file.

Source: PythonInterface/tests/reviewer_tests/files_for_tests/generate/gpu/short/
Man_Symm_Impl_No_Charges_{wo,With}_Hydr_{MC,VEGAS,Ga_Kr,Hybrid_MC,Hybrid_VEGAS}
of the reference: a two-level ManualSymmetry (18 outer copies of an inner
symmetry of one copy) of the 3J6F GDP tubulin dimer PDB, dummy-atom solvent
at 334 e/nm^3 (with hydration: a 0.28 nm layer at 364 e/nm^3, holes filled),
grid 150, qmax 5, convergence 1e-3, and the I(q) the reference's GPU path
gave, averaged over 10 runs (q, I, sigma per point, plus the runs' mean
chi-square and its spread), which its acceptance test compares against
(test_generate/test_generate_results.py:99-199).

Stored per case: the state document without its viewport and fitting blocks,
the standard's q / I / sigma columns and chi-square figures.  Stored once:
the ATOM / HETATM / MODEL / ENDMDL records of the PDB (the same file in every
case; the public PDB entry 3J6F, 6,763 atoms).  The *_Amp variants read
amplitude files that are not in the checkout (Git LFS pointers) and are left
out.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPX_REF_ROOT", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: %s REFERENCE_ROOT (or set DPX_REF_ROOT)" % sys.argv[0])
HERE = os.path.dirname(os.path.abspath(__file__))
BASE = os.path.join(REF, "PythonInterface/tests/reviewer_tests/files_for_tests/generate/gpu/short")
CASES = ["Man_Symm_Impl_No_Charges_%s_Hydr_%s" % (h, m) for h in ("wo", "With")
         for m in ("MC", "VEGAS", "Ga_Kr", "Hybrid_MC", "Hybrid_VEGAS")]


def standard(path):
    """The columns and chi-square lines of a *TestStandard.out (as the
    reference's tests/reviewer_tests/utils.py Expected reads them)."""
    q, I, s = [], [], []
    chi = sig = None
    for line in open(path):
        if not line.strip():
            continue
        if line[0] == "#":
            if "Average Chi square" in line:
                chi = float(line.split()[-1])
            if "Sigma Chi square" in line:
                sig = float(line.split()[-1])
            continue
        if line[0] == "q":
            continue
        a = line.split()
        q.append(float(a[0]))
        I.append(float(a[1]))
        s.append(float(a[2]) if len(a) > 2 else 0.0)
    return {"q": q, "I": I, "sigma": s, "chi_square": chi, "sigma_chi_square": sig}


def main():
    out = {"cases": {}}
    pdb_hash = None
    for name in CASES:
        d = os.path.join(BASE, name)
        with open(os.path.join(d, name + ".state")) as f:
            st = json.load(f)
        st.pop("Viewport", None)
        st.pop("FittingPreferences", None)
        pdbs = [x for x in os.listdir(d) if x.lower().endswith(".pdb")]
        assert len(pdbs) == 1, pdbs
        raw = open(os.path.join(d, pdbs[0]), "rb").read()
        h = hashlib.sha256(raw).hexdigest()
        if pdb_hash is None:
            pdb_hash = h
            lines = [ln for ln in raw.decode("latin-1").split("\n")
                     if ln[:6] in ("ATOM  ", "HETATM", "MODEL ", "ENDMDL")]
            out["pdb_name"] = pdbs[0]
            out["pdb_lines"] = lines
        assert h == pdb_hash, "the cases do not share one PDB file"
        out["cases"][name] = {"state": st, "standard": standard(os.path.join(d, name + "TestStandard.out"))}
    dst = os.path.join(HERE, "mansymm.json.gz")
    with gzip.open(dst, "wt") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", dst, os.path.getsize(dst), "bytes,", len(out["pdb_lines"]), "PDB records")


if __name__ == "__main__":
    main()
