"""Regenerate tests/golden/scripted.json.gz from the reference's scripted-symmetry goldens.

Run in a container that holds the reference checkout, given as the first
argument (or DPX_REF_ROOT); the GPU machine and the tests only read the committed
file.

Source: PythonInterface/tests/reviewer_tests/files_for_tests/generate/gpu/short/
Scripted_Symm_Impl_No_Charges_{wo,With}_Hydr_{MC,VEGAS,Ga_Kr,Hybrid_MC,
Hybrid_VEGAS} of the reference: a Lua-scripted symmetry (the "Space filling
symmetry - Cartesian" script: a 3 x 2 x 3 lattice of copies 4, 4 and 8.13 nm
apart) over a ManualSymmetry of one placed copy of the 3J6F GDP tubulin dimer
PDB, dummy-atom solvent at 334 e/nm^3 (with hydration: a voxelized layer),
grid 150, qmax 5, and the I(q) the reference's GPU path gave, averaged over
10 runs (q, I, sigma per point, plus the runs' mean chi-square and its
spread), which its acceptance test compares against
(test_generate/test_generate_results.py:99-199).

Stored per case: the state document without its viewport and fitting blocks
and the standard's columns and chi-square figures.  Stored once: the Lua
script (the same file in every case) and the SHA-256 of the PDB, which must
equal the one whose records tests/golden/mansymm.json.gz holds (the tests take
the records from there).  The *_Amp variants read amplitude files that are not
in the checkout (Git LFS pointers) and are left out.
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
CASES = ["Scripted_Symm_Impl_No_Charges_%s_Hydr_%s" % (h, m) for h in ("wo", "With")
         for m in ("MC", "VEGAS", "Ga_Kr", "Hybrid_MC", "Hybrid_VEGAS")]

sys.path.insert(0, HERE)
from make_mansymm import standard  # noqa: E402  (the same standard-file reader)


def main():
    with gzip.open(os.path.join(HERE, "mansymm.json.gz"), "rt") as f:
        mans = json.load(f)
    out = {"cases": {}, "pdb_name": mans["pdb_name"]}
    script = script_name = None
    for name in CASES:
        d = os.path.join(BASE, name)
        with open(os.path.join(d, name + ".state")) as f:
            st = json.load(f)
        st.pop("Viewport", None)
        st.pop("FittingPreferences", None)
        pdbs = [x for x in os.listdir(d) if x.lower().endswith(".pdb")]
        luas = [x for x in os.listdir(d) if x.lower().endswith(".lua")]
        assert len(pdbs) == 1 and len(luas) == 1, (pdbs, luas)
        h = hashlib.sha256(open(os.path.join(d, pdbs[0]), "rb").read()).hexdigest()
        out.setdefault("pdb_sha256", h)
        assert h == out["pdb_sha256"], "the cases do not share one PDB file"
        text = open(os.path.join(d, luas[0]), encoding="latin-1").read()
        if script is None:
            script, script_name = text, luas[0]
        assert text == script, "the cases do not share one script"
        out["cases"][name] = {"state": st, "standard": standard(os.path.join(d, name + "TestStandard.out"))}
    # the records the tests use come from mansymm.json.gz: check they are this PDB's
    lines = [ln for ln in open(os.path.join(BASE, CASES[0], pdbs[0]), "rb").read().decode("latin-1").split("\n")
             if ln[:6] in ("ATOM  ", "HETATM", "MODEL ", "ENDMDL")]
    assert lines == mans["pdb_lines"], "the PDB records differ from mansymm.json.gz's"
    out["script_name"], out["script"] = script_name, script
    dst = os.path.join(HERE, "scripted.json.gz")
    with gzip.open(dst, "wt") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
