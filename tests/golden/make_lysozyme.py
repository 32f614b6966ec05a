"""Regenerate tests/golden/lysozyme.json from the reference's lysozyme example.

Run in a container that holds the reference checkout, given as the first
argument (or DPX_REF_ROOT); the GPU machine and the tests only read the committed JSON file.

Source: "Example Files/Examples/CPU/Fast_CPU/6_Lysozyme/" of the reference:

* ``pdb_lines``  — the ATOM / HETATM / MODEL / ENDMDL records of 1lyz.pdb
  (the public PDB entry 1LYZ, 1102 atoms with waters);
* ``implicit``   — what the reference's reader reported for it in the output
  headers ("1001 of 1102 atoms are treated as having implicit hydrogen atoms
  (129 amino acids)");
* ``debye``      — 1lyzDebye.out: the reference's DebyeCalculator on its CPU
  (512 q in [0, 6] nm^-1, no solvent, no B factors), printed to 6 digits;
* ``fitted`` / ``fitted_outer`` — Fitted_Scale_and_Constant.out and
  Fitted_Outer_Solvent_ED_Constant_and_Scale.out: D+'s I(q) of the state in
  each header (grid 50, qmax 3.78909, Gauss-Kronrod, convergence 0.01), full
  precision, with the header's model parameters parsed into ``model``.
"""
from __future__ import annotations

import json
import os
import sys
import re

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPX_REF_ROOT", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: %s REFERENCE_ROOT (or set DPX_REF_ROOT)" % sys.argv[0])
HERE = os.path.dirname(os.path.abspath(__file__))
EX = os.path.join(REF, "Example Files", "Examples", "CPU", "Fast_CPU", "6_Lysozyme")


def numbers(path):
    q, I = [], []
    for line in open(path):
        if line.startswith("#") or not line.strip():
            continue
        a, b = line.split()[:2]
        q.append(float(a))
        try:  # the reference prints NaN as "1.#QNAN" at a few q of one file: kept as null
            v = float(b)
        except ValueError:
            v = float("nan")
        I.append(None if v != v else v)
    return q, I


def header(path):
    """Composite scale / constant, integration settings and the leaves in file
    order, each with the numbers its header block prints and the scale of the
    manual symmetry it sits in (1 for a top-level leaf)."""
    out = {"leaves": []}
    sym = None   # the open manual symmetry: {"depth", "scale"}
    cur = None   # the block the next parameter lines belong to
    keys = {"Solvent ED amplitude subtracted": "solvent_ed", "c1": "c1", "Solvent probe radius": "probe",
            "Solvation thickness": "thickness", "Solvent ED step size": "voxel_step",
            "Outer Solvent ED": "outer_solvent_ed"}
    for ln in open(path):
        if not ln.startswith("#"):
            break
        depth = len(ln) - len(ln.lstrip("#"))
        body = ln.lstrip("#").strip()
        m = re.match(r"(Orientation Method|Orientation Iterations|Convergence|qmax)\t(.*)", body)
        if m:
            out[m.group(1)] = m.group(2)
        elif depth == 1 and body.startswith("Scale:"):
            out["scale"] = float(body.split(":")[1])
        elif depth == 1 and body.startswith("Constant:"):
            out["constant"] = float(body.split(":")[1])
        elif body.startswith("Grid size ="):
            out["grid_size"] = int(body.split("=")[1])
        elif body == "Manual symmetry":
            sym = cur = {"depth": depth, "scale": 1.0, "kind": "sym"}
        elif body.startswith("PDB file:"):
            inside = sym is not None and sym["depth"] == depth - 1
            cur = {"depth": depth, "kind": "leaf", "sym_scale": sym["scale"] if inside else 1.0,
                   "solvent_only": False, "centered": False}
            out["leaves"].append(cur)
        elif cur is not None and depth == cur["depth"] and ":" in body:
            k, v = body.split(":", 1)
            if k == "Scale":
                cur["scale"] = float(v)
            elif cur["kind"] == "leaf" and k in keys:
                cur[keys[k]] = float(v)
            elif cur["kind"] == "leaf" and k == "Fill holes":
                cur["fill_holes"] = v.strip() == "true"
            elif cur["kind"] == "leaf" and k == "Solvent radius type":
                cur["rad_type"] = v.strip()
        elif cur is not None and cur["kind"] == "leaf" and depth == cur["depth"]:
            if body.startswith("The amplitude calculated corresponds to the solvent"):
                cur["solvent_only"] = True
            elif body.startswith("The atoms were centered"):
                cur["centered"] = True
    for lf in out["leaves"]:
        lf.pop("kind")
    return out


def main():
    pdb = [ln.rstrip("\r\n") for ln in open(os.path.join(EX, "1lyz.pdb"), newline="")
           if ln[:6] in ("ATOM  ", "HETATM", "MODEL ", "ENDMDL")]
    fitted = os.path.join(EX, "Fitted_Scale_and_Constant.out")
    imp = None
    for ln in open(fitted):
        m = re.search(r"(\d+) of (\d+) atoms are treated as having implicit hydrogen atoms \((\d+) amino acids\)", ln)
        if m:
            imp = {"atoms": int(m.group(1)), "total": int(m.group(2)), "residues": int(m.group(3))}
            break
    dq, dI = numbers(os.path.join(EX, "1lyzDebye.out"))
    out = {"source": "Example Files/Examples/CPU/Fast_CPU/6_Lysozyme", "pdb_lines": pdb, "implicit": imp,
           # q printed to 6 digits; DebyeCalculator computed it as qMin + (qMax - qMin) i / (n - 1)
           # with its defaults qMin 0, qMax 6, n 512 (DebyeCalculator.cpp:116-121, 232-235)
           "debye": {"q": dq, "I": dI, "qmin": 0.0, "qmax": 6.0, "n": 512, "solvent_ed": 0.0,
                     "debye_waller": False}}
    for key, name in (("fitted", "Fitted_Scale_and_Constant.out"),
                      ("fitted_outer", "Fitted_Outer_Solvent_ED_Constant_and_Scale.out")):
        q, I = numbers(os.path.join(EX, name))
        out[key] = {"file": name, "model": header(os.path.join(EX, name)), "q": q, "I": I}
    with open(os.path.join(HERE, "lysozyme.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote lysozyme.json:", len(pdb), "records,", len(dq), "Debye points")


if __name__ == "__main__":
    main()
