"""Regenerate the golden fixtures under tests/golden/ from the reference checkout.

Run in a container that holds the reference checkout, given as the first
argument (or DPX_REF_ROOT); the GPU machine and the tests only read the committed JSON files.

* grid_index.json   — cell index <-> (i, j, k) <-> (q, theta, phi) from the
  reference's own Python Grid class (PythonInterface/dplus/Amplitudes.py:48-200).
* single_atom.json  — the deterministic single-atom known-answer fixtures
  (PythonInterface/tests/reviewer_tests/files_for_tests/generate/cpu/short/
  {c,n,o,h}_explicit_*, {ch,ch2,ch3,nh,nh2,nh3,oh}_implicit_*): state
  parameters, the state document itself (without its viewport and fitting
  blocks) with its one-atom PDB record, and the reference's I(q) columns,
  plus the reference's own coefficient rows and dummy radii for those ions
  (PDBReaderLib.cpp).
* points.json       — the six-atom statistical fixture points_explicit_* (q, I, sigma).
"""
from __future__ import annotations

import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPX_REF_ROOT", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: %s REFERENCE_ROOT (or set DPX_REF_ROOT)" % sys.argv[0])
HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(REF, "PythonInterface/tests/reviewer_tests/files_for_tests/generate/cpu/short")

GROUPS = {"c": "C", "n": "N", "o": "O", "h": "H", "ch": "CH", "ch2": "CH2", "ch3": "CH3", "nh": "NH",
          "nh2": "NH2", "nh3": "NH3", "oh": "OH"}
# comment labels of the reference's X-ray table rows (PDBReaderLib.cpp:2270+)
TABLE_LABEL = {"H": "H", "C": "Carbon", "N": "N", "O": "O", "S": "S", "P": "P", "MG": "Mg", "CH": "CH",
               "CH2": "CH2", "CH3": "CH3", "NH": "NH", "NH2": "NH2", "NH3": "NH3", "OH": "OH", "SH": "SH"}
SVG_INDEX = {"H": 1, "C": 6, "N": 7, "O": 8, "S": 16, "MG": 12, "P": 15, "CH": 119, "CH2": 120, "CH3": 121,
             "NH": 122, "NH2": 123, "NH3": 124, "OH": 125, "SH": 126}


def read_out(path):
    q, I, s = [], [], []
    for line in open(path):
        if line.startswith("#") or line.startswith("q"):
            continue
        p = line.split()
        if len(p) >= 2:
            q.append(float(p[0]))
            I.append(float(p[1]))
            s.append(float(p[2]) if len(p) > 2 else 0.0)
    return q, I, s


def read_state(path):
    st = json.load(open(path))
    dp = st["DomainPreferences"]
    txt = open(path).read()
    extra = json.loads(re.search(r'"ExtraParameters":(\[[^\]]*\])', txt).group(1))
    centered = '"Centered":true' in txt
    return dict(gridSize=dp["GridSize"], qMax=dp["qMax"], convergence=dp["Convergence"],
                iterations=dp["OrientationIterations"], method=dp["OrientationMethod"], extra=extra,
                centered=centered)


def xray_rows():
    src = open(os.path.join(REF, "PDBReaderLib/PDBReaderLib.cpp")).read()
    start = src.index("atmFFcoefsMap << 0.49300")
    end = src.index("#pragma endregion", start)
    rows = {}
    for line in src[start:end].splitlines():
        m = re.match(r"\s*(?:atmFFcoefsMap <<\s*)?([-0-9.eE+,\s]+?)\s*,?\s*//\s*(\S+)", line)
        if not m:
            continue
        vals = [float(v) for v in re.sub(r"\s+", "", m.group(1)).split(",") if v]
        if len(vals) == 9 and m.group(2) not in rows:
            rows[m.group(2)] = vals
    return rows


def svg_radii():
    src = open(os.path.join(REF, "PDBReaderLib/PDBReaderLib.cpp")).read()
    out = {}
    for m in re.finditer(r"svgRad\[(\d+)\]\s*=\s*([0-9.]+);", src):
        out[int(m.group(1))] = float(m.group(2))
    return out


def main():
    sys.path.insert(0, os.path.join(REF, "PythonInterface"))
    from dplus.Amplitudes import Grid  # the reference's pure-Python grid

    idx = {}
    for gs, qmax in ((8, 50.0), (20, 7.5)):
        g = Grid(gs, qmax)
        cells = []
        for m, (q, th, ph) in g.create_grid():
            i, j, k = g.indices_from_index(m)
            cells.append([m, i, j, k, float(q), float(th), float(ph)])
        idx[f"{gs}_{qmax}"] = cells if gs == 8 else cells[::5]
    json.dump(idx, open(os.path.join(HERE, "grid_index.json"), "w"))

    rows = xray_rows()
    svg = svg_radii()
    ions = {}
    for sym, label in TABLE_LABEL.items():
        ions[sym] = dict(coeffs=rows[label], dummy_radius=svg.get(SVG_INDEX[sym]))
    fixtures = []
    for name in sorted(os.listdir(FIX)):
        m = re.match(r"([a-z0-9]+)_(explicit|implicit)_(Vacuum|SS334)$", name)
        if not m or m.group(1) not in GROUPS:
            continue
        d = os.path.join(FIX, name)
        st = read_state(os.path.join(d, name + ".state"))
        q, I, s = read_out(os.path.join(d, name + "TestStandard.out"))
        doc = json.load(open(os.path.join(d, name + ".state")))
        doc.pop("Viewport", None)
        doc.pop("FittingPreferences", None)
        pdbs = [x for x in os.listdir(d) if x.lower().endswith(".pdb")]
        pdb_lines = [ln for ln in open(os.path.join(d, pdbs[0])).read().split("\n")
                     if ln[:6] in ("ATOM  ", "HETATM")] if pdbs else []
        fixtures.append(dict(name=name, ion=GROUPS[m.group(1)], q=q, I=I, sigma=s, state=doc,
                             pdb_name=pdbs[0] if pdbs else None, pdb_lines=pdb_lines, **st))
    json.dump(dict(ions=ions, fixtures=fixtures), open(os.path.join(HERE, "single_atom.json"), "w"))

    pts = []
    for name in ("points_explicit_Vacuum", "points_explicit_SS334"):
        d = os.path.join(FIX, name)
        st = read_state(os.path.join(d, name + ".state"))
        q, I, s = read_out(os.path.join(d, name + "TestStandard.out"))
        atoms = []
        for line in open(os.path.join(d, "points_explicit.pdb")):
            if line.startswith("ATOM"):
                atoms.append([line[76:78].strip(), float(line[30:38]) / 10, float(line[38:46]) / 10,
                              float(line[46:54]) / 10])
        pts.append(dict(name=name, atoms=atoms, q=q, I=I, sigma=s, **st))
    json.dump(pts, open(os.path.join(HERE, "points.json"), "w"))
    print("wrote", len(fixtures), "single-atom fixtures,", sum(len(v) for v in idx.values()), "grid cells")


if __name__ == "__main__":
    main()
