"""PDB files as D+ reads them for X-ray scattering (PDBReaderOb::readPDBstream,
PDBReaderLib/PDBReaderLib.cpp:815-1051):

* ATOM / HETATM records; alternate locations other than ' ' and 'A' are
  skipped (column 17); with ``model`` > 0 only that MODEL block is read;
* coordinates from columns 31-54 in Angstrom, stored in nm; occupancy and
  B factor from columns 55-66;
* the ion from columns 77-80 (element and charge, e.g. " N1+"), or, when those
  are blank, from the atom-name columns 13-14 with a leading digit dropped;
* residues (runs of equal residue number and name) that carry no hydrogen
  atom get implicit-hydrogen groups (ChangeResidueGroupsToImplicit,
  PDBReaderLib.cpp:1533-1757, pH 7.4): CA of alanine becomes a CH, its CB a
  CH3, and so on for the 20 amino acids (and selenocysteine) and the RNA / DNA
  nucleotides.  A residue with an atom the table does not know keeps its
  explicit atoms; OXT stays an oxygen.

The ions are named by this package's element table (``dpx.elements``):
element symbols ("C", "MG") and groups ("CH2", "NH3").
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .elements import IONS

# Implicit-hydrogen groups per residue: atom label (digits removed except in
# trp, ile and the one- and two-letter nucleotides) -> group ("" = keep the
# element).  The table is data: the same groups give the same form factors.
_BACKBONE = "n:nh ca:ch c: o:"
_SUGAR_RNA = ("p: op1: op2: op: op3: o5': c5':ch2 c4':ch o4': c3':ch o3': c2':ch o2':oh c1':ch")
_SUGAR_DNA = ("p: op1: op2: op: op3: o5': c5':ch2 o4': c4':ch o3': c3':ch c2':ch2 c1':ch")
_PURINE_A = "n9: c8:ch n7: c6: c5: n6:nh2 n1: c2:ch n3: c4:"
_PYR_U = "n1: c2: o2: n3:nh c4: o4: c5:ch c6:ch"
_PYR_C = "n1: c2: o2: n3: c4: n4:nh2 c5:ch c6:ch"
_PURINE_G = "n9: c8:ch n7: c5: c6: o6: n1:nh c2: n2:nh2 n3: c4:"
_PYR_T = "n1: c2: o2: n3:nh c4: o4: c5: c7:ch3 c6:ch"

_RESIDUES = {
    "arg": _BACKBONE + " cb:ch2 cg:ch2 cd:ch2 ne:nh cz: nh:nh2",
    "his": _BACKBONE + " cb:ch2 cg: nd:nh cd:ch ce:ch ne:nh",
    "lys": _BACKBONE + " cb:ch2 cg:ch2 cd:ch2 ce:ch2 nz:nh3",
    "asp": _BACKBONE + " cb:ch2 cg: od:",
    "glu": _BACKBONE + " cb:ch2 cg:ch2 cd: oe:",
    "ser": _BACKBONE + " cb:ch2 og:oh",
    "thr": _BACKBONE + " cb:ch cg:ch3 og:oh",
    "asn": _BACKBONE + " cb:ch2 cg: od: nd:nh2",
    "gln": _BACKBONE + " cb:ch2 cg:ch2 cd: oe: ne:nh2",
    "cys": _BACKBONE + " cb:ch2 sg:sh",
    "sec": _BACKBONE + " cb:ch2 seg:",
    "gly": "n:nh ca:ch2 c: o:",
    "pro": "n: ca:ch c: o: cb:ch2 cg:ch2 cd:ch2",
    "ala": _BACKBONE + " cb:ch3",
    "val": _BACKBONE + " cb:ch cg:ch3",
    "ile": _BACKBONE + " cb:ch cg1:ch2 cg2:ch3 cd1:ch3 cd:ch3",
    "leu": _BACKBONE + " cb:ch2 cg:ch cd:ch3",
    "met": _BACKBONE + " cb:ch2 cg:ch2 sd: ce:ch3",
    "phe": _BACKBONE + " cb:ch2 cg: cd:ch ce:ch cz:ch",
    "tyr": _BACKBONE + " cb:ch2 cg: cd:ch ce:ch cz: oh:oh",
    "trp": _BACKBONE + " cb:ch2 cg: cd1:ch cd2: ne1:nh ce2: ce3:ch cz2:ch cz3:ch ch2:ch",
    "a": _SUGAR_RNA + " " + _PURINE_A,
    "u": _SUGAR_RNA + " " + _PYR_U,
    "c": _SUGAR_RNA + " " + _PYR_C,
    "g": _SUGAR_RNA + " " + _PURINE_G,
    "t": _SUGAR_RNA + " " + _PYR_T,
    "da": _SUGAR_DNA + " " + _PURINE_A,
    "du": _SUGAR_DNA + " " + _PYR_U,
    "dc": _SUGAR_DNA + " " + _PYR_C,
    "dg": _SUGAR_DNA + " " + _PURINE_G,
    "dt": _SUGAR_DNA + " " + _PYR_T,
}
IMPLICIT_GROUPS = {res: dict(tuple(p.split(":")) for p in spec.split()) for res, spec in _RESIDUES.items()}

# ion strings of columns 77-80 that name the same form factor as the neutral
# atom (getAtomIonIndices, PDBReaderLib.cpp:1971-2194: " n1+" and " n+1" are
# nitrogen's row)
_SAME_AS_NEUTRAL = {" n1+": "N", " n+1": "N"}


@dataclass
class PdbAtoms:
    symbols: list              # ion per atom, in file order ("C", "CH2", ...)
    xyz: np.ndarray            # [n, 3] nm, float64 as read
    bfactor: np.ndarray        # [n]
    occupancy: np.ndarray      # [n]
    atom_names: list = field(default_factory=list)
    res_names: list = field(default_factory=list)
    implicit_atoms: int = 0     # atoms in residues given implicit hydrogens
    implicit_residues: int = 0


def _ion_string(line: str) -> str:
    """The 4-character ion field (element + charge) of an ATOM record."""
    last = line[76:80] if len(line) > 76 else ""
    if not last.strip():
        last = ""
    n = len(last)
    if n == 4 and last[3] == "\r":
        last = last[:3] + " "
    if n in (3, 4) and last[2] == "\r":
        last = last[:2] + "  "
    elif n == 2:
        last = last + "  "
    elif n == 0:
        last = line[12:14] + "  "
        if last[0].isdigit():
            last = " " + last[1:]
    return last


def _symbol(key: str) -> str:
    """This package's ion name for a 4-character ion field or a group name."""
    k = key[:2].lower() + key[2:]
    if k in _SAME_AS_NEUTRAL:
        return _SAME_AS_NEUTRAL[k]
    sym = k[:2].strip().upper()
    if len(k) == 4 and k[2:] == "  " and sym in IONS:
        return sym
    raise KeyError(f"no form-factor entry for the ion {key!r}")


def _implicit(res: str, names: list) -> list | None:
    """Group per atom of one residue, or None when the residue keeps its atoms."""
    table = IMPLICIT_GROUPS.get(res.replace(" ", "").lower())
    if table is None:
        return None
    r = res.replace(" ", "").lower()
    keep_digits = r in ("trp", "ile") or len(r) < 3
    out = []
    for name in names:
        label = "".join(ch for ch in name if not ch.isspace())
        if not keep_digits:
            label = "".join(ch for ch in label if not ch.isdigit())
        label = label.lower()
        if label == "oxt":
            out.append("")
            continue
        if label not in table:
            return None
        out.append(table[label])
    return out


def read_pdb(path_or_lines, model: int = 0) -> PdbAtoms:
    """Atoms of a PDB file (path, or an iterable of lines) as D+ reads them."""
    if isinstance(path_or_lines, str):
        with open(path_or_lines, newline="") as f:
            lines = f.read().split("\n")
    else:
        lines = [ln.rstrip("\n") for ln in path_or_lines]
    keys, xyz, bf, occ, names, resn, resno = [], [], [], [], [], [], []
    ignore = False
    for line in lines:
        tag = line[0:6]
        if tag in ("ATOM  ", "HETATM"):
            if ignore:
                continue
            alt = line[16:18]
            if alt and alt[0] not in (" ", "A"):
                continue
            keys.append(_ion_string(line))
            xyz.append((float(line[30:38]) / 10.0, float(line[38:46]) / 10.0, float(line[46:54]) / 10.0))
            occ.append(float(line[54:60] or 0.0) if line[54:60].strip() else 0.0)
            bf.append(float(line[60:66]) if line[60:66].strip() else 0.0)
            names.append(line[12:16])
            resn.append(line[17:20])
            resno.append(line[22:26])
        elif tag == "MODEL ":
            if model > 0 and int(line[10:14]) != model:
                ignore = True
        elif tag == "ENDMDL":
            ignore = False
    if not keys:
        raise ValueError("no ATOM / HETATM records")
    groups = [""] * len(keys)
    n_imp = n_res = 0
    i = 0
    while i < len(keys):
        j = i
        has_h = False
        while j < len(keys) and resno[j] == resno[i] and resn[j] == resn[i]:
            has_h |= keys[j] in (" H  ", " h  ")
            j += 1
        if not has_h:
            g = _implicit(resn[i], names[i:j])
            if g is not None:
                groups[i:j] = g
                n_imp += j - i
                n_res += 1
        i = j
    symbols = [g.upper() if g else _symbol(k) for g, k in zip(groups, keys)]
    return PdbAtoms(symbols, np.array(xyz, dtype=np.float64), np.array(bf), np.array(occ), names, resn, n_imp, n_res)
