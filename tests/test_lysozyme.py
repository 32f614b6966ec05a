"""The reference's lysozyme example on the CPU: D+'s PDB reading (implicit
hydrogen groups) and the oracle's Debye sum against the reference's own
DebyeCalculator output (tests/golden/lysozyme.json, made by make_lysozyme.py)."""
import json
import os

import numpy as np
import pytest

from dpx import models as M
from dpx import pdb as P
import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lysozyme.json")


@pytest.fixture(scope="module")
def lyz():
    with open(GOLD) as f:
        return json.load(f)


def leaf_of(gold, extra=(1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0), centered=False):
    a = P.read_pdb(gold["pdb_lines"])
    return M.PDBAmplitude(a.symbols, a.xyz, list(extra), centered=centered, bfactors=a.bfactor)


def test_reader_implicit_hydrogen_groups_as_the_reference_reports(lyz):
    """The reference printed "1001 of 1102 atoms are treated as having implicit
    hydrogen atoms (129 amino acids)" for this file."""
    a = P.read_pdb(lyz["pdb_lines"])
    imp = lyz["implicit"]
    assert (len(a.symbols), a.implicit_atoms, a.implicit_residues) == (imp["total"], imp["atoms"], imp["residues"])
    # waters (HOH) are not amino acids and keep their oxygens
    assert all(s == "O" for s, r in zip(a.symbols, a.res_names) if r == "HOH")
    assert {"CH", "CH2", "CH3", "NH", "NH2", "NH3", "OH", "SH"} <= set(a.symbols)


def test_oracle_debye_matches_the_reference_debye_calculator(lyz):
    """FP64 oracle Debye sum of 1lyz (no solvent) against the reference's CPU
    DebyeCalculator output: within its 6-digit printing (5e-6) at the q grid it
    computed on; the printed q agree with that grid to their 6 digits."""
    g = lyz["debye"]
    q = g["qmin"] + (g["qmax"] - g["qmin"]) * np.arange(g["n"]) / (g["n"] - 1)
    assert np.abs(q - np.array(g["q"])).max() <= 5e-6
    s = O.Struct.from_pdb(leaf_of(lyz))
    I = O.debye(s, q, mode=O.FP64)
    assert np.abs(I / np.array(g["I"]) - 1).max() <= 6e-6
    # the reference-exact (float pair terms) restatement stays within 2e-5
    Iref = O.debye(s, q, mode=O.REFEXACT)
    assert np.abs(Iref / np.array(g["I"]) - 1).max() <= 2e-5


def _rec(serial, name, res, resno, x, el, alt=" ", tag="ATOM  "):
    return "%s%5d %-4s%s%3s A%4d    %8.3f%8.3f%8.3f  1.00 10.00          %2s  " % (
        tag, serial, name, alt, res, resno, x, 0.0, 0.0, el)


def test_reader_rules():
    lines = [
        _rec(1, " N  ", "GLY", 1, 0.0, " N"), _rec(2, " CA ", "GLY", 1, 1.0, " C"),
        _rec(3, " C  ", "GLY", 1, 2.0, " C"), _rec(4, " O  ", "GLY", 1, 3.0, " O"),
        _rec(5, " OXT", "GLY", 1, 4.0, " O"),
        # alternate location B is skipped, A is kept
        _rec(6, " CA ", "ALA", 2, 5.0, " C", alt="B"), _rec(7, " CA ", "ALA", 2, 5.5, " C", alt="A"),
        _rec(8, " CB ", "ALA", 2, 6.0, " C"),
        # a residue with an explicit hydrogen keeps all its atoms
        _rec(9, " CA ", "SER", 3, 7.0, " C"), _rec(10, " HA ", "SER", 3, 8.0, " H"),
        # an atom the table does not know keeps the residue explicit
        _rec(11, " CA ", "VAL", 4, 9.0, " C"), _rec(12, " XX ", "VAL", 4, 10.0, " C"),
        # blank element columns: the element comes from the atom name, a leading digit dropped
        _rec(13, " CA ", "LEU", 5, 11.0, "  ")[:76], _rec(14, "1HB ", "XYZ", 6, 12.0, "  ")[:76],
    ]
    a = P.read_pdb(lines)
    assert a.symbols == ["NH", "CH2", "C", "O", "O", "CH", "CH3", "C", "H", "C", "C", "CH", "H"]
    assert (a.implicit_atoms, a.implicit_residues) == (8, 3)
    assert np.allclose(a.xyz[:, 0], [0, .1, .2, .3, .4, .55, .6, .7, .8, .9, 1.0, 1.1, 1.2])
    assert np.allclose(a.bfactor, 10.0)
    with pytest.raises(KeyError):  # no form-factor row for a charged ion this package does not carry
        P.read_pdb([_rec(1, "FE  ", "HEM", 1, 0.0, "FE")[:78] + "2+"])
    # MODEL selection
    m = ["MODEL        1", _rec(1, " O  ", "HOH", 1, 0.0, " O"), "ENDMDL",
         "MODEL        2", _rec(2, " O  ", "HOH", 1, 5.0, " O"), "ENDMDL"]
    assert len(P.read_pdb(m).symbols) == 2 and np.allclose(P.read_pdb(m, model=2).xyz[:, 0], [0.5])
