"""JSON state decoding on the CPU: preferences, populations, nested manual
symmetries flattened into composed copies, the PDB reader, rejected types."""
import json
import math

import numpy as np
import pytest

from dpx import models as M
from dpx import state as S


def _pdb(path, atoms):
    with open(path, "w") as f:
        for k, (el, x, y, z) in enumerate(atoms):
            f.write("ATOM  %5d  %-3s ALA A   1    %8.3f%8.3f%8.3f  1.00  0.00          %2s\n"
                    % (k + 1, el, x, y, z, el))
        f.write("END\n")


def _node(t, **kw):
    d = {"Type": t, "Location": {"x": 0, "y": 0, "z": 0, "alpha": 0, "beta": 0, "gamma": 0}, "Use_Grid": True}
    d.update(kw)
    return d


def _state(models, method="Monte Carlo (Mersenne Twister)", pops=None):
    return {"DomainPreferences": {"GridSize": 24, "qMax": 4.0, "OrientationMethod": method,
                                  "OrientationIterations": 1000, "Convergence": 0.001, "UseGrid": False},
            "Domain": {"Scale": 2.0, "Constant": 0.5,
                       "Populations": pops or [{"PopulationSize": 1.5, "Models": models}]}}


def test_read_pdb(tmp_path):
    p = str(tmp_path / "a.pdb")
    _pdb(p, [("C", 1.0, 2.0, 3.0), ("N", -1.5, 0.0, 10.0), ("S", 0.0, 0.0, 0.0)])
    syms, xyz = S.read_pdb(p)
    assert syms == ["C", "N", "S"] and np.allclose(xyz[1], [-0.15, 0.0, 1.0])


def test_nested_manual_symmetry_is_flattened(tmp_path):
    p = str(tmp_path / "sub.pdb")
    _pdb(p, [("C", 0, 0, 0), ("O", 1.2, 0, 0)])
    leaf = _node("PDB", Filename="C:\\\\x\\\\sub.pdb", Centered=False,
                 ExtraParameters=[1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
    leaf["Location"].update(x=0.1, alpha=0.3)
    inner = _node(",26", Parameters=[[1, 0, 0, 0, 0, 90], [0, 2, 0, 30, 0, 0], [0, 0, 3, 0, 45, 0]],
                  ExtraParameters=[0.5], Children=[leaf])
    outer = _node(",26", Parameters=[[0, 0, 0, 0, 0, 0], [5, 0, 0, 0, 0, 180]], ExtraParameters=[2.0],
                  Children=[inner])
    outer["Location"].update(z=1.0, gamma=0.2)
    job = S.decode(_state([outer]), base_dir=str(tmp_path))
    assert (job.grid_size, job.qmax, job.method, job.scale, job.constant) == (24, 4.0, "MC", 2.0, 0.5)
    (w, amps), = job.populations
    assert w == 1.5 and len(amps) == 1
    ms = amps[0]
    assert isinstance(ms, M.ManualSymmetry) and len(ms.trans) == 6 and abs(ms.scale - 1.0) < 1e-15
    assert ms.child.location == (0.1, 0.0, 0.0, 0.3, 0.0, 0.0)
    # copy (outer o, inner i): R = Rn Ro Ri with the outer node's placement Rn, t = Rn(Ro ti + to) + tn
    Rn, tn = S._euler_matrix(0, 0, 0.2), np.array([0, 0, 1.0])
    k = 0
    for o in ([0, 0, 0, 0, 0, 0], [5, 0, 0, 0, 0, 180]):
        Ro = S._euler_matrix(*np.radians(o[3:]))
        for i in ([1, 0, 0, 0, 0, 90], [0, 2, 0, 30, 0, 0], [0, 0, 3, 0, 45, 0]):
            Ri = S._euler_matrix(*np.radians(i[3:]))
            R = Rn @ Ro @ Ri
            t = Rn @ (Ro @ np.array(i[:3], float) + np.array(o[:3], float)) + tn
            assert np.allclose(S._euler_matrix(*ms.rot[k]), R, atol=1e-12)
            assert np.allclose(ms.trans[k], t, atol=1e-12)
            k += 1


def test_methods_populations_and_rejections(tmp_path):
    p = str(tmp_path / "s.pdb")
    _pdb(p, [("C", 0, 0, 0)])
    leaf = _node("PDB", Filename=p, Centered=True, ExtraParameters=[1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
    pops = [{"PopulationSize": 1, "Models": [leaf]}, {"PopulationSize": 3, "Models": [leaf]}]
    job = S.decode(json.dumps({"state": _state(None, "Adaptive (VEGAS) Monte Carlo", pops), "x": [0.1, 0.2]}))
    assert job.method == "VEGAS" and [w for w, _ in job.populations] == [1.0, 3.0]
    assert np.array_equal(job.q, [0.1, 0.2])
    assert S.decode(_state([leaf], "Adaptive Gauss Kronrod")).method == "GK"
    with pytest.raises(NotImplementedError):
        S.decode(_state([_node(",2", Parameters=[[1, 333]])]))
    with pytest.raises(ValueError):  # a scripted symmetry without its script
        S.decode(_state([_node("Scripted Symmetry", Children=[leaf])]))
    with pytest.raises(FileNotFoundError):
        S.decode(_state([_node("PDB", Filename="nowhere.pdb")]), base_dir=str(tmp_path))


def test_space_filling_rows(tmp_path):
    p = str(tmp_path / "s.pdb")
    _pdb(p, [("C", 0, 0, 0), ("N", 1, 0, 0)])
    leaf = _node("PDB", Filename=p, ExtraParameters=[1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
    sf = _node(",25", Parameters=[[3.0, 90, 2], [3.5, 80, 3], [4.0, 100, 4]], ExtraParameters=[0.7], Children=[leaf])
    (w, amps), = S.decode(_state([sf])).populations
    ref = M.SpaceFillingSymmetry([], 3.0, 3.5, 4.0, 90, 80, 100, 2, 3, 4)
    assert np.allclose(amps[0].lattice, ref.lattice) and amps[0].scale == 0.7 and math.isclose(w, 1.5)


def test_grid_subtree_stays_one_assembly_grid(tmp_path):
    """As the reference's hybrid FlattenTree: a symmetry whose subtree uses grids
    is one assembly grid; a symmetry above it that does not use grids docks
    that grid per orientation; with grids all the way up, grid of grid."""
    p = str(tmp_path / "sub.pdb")
    _pdb(p, [("C", 0, 0, 0), ("O", 1.2, 0, 0)])
    leaf = _node("PDB", Filename=p, ExtraParameters=[1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
    inner = _node(",26", Parameters=[[-4, -2, -8.13, 90, 0, 0]], ExtraParameters=[1], Children=[leaf])
    for outer_grid in (False, True):
        outer = _node(",26", Parameters=[[0, 0, 0, 0, 0, 0], [4, 0, 0, 0, 0, 0], [8, 0, 0, 0, 0, 0]],
                      ExtraParameters=[1], Children=[inner], Use_Grid=outer_grid)
        st = _state([outer])
        st["DomainPreferences"]["UseGrid"] = True
        (w, amps), = S.decode(st, base_dir=str(tmp_path)).populations
        ms, = amps
        assert isinstance(ms, M.ManualSymmetry) and ms.use_grid is outer_grid and len(ms.trans) == 3
        assert isinstance(ms.child, M.ManualSymmetry) and ms.child.use_grid and len(ms.child.trans) == 1
        assert isinstance(ms.child.child, M.PDBAmplitude)
        assert np.allclose(ms.child.trans[0], [-4, -2, -8.13]) and np.allclose(ms.child.rot[0], [np.pi / 2, 0, 0])
        assert np.allclose(ms.trans[:, 0], [0, 4, 8])


def test_reference_single_atom_states_decode():
    """The reference's own single-atom state documents (generate/cpu/short/
    {c,n,o,h}_explicit_*, {ch,...,oh}_implicit_*, kept in tests/golden with their
    one-atom PDB records) decode to the grid, method and leaf they describe."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "single_atom.json")) as f:
        fixtures = json.load(f)["fixtures"]
    assert len(fixtures) == 22
    for fx in fixtures:
        job = S.decode(fx["state"], files={fx["pdb_name"]: fx["pdb_lines"]})
        assert (job.grid_size, job.qmax, job.convergence) == (fx["gridSize"], fx["qMax"], fx["convergence"])
        assert job.method == S.METHODS[fx["method"]]
        (w, amps), = job.populations
        leaf, = amps
        assert isinstance(leaf, M.PDBAmplitude) and leaf.symbols == [fx["ion"]], fx["name"]
        e = fx["extra"]
        assert (leaf.scale, leaf.solventED, leaf.c1, leaf.outerSolventED) == (e[0], e[1], e[2], e[6])
        if fx["centered"]:
            assert np.allclose(leaf.xyz, 0.0)
