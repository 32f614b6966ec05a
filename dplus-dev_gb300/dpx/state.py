"""D+'s JSON state (the document the Python API and the GUI send, see
BackendWrapper::StartGenerate, Backend/Backend/BackendWrapper.cpp:313-374, and
the parameter tree, Backend/Backend/LocalBackendParameterTree.cpp:117-272)
decoded into this package's model tree, for the scattering path:

* ``DomainPreferences``: grid size, qmax, orientation method, iterations,
  convergence, use of grids;
* ``Domain``: ``Scale``, ``Constant`` and ``Populations`` (each with its
  ``PopulationSize``); I(q) = Scale * sum_p PopulationSize_p I_p(q) + Constant
  (CompositeModel::CalculateVector, Backend/Backend/CompositeModel.cpp:165-176);
* model nodes: ``PDB`` (a PDB file: ExtraParameters, Centered, Location),
  ``AMP`` (an amplitude-grid file, ExtraParameters [scale]), ``,26``
  ManualSymmetry (rows x, y, z, alpha, beta, gamma in degrees; scale),
  ``Scripted Symmetry`` (a Lua script whose Populate(p, nlayers) gives those
  rows, run by dpx.lua; LuaSymmetry, Backend/Backend/Symmetry.cpp:404-521) and
  ``,25`` space-filling symmetry (three rows of distance, angle, repetitions).

Nested symmetry nodes are flattened (FlattenTree, Backend/Backend/
Amplitude.cpp:577-691): every leaf gets the composition of the symmetry copies
and node placements above it.  Geometric form-factor models and electron PDBs
are outside the scattering path and are rejected.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib
from . import lua as L
from . import models as M
from . import pdb as P

METHODS = {"Monte Carlo (Mersenne Twister)": "MC", "Adaptive (VEGAS) Monte Carlo": "VEGAS",
           "Adaptive Gauss Kronrod": "GK"}


def _euler_matrix(a, b, c):
    """Tait-Bryan X1Y2Z3 rotation (the reference's EulerD), radians."""
    c1, s1, c2, s2, c3, s3 = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
    return np.array([[c2 * c3, -c2 * s3, s2], [c1 * s3 + c3 * s1 * s2, c1 * c3 - s1 * s2 * s3, -c2 * s1],
                     [s1 * s3 - c1 * c3 * s2, c3 * s1 + c1 * s2 * s3, c1 * c2]])


def _euler_angles(R):
    b = math.asin(max(-1.0, min(1.0, R[0, 2])))
    if abs(R[0, 2]) > 1.0 - 1e-12:
        return math.atan2(R[2, 1], R[1, 1]), b, 0.0
    return math.atan2(-R[1, 2], R[2, 2]), b, math.atan2(-R[0, 1], R[0, 0])


def read_pdb(path: str):
    """(ions, xyz in nm) of a PDB file as D+ reads it (``dpx.pdb.read_pdb``:
    alternate locations, element and charge columns, implicit-hydrogen groups)."""
    atoms = P.read_pdb(path)
    return atoms.symbols, atoms.xyz


def _location(node):
    loc = node.get("Location", {})
    return tuple(float(loc.get(k, 0.0)) for k in ("x", "y", "z", "alpha", "beta", "gamma"))


def _transform(loc):
    """(R, t) of a location (x, y, z nm, alpha, beta, gamma radians)."""
    return _euler_matrix(loc[3], loc[4], loc[5]), np.array(loc[:3], dtype=np.float64)


@dataclass
class Job:
    """A decoded state: grid and orientation settings plus populations."""
    grid_size: int
    qmax: float
    method: str
    iterations: int
    convergence: float
    use_grid: bool
    scale: float
    constant: float
    populations: list = field(default_factory=list)  # [(weight, [amplitudes])]
    q: np.ndarray | None = None  # the request's q values ("x"), when the document carries them

    def domain_models(self, precision=M.FP32):
        return [(w, M.DomainModel(amps, self.grid_size, self.qmax, precision)) for w, amps in self.populations]

    def intensity(self, ctx, Q, dirs=None, precision=M.FP32, seed=0, points_per_iter=4096,
                  iterations: int | None = None, mc_rule: str = "cpu"):
        """I(q) of the state (MC needs the direction set, as dpx's averages take
        directions explicitly).  ``mc_rule`` picks the Monte Carlo convergence
        test: "cpu" (the reference's CPU rule) or "gpu" (its GPU averages'
        rule: 8192 samples a step on the grid path, 4096 on the hybrid path)."""
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        n = self.iterations if iterations is None else int(iterations)
        total = np.zeros(len(Q))
        for w, dom in self.domain_models(precision):
            if self.method == "MC":
                if dirs is None:
                    raise ValueError("Monte Carlo needs a direction set")
                if mc_rule == "gpu":
                    hybrid = any(isinstance(a, M.ManualSymmetry) and not a.use_grid for a in dom.amps)
                    ctx.set_convergence(_lib.DPX_CONV_GPU, 4096 if hybrid else 8192)
                try:
                    I = dom.CalculateIntensityVector(ctx, Q, self.convergence, min(n, len(dirs)), dirs)
                finally:
                    if mc_rule == "gpu":
                        ctx.set_convergence(_lib.DPX_CONV_CPU)
            elif self.method == "VEGAS":
                I = dom.CalculateIntensityVector(ctx, Q, self.convergence, n, method="VEGAS", seed=seed,
                                                 points_per_iter=points_per_iter)
            else:
                I = dom.CalculateIntensityVector(ctx, Q, self.convergence, n, method="GK")
            total += w * I
        return self.scale * total + self.constant


class _Decoder:
    def __init__(self, base_dir, files, use_grid):
        self.base_dir = base_dir
        self.files = files or {}
        self.use_grid = use_grid

    def resolve(self, filename):
        base = os.path.basename(filename.replace("\\", "/"))
        if base in self.files:
            return self.files[base]
        for cand in (filename, os.path.join(self.base_dir or "", base)):
            if cand and os.path.exists(cand):
                return cand
        raise FileNotFoundError(f"model file {filename!r} (looked for {base!r} in {self.base_dir!r})")

    def leaf(self, node):
        t = node.get("Type")
        if t == "PDB":
            atoms = P.read_pdb(self.resolve(node["Filename"]))
            extra = list(node.get("ExtraParameters", [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0]))
            return M.PDBAmplitude(atoms.symbols, atoms.xyz, extra, centered=bool(node.get("Centered", False)),
                                  location=_location(node), bfactors=atoms.bfactor)
        if t == "AMP":
            extra = node.get("ExtraParameters", [1])
            return M.AmpGridAmplitude(self.resolve(node["Filename"]), scale=float(extra[0] if extra else 1.0),
                                      location=_location(node))
        raise NotImplementedError(f"model type {t!r} is outside the scattering path (geometric form factors "
                                  "and electron PDBs are not carried)")

    def grid_subtree(self, node) -> bool:
        """The node and every node under it use grids (the reference's
        GetUseGridWithChildren); with the preferences' UseGrid off nothing does."""
        return (self.use_grid and bool(node.get("Use_Grid", True))
                and all(self.grid_subtree(c) for c in node.get("Children", [])))

    def node(self, node, copies=None):
        """Amplitudes of one node; ``copies`` = [(R, t)] applied above it.

        As the reference's hybrid FlattenTree (Backend/Backend/Amplitude.cpp:
        577-691) does, a ManualSymmetry whose subtree uses grids stays one
        object: its assembly grid (ManualSymmetry::calculateGrid over its
        children's grids, Symmetries.cpp:879-962); the copies above it dock that
        grid per orientation.  A symmetry that does not use grids is flattened:
        its rows (and its own placement) compose into the copies of its
        children."""
        t = node.get("Type")
        if t in (",26", "Scripted Symmetry"):
            if t == ",26":
                rows = np.asarray(node.get("Parameters", []), dtype=np.float64).reshape(-1, 6)
            else:  # the script's Populate(p, nlayers) gives the rows (LuaSymmetry, Symmetry.cpp:463-521)
                if not node.get("Filename"):
                    raise ValueError("a scripted symmetry needs its script (Filename)")
                script = self.resolve(node["Filename"])  # a path, or the text given in ``files``
                if isinstance(script, (list, tuple)):
                    script = "\n".join(script)
                elif os.path.exists(script):
                    with open(script) as f:
                        script = f.read()
                params = node.get("Parameters", [])
                rows = L.populate(script, params, int(node.get("nLayers", len(params))))
            Rn, tn = _transform(_location(node))
            scale = float((node.get("ExtraParameters") or [1.0])[0])
            mine = []
            for r in rows:
                Rr = _euler_matrix(*np.radians(r[3:6]))
                mine.append((Rn @ Rr, Rn @ r[:3] + tn))
            if self.grid_subtree(node):
                # one assembly grid of this node's rows over each child's grid
                out = []
                for child in node.get("Children", []):
                    for kid in self.node(child, None):
                        g = M.ManualSymmetry(kid, _rows(mine), scale=scale, use_grid=True)
                        out.append(g if copies is None else
                                   M.ManualSymmetry(g, _rows(copies), scale=1.0, use_grid=False))
                return out
            composed = mine if copies is None else [(Ro @ Ri, Ro @ ti + to) for Ro, to in copies for Ri, ti in mine]
            out = []
            for child in node.get("Children", []):
                for a in self.node(child, composed):
                    out.append(a if scale == 1.0 else _scaled(a, scale))
            return out
        if t == ",25":  # space-filling symmetry of its children (grid path)
            rows = np.asarray(node.get("Parameters", []), dtype=np.float64).reshape(3, 3)
            scale = float((node.get("ExtraParameters") or [1.0])[0])
            kids = []
            for child in node.get("Children", []):
                kids += self.node(child, None)
            sf = M.SpaceFillingSymmetry(kids, rows[0, 0], rows[1, 0], rows[2, 0], rows[0, 1], rows[1, 1],
                                        rows[2, 1], rows[0, 2], rows[1, 2], rows[2, 2], scale=scale,
                                        location=_location(node))
            if copies is not None:
                raise NotImplementedError("a space-filling symmetry inside a manual symmetry is not carried")
            return [sf]
        leaf = self.leaf(node)
        if copies is None:
            return [leaf]
        if isinstance(leaf, M.AmpGridAmplitude):
            raise NotImplementedError("docked copies of an amplitude-file leaf are not carried")
        # copies reach a leaf only from symmetries that do not use grids: the
        # leaf's grid is docked per orientation
        return [M.ManualSymmetry(leaf, _rows(copies), scale=1.0, use_grid=False)]


def _rows(copies):
    """ManualSymmetry rows (x, y, z nm, alpha, beta, gamma degrees) of [(R, t)]."""
    rows = []
    for R, tt in copies:
        a, b, c = _euler_angles(R)
        rows.append([tt[0], tt[1], tt[2], math.degrees(a), math.degrees(b), math.degrees(c)])
    return rows


def _scaled(a, s):
    if isinstance(a, M.ManualSymmetry):
        a.scale *= s
        return a
    raise NotImplementedError("a symmetry scale over a non-symmetry node is not carried")


def decode(state, base_dir: str | None = None, files: dict | None = None) -> Job:
    """A Job from a state dict (or a path / JSON string).  Model files are found
    by basename in ``files``, then at their stored path, then in ``base_dir``."""
    if isinstance(state, str):
        if os.path.exists(state):
            base_dir = base_dir or os.path.dirname(os.path.abspath(state))
            with open(state) as f:
                state = json.load(f)
        else:
            state = json.loads(state)
    q = None
    if "state" in state and "Domain" not in state:
        q = state.get("x")
        state = state["state"]
    prefs = state.get("DomainPreferences", {})
    dom = state["Domain"]
    method = METHODS.get(prefs.get("OrientationMethod", "Monte Carlo (Mersenne Twister)"))
    if method is None:
        raise NotImplementedError(f"orientation method {prefs.get('OrientationMethod')!r}")
    use_grid = bool(prefs.get("UseGrid", True))
    job = Job(grid_size=int(prefs.get("GridSize", 100)), qmax=float(prefs.get("qMax", 7.5)), method=method,
              iterations=int(prefs.get("OrientationIterations", 1_000_000)),
              convergence=float(prefs.get("Convergence", 0.001)), use_grid=use_grid,
              scale=float(dom.get("Scale", 1.0)), constant=float(dom.get("Constant", 0.0)),
              q=None if q is None else np.asarray(q, dtype=np.float64))
    dec = _Decoder(base_dir, files, use_grid)
    for pop in dom.get("Populations", []):
        amps = []
        for model in pop.get("Models", []):
            amps += dec.node(model)
        job.populations.append((float(pop.get("PopulationSize", 1.0)), amps))
    return job
