"""Seeded synthetic workloads of the scattering path (no dataset exists for it).

* ``batch_mix`` — independent solves of uneven size: atom counts log-uniform
  in [500, 200,000], globule radius 2.5 nm x (N / 2000)^(1/3), qmax uniform in
  [2, 10] nm^-1, radial layers uniform in [40, 250], half of them with
  dummy-atom solvent (333 e/nm^3), the rest in vacuum.
* ``request_stream`` — a Poisson stream of I(q) requests for the serving
  engine (see ``dpx.serve``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import models as M

SOLVENT = [1, 333, 1, 0.05, 0.14, 0.28, 0, 0, 0, 4]  # scale, solventED, c1, ..., radType 4 (dummy atoms)
VACUUM = [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0]


def globule_radius(n_atoms: int) -> float:
    """Radius (nm) of an n-atom globule: 2.5 nm at 2,000 atoms, R ~ N^(1/3)."""
    return 2.5 * (n_atoms / 2000.0) ** (1.0 / 3.0)


@dataclass
class SolveSpec:
    atoms: int
    qmax: float
    layers: int
    solvent: bool
    seed: int

    @property
    def grid_size(self) -> int:
        return 2 * self.layers

    def cells(self) -> int:
        lp = self.layers + 3
        return 6 * lp * (lp + 1) ** 2 + 1

    def pairs(self) -> float:
        return float(self.atoms) * self.cells()

    def leaf(self) -> M.PDBAmplitude:
        sym, xyz = M.make_globule(self.atoms, globule_radius(self.atoms), self.seed)
        return M.PDBAmplitude(sym, xyz, SOLVENT if self.solvent else VACUUM)


def batch_mix(n: int = 512, seed: int = 3003, n_min: int = 500, n_max: int = 200_000) -> list:
    rng = np.random.default_rng(seed)
    atoms = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n))).astype(int)
    qmax = rng.uniform(2.0, 10.0, n)
    layers = rng.integers(40, 251, n)
    solvent = rng.permutation(np.arange(n) < n // 2)
    return [SolveSpec(int(a), float(q), int(l), bool(s), seed * 1000 + j)
            for j, (a, q, l, s) in enumerate(zip(atoms, qmax, layers, solvent))]
