"""Seeded synthetic workloads of the scattering path (no dataset exists for it).

* ``batch_mix`` — independent solves of uneven size: atom counts log-uniform
  in [500, 200,000], globule radius 2.5 nm x (N / 2000)^(1/3), qmax uniform in
  [2, 10] nm^-1, radial layers uniform in [40, 250], half of them with
  dummy-atom solvent (333 e/nm^3), the rest in vacuum.
* ``icosahedral_rotations`` / ``helix_copies`` — docked-assembly placements:
  the 60 rotations of the icosahedral group with translations R_k (0, 0, r),
  and helical copies (radius, copies per turn, rise per turn) each with its own
  seeded rotation.
* ``request_stream`` — a Poisson stream of I(q) requests for the serving
  engine (``dpx.serve``): single solvated subunits, docked assemblies and
  very large helical assemblies, with fitting-style repeats that change only
  the placements of an earlier request.
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


def euler_from_matrix(R: np.ndarray):
    """Tait-Bryan X1Y2Z3 angles (radians) of R = Rx(a) Ry(b) Rz(c), the
    convention of the reference's EulerD."""
    b = math.asin(max(-1.0, min(1.0, R[0, 2])))
    if abs(R[0, 2]) > 1.0 - 1e-12:  # gimbal lock: only a +- c is defined; take c = 0
        return math.atan2(R[2, 1], R[1, 1]), b, 0.0
    c = math.atan2(-R[0, 1], R[0, 0])
    a = math.atan2(-R[1, 2], R[2, 2])
    return a, b, c


def _axis_rotation(axis, ang):
    x, y, z = np.asarray(axis, dtype=np.float64) / np.linalg.norm(axis)
    c, s, C1 = math.cos(ang), math.sin(ang), 1.0 - math.cos(ang)
    return np.array([[c + x * x * C1, x * y * C1 - z * s, x * z * C1 + y * s],
                     [y * x * C1 + z * s, c + y * y * C1, y * z * C1 - x * s],
                     [z * x * C1 - y * s, z * y * C1 + x * s, c + z * z * C1]])


def icosahedral_rotations() -> list:
    """The 60 rotation matrices of the icosahedral group: closure of a 5-fold
    rotation about a vertex axis (0, 1, phi) and a 3-fold rotation about the
    face axis (1, 1, 1) of the icosahedron with vertices (0, +-1, +-phi) cycled."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    gens = [_axis_rotation((0.0, 1.0, phi), 2 * math.pi / 5), _axis_rotation((1.0, 1.0, 1.0), 2 * math.pi / 3)]
    group = [np.eye(3)]
    frontier = [np.eye(3)]
    while frontier:
        nxt = []
        for g in frontier:
            for h in gens:
                m = h @ g
                if not any(np.allclose(m, x, atol=1e-9) for x in group):
                    group.append(m)
                    nxt.append(m)
        frontier = nxt
    return group


def icosahedral_copies(radius_nm: float = 12.0):
    """(rot [60, 3] rad, tr [60, 3] nm): R_k and R_k (0, 0, radius)."""
    rots, trs = [], []
    for R in icosahedral_rotations():
        rots.append(euler_from_matrix(R))
        trs.append(R @ np.array([0.0, 0.0, radius_nm]))
    return np.array(rots), np.array(trs)


def helix_copies(n: int, radius_nm: float = 12.0, per_turn: int = 13, rise_per_turn_nm: float = 8.0,
                 seed: int = 0, screw: bool = True):
    """(rot [n, 3] rad, tr [n, 3] nm) of n helical copies: copy k at azimuth
    2 pi k / per_turn and height rise_per_turn k / per_turn.
    screw=True: copy k is the seeded subunit orientation R0 turned by its
    azimuth about the helix axis (a screw-symmetric filament: only per_turn
    distinct rotations, each shared by n / per_turn translations);
    screw=False: every copy gets its own seeded rotation (0-360 deg)."""
    rng = np.random.default_rng(seed)
    k = np.arange(n)
    ang = 2 * math.pi * (k % per_turn) / per_turn  # exact repeats of the azimuth
    tr = np.stack([radius_nm * np.cos(ang), radius_nm * np.sin(ang), rise_per_turn_nm * k / per_turn], -1)
    if not screw:
        return rng.uniform(0.0, 2 * math.pi, (n, 3)), tr
    c = rng.uniform(0.0, 2 * math.pi, 3)
    ca, sa, cb, sb, cc, sc = math.cos(c[0]), math.sin(c[0]), math.cos(c[1]), math.sin(c[1]), math.cos(c[2]), \
        math.sin(c[2])
    R0 = np.array([[cb * cc, -cb * sc, sb], [ca * sc + cc * sa * sb, ca * cc - sa * sb * sc, -cb * sa],
                   [sa * sc - ca * cc * sb, cc * sa + ca * sb * sc, ca * cb]])
    per = []
    for m in range(per_turn):
        a = 2 * math.pi * m / per_turn
        Rz = np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
        per.append(euler_from_matrix(Rz @ R0))
    rot = np.array([per[m] for m in (k % per_turn)])
    return rot, tr


@dataclass
class ServeRequest:
    arrival_s: float
    kind: str            # "subunit" | "assembly" | "helix"
    repeat_of: int       # -1, or the index of the request whose grid this one reuses
    leaf: object         # PDBAmplitude
    location: tuple      # leaf placement (x, y, z nm, a, b, c rad)
    copies: object       # None or (rot [K, 3], tr [K, 3])
    grid_size: int
    qmax: float
    Q: np.ndarray

    def models(self):
        return [(0, self.location, self.copies, 1.0)]


def request_stream(n: int, rate_hz: float = 200.0, seed: int = 4004, nq: int = 100, repeat_frac: float = 0.3,
                   helix_copies_n: int = 100_000) -> list:
    """Seeded Poisson stream: 70 % single subunits (20,000 atoms, r = 5 nm,
    dummy-atom solvent, radial step 7.5/200 nm^-1 as the 20k-atom subunit
    workload), 25 % docked assemblies of a 5,000-atom subunit (r = 3 nm, step
    4/150) with 60-5,000 screw-symmetric helical copies (log-uniform; radius
    12 nm, 13 per 8 nm turn), 5 % such helices of ``helix_copies_n`` copies of a
    2,000-atom subunit (r = 2.5 nm, step 5/60);
    qmax uniform in [2, 8] nm^-1; ``repeat_frac`` of the requests repeat an
    earlier request of the same kind with new placements only (a new leaf
    rotation / translation, or a new copy set), reusing its grid."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, n))
    out = []
    for j in range(n):
        u = rng.random()
        kind = "subunit" if u < 0.70 else ("assembly" if u < 0.95 else "helix")
        prev = [i for i, r in enumerate(out) if r.kind == kind and r.repeat_of < 0]
        if prev and rng.random() < repeat_frac:
            base = out[prev[int(rng.integers(len(prev)))]]
            loc = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
            copies = None
            if kind == "subunit":
                loc = tuple(rng.uniform(-1, 1, 3)) + tuple(rng.uniform(0, 2 * math.pi, 3))
            else:
                K = len(base.copies[1])
                copies = helix_copies(K, 12.0 * rng.uniform(0.9, 1.1), 13, 8.0 * rng.uniform(0.9, 1.1),
                                      seed=seed * 7919 + j)
            out.append(ServeRequest(float(t[j]), kind, out.index(base), base.leaf, loc,
                                    copies, base.grid_size, base.qmax, base.Q))
            continue
        qmax = float(rng.uniform(2.0, 8.0))
        if kind == "subunit":
            n_at, radius, step, solvent, copies = 20_000, 5.0, 7.5 / 200, True, None
        elif kind == "assembly":
            n_at, radius, step, solvent = 5_000, 3.0, 4.0 / 150, False
            K = int(round(math.exp(rng.uniform(math.log(60), math.log(5000)))))
            copies = helix_copies(K, 12.0, 13, 8.0, seed=seed * 7919 + j)
        else:
            n_at, radius, step, solvent = 2_000, 2.5, 5.0 / 60, False
            copies = helix_copies(helix_copies_n, 12.0, 13, 8.0, seed=seed * 7919 + j)
        layers = max(8, int(round(qmax / step)))
        sym, xyz = M.make_globule(n_at, radius, seed * 1000 + j)
        leaf = M.PDBAmplitude(sym, xyz, SOLVENT if solvent else VACUUM)
        out.append(ServeRequest(float(t[j]), kind, -1, leaf, (0.0,) * 6, copies, 2 * layers, qmax,
                                np.linspace(0.0, qmax, nq)))
    return out
