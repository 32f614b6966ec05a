"""Element / atomic-group tables used to describe a PDB leaf.

These are data tables that must equal D+'s own to give the same scattering:

* X-ray form-factor coefficients f(s) = sum_{k<4} a_k exp(-b_k s^2) + c, in
  the row order (a1, b1, a2, b2, a3, b3, a4, b4, c).  Atoms use the published
  International Tables for X-ray Crystallography values; the implicit-hydrogen
  groups (CH, CH2, ...) use D+'s fitted "modified form factors"
  (PDBReaderLib/PDBReaderLib.cpp:2270-2480).
* Dummy-atom (excluded-volume) radii in nm, D+'s ``svgRad`` table
  (PDBReaderLib/PDBReaderLib.cpp:204-265).
* Atomic weights used for centring to the centre of mass (moveCOMToOrigin,
  PDBReaderLib.cpp:271-293); a group weighs what its heavy atom weighs there.

``ion_key`` is the row of the ion in D+'s coefficient table; atoms are sorted by
it (PDBReaderLib.cpp:1058) so that ions form contiguous runs.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass(frozen=True)
class Ion:
    symbol: str
    ion_key: int
    coeffs: tuple  # (a1, b1, a2, b2, a3, b3, a4, b4, c)
    dummy_radius: float  # nm
    weight: float


_T = {
    "H": (0, (0.49300, 10.51090, 0.32290, 26.1257, 0.14020, 3.14240, 0.04080, 57.79980, 0.0030), 0.107, 1.008),
    "C": (7, (2.31000, 20.8439, 1.02000, 10.2075, 1.58860, 0.56870, 0.86500, 51.65120, 0.2156), 0.1577, 12.011),
    "N": (8, (12.2126, 0.00570, 3.13220, 9.89330, 2.01250, 28.9975, 1.16630, 0.58260, -11.5290), 0.08414, 14.007),
    "O": (9, (3.04850, 13.2771, 2.28680, 5.70110, 1.54630, 0.32390, 0.86700, 32.90890, 0.2508), 0.130, 15.999),
    "MG": (16, (5.42040, 2.82750, 2.17350, 79.2611, 1.22690, 0.38080, 2.30730, 7.19370, 0.8584), 0.160, 24.3050),
    "P": (22, (6.43450, 1.90670, 4.17910, 27.1570, 1.78000, 0.52600, 1.49080, 68.16450, 1.1149), 0.111, 30.97376),
    "S": (23, (6.90530, 1.46790, 5.20340, 22.2151, 1.43790, 0.25360, 1.58630, 56.1720, 0.86690), 0.168, 32.06),
    "CH": (208, (0.894937, 55.7145, 0.894429, 4.03158, 3.78824, 24.8323, 3.14683e-6, 956.628, 1.42149), 0.173,
           12.011),
    "CH2": (209, (1.61908, 52.1451, 2.27205, 24.6589, 2.1815, 24.6587, 0.0019254, 152.165, 1.92445), 0.185, 12.011),
    "CH3": (210, (12.5735, 38.7341, -0.456658, -6.28167, 5.71547, 54.955, -11.711, 47.898, 2.87762), 0.197, 12.011),
    "NH": (211, (0.00506991, 108.256, 2.03147, 14.6199, 1.82122, 14.628, 2.06506, 35.4102, 2.07168), 0.122, 14.007),
    "NH2": (212, (3.00872, 28.3717, 0.288137, 63.9637, 3.39248, 3.51866, 2.03511, 28.3675, 0.269952), 0.145,
            14.007),
    "NH3": (213, (0.294613, 67.4408, 6.48379, 29.1576, 5.67182, 0.54735, 6.57164, 0.547493, -9.02757), 0.162,
            14.007),
    "OH": (214, (-2.73406, 22.1288, 0.00966263, 94.3428, 6.64439, 13.9044, 2.67949, 32.7607, 2.39981), 0.150,
           15.999),
    "SH": (215, (-127.811, 7.19935, 62.5514, 12.1591, 160.747, 1.88979, 2.34822, 55.952, -80.836), 0.181, 32.06),
}

IONS = {k: Ion(k, *v) for k, v in _T.items()}

# element codes of the synthetic globule generator (dpx_make_globule)
GLOBULE_CODES = ("C", "N", "O", "S")


def ion(symbol: str) -> Ion:
    try:
        return IONS[symbol.upper()]
    except KeyError:
        raise KeyError(f"no form-factor entry for {symbol!r}") from None
