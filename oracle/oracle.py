"""ctypes binding of the CPU oracle (oracle/build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product (libdpx) never uses it.

``ref()`` additionally exposes oracle/_ref/libdplus_ref.so, the reference's own
Grid.cpp / Atomic Form Factor.cpp built from source where the reference
checkout exists (the build container); it is absent elsewhere.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libdplus_ref.so")

FP64, REFEXACT = 0, 1

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)


class Leaf(C.Structure):
    _fields_ = [("data", _D), ("coeffs", _D), ("rot", C.c_double * 3), ("tr", C.c_double * 3),
                ("n_copies", C.c_int), ("copy_rot", _D), ("copy_tr", _D), ("sym_scale", C.c_double)]


_o = None
_r = None


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_D)


def lib():
    global _o
    if _o is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = C.CDLL(LIB)
        L.orc_grid_cells.restype = C.c_int64
        L.orc_grid_cells.argtypes = [C.c_int]
        L.orc_index_from_indices.restype = C.c_int64
        L.orc_index_from_indices.argtypes = [C.c_int, C.c_int64, C.c_int64]
        L.orc_indices_from_index.argtypes = [C.c_int64, _I, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_aff_table.argtypes = [C.c_int, _D, _I, _D, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                    C.c_double, C.c_int, _D]
        L.orc_grid_fill.argtypes = [C.c_int, C.c_double, C.c_int64, _D, C.c_int, _I, _D, _D, C.c_int, C.c_double,
                                    C.c_double, C.c_double, C.c_int, C.c_int, _D]
        L.orc_grid_fill_shells.argtypes = [C.c_int, C.c_double, C.c_int64, _D, C.c_int, _I, _D, _D, C.c_int,
                                           C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                           _D]
        L.orc_grid_splines.argtypes = [C.c_int, _D, _D, C.c_int, C.c_int]
        L.orc_grid_add_boxes.argtypes = [C.c_int, C.c_double, C.c_int64, _F, C.c_double, C.c_int, C.c_int, _D]
        L.orc_grid_add_boxes_shells.argtypes = [C.c_int, C.c_double, C.c_int64, _F, C.c_double, C.c_int, C.c_int,
                                                C.c_int, C.c_int, _D]
        L.orc_grid_amplitudes_at_points.argtypes = [C.c_int, C.c_double, _D, _D, C.c_int, _D, C.c_double,
                                                    C.c_double, _D]
        L.orc_mc_directions.argtypes = [C.c_uint32, C.c_int64, _D]
        L.orc_layer_seeds.argtypes = [C.c_uint32, C.c_int, C.c_int, C.POINTER(C.c_uint32)]
        L.orc_integrate_layers.restype = C.c_int
        L.orc_integrate_layers.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(Leaf), C.c_int, _D, _D,
                                           C.c_int64, C.c_int64, C.c_double, C.c_int, _D]
        L.orc_q_brackets.argtypes = [C.c_int, C.c_double, C.c_int, _D, _I]
        L.orc_direct_intensity.argtypes = [C.c_int64, _D, C.c_int, _I, _D, _D, C.c_int, C.c_double, C.c_double,
                                           C.c_double, C.c_int64, _F, C.c_int, _D, _D, C.c_int, _D, C.c_int64, _D,
                                           C.c_int, _D]
        L.orc_debye.argtypes = [C.c_int64, _D, C.c_int, _I, _D, _D, C.c_int, C.c_double, C.c_double, _D, _D,
                                C.c_int, _D, C.c_int, C.c_int, _D]
        L.orc_gk_intensity.restype = C.c_double
        L.orc_gk_intensity.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(Leaf), C.c_double, C.c_double,
                                       C.c_int64]
        _o = L
    return _o


def have_ref() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    global _r
    if _r is None:
        L = C.CDLL(REF_LIB)
        L.ref_grid_fill.argtypes = [C.c_int, C.c_double, C.c_int, _F, C.c_int, _I, _F, _F, C.c_int, C.c_float,
                                    C.c_float, C.c_double, _D, _D]
        L.ref_grid_splines.argtypes = [C.c_int, C.c_double, _D, _D]
        L.ref_grid_amplitudes_at_points.argtypes = [C.c_int, C.c_double, _D, _D, C.c_int, _D, C.c_double,
                                                    C.c_double, _D]
        L.ref_grid_sphr.argtypes = [C.c_int, C.c_double, _D, _D, C.c_int, _D, _D]
        L.ref_aff_qmajor.argtypes = [C.c_int, _I, _F, _F, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, _F]
        _r = L
    return _r


# ---- convenience wrappers -------------------------------------------------

class Struct:
    """Oracle-side view of a PDB leaf (atoms sorted by ion)."""

    def __init__(self, xyz, atoms_per_ion, coeffs, ion_rads, flags, sol_ed=0.0, c1=1.0, scale=1.0, boxes=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.api = np.ascontiguousarray(atoms_per_ion, dtype=np.int32)
        self.coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        self.rads = np.ascontiguousarray(ion_rads, dtype=np.float64)
        self.flags, self.sol_ed, self.c1, self.scale = int(flags), float(sol_ed), float(c1), float(scale)
        # voxelized-solvent boxes: [n, 8] float32 {cx, cy, cz, w, Lx, Ly, Lz, 0}
        self.boxes = None if boxes is None or len(boxes) == 0 else \
            np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 8)

    @classmethod
    def from_pdb(cls, amp):
        return cls(amp.xyz, amp.atoms_per_ion, amp.coeffs, amp.ion_rads, amp.flags, amp.solventED, amp.c1,
                   amp.scale, getattr(amp, "solvent_boxes", lambda: None)())


def make_globule(n_atoms, radius_nm, seed):
    """(element codes 0..3 for C, N, O, S, xyz [n, 3] float32 nm) of the seeded
    globule generator, without the library."""
    L = lib()
    L.orc_make_globule.restype = C.c_int
    L.orc_make_globule.argtypes = [C.c_int64, C.c_double, C.c_uint64, _F, _I]
    xyz = np.empty((n_atoms, 3), dtype=np.float32)
    el = np.empty(n_atoms, dtype=np.int32)
    if L.orc_make_globule(n_atoms, radius_nm, seed, xyz.ctypes.data_as(_F), el.ctypes.data_as(_I)) != 0:
        raise ValueError("globule of radius %g nm cannot hold %d atoms" % (radius_nm, n_atoms))
    return el, xyz


def grid_cells(grid_size):
    return lib().orc_grid_cells(grid_size)


def grid_fill(s: Struct, grid_size, qmax, mode=FP64, nthreads=0):
    out = np.zeros(2 * grid_cells(grid_size))
    lib().orc_grid_fill(grid_size, qmax, len(s.xyz), _d(s.xyz), len(s.api), s.api.ctypes.data_as(_I), _d(s.coeffs),
                        _d(s.rads), s.flags, s.sol_ed, s.c1, s.scale, mode, nthreads, out.ctypes.data_as(_D))
    if s.boxes is not None:
        lib().orc_grid_add_boxes(grid_size, qmax, len(s.boxes), s.boxes.ctypes.data_as(_F), s.scale, mode, nthreads,
                                 out.ctypes.data_as(_D))
    return out


def grid_fill_shells(s: Struct, grid_size, qmax, lo, hi, mode=FP64, nthreads=0, out=None):
    if out is None:
        out = np.zeros(2 * grid_cells(grid_size))
    lib().orc_grid_fill_shells(grid_size, qmax, len(s.xyz), _d(s.xyz), len(s.api), s.api.ctypes.data_as(_I),
                               _d(s.coeffs), _d(s.rads), s.flags, s.sol_ed, s.c1, s.scale, mode, nthreads, lo, hi,
                               out.ctypes.data_as(_D))
    if s.boxes is not None:
        lib().orc_grid_add_boxes_shells(grid_size, qmax, len(s.boxes), s.boxes.ctypes.data_as(_F), s.scale, mode,
                                        nthreads, lo, hi, out.ctypes.data_as(_D))
    return out


def grid_splines(grid_size, data, mode=FP64, nthreads=0):
    data = np.ascontiguousarray(data, dtype=np.float64)
    out = np.zeros_like(data)
    lib().orc_grid_splines(grid_size, data.ctypes.data_as(_D), out.ctypes.data_as(_D), mode, nthreads)
    return out


def amplitudes_at_points(grid_size, qmax, data, coeffs, qs, theta, phi):
    qs = np.ascontiguousarray(qs, dtype=np.float64)
    out = np.zeros(2 * len(qs))
    lib().orc_grid_amplitudes_at_points(grid_size, qmax, _d(data), _d(coeffs), len(qs), qs.ctypes.data_as(_D),
                                        theta, phi, out.ctypes.data_as(_D))
    return out[0::2] + 1j * out[1::2]


def aff_table(s: Struct, nq, q0, dq, mode=FP64):
    U = len(s.api)
    out = np.zeros(nq * U)
    lib().orc_aff_table(U, _d(s.coeffs), s.api.ctypes.data_as(_I), _d(s.rads), s.flags, s.sol_ed, s.c1, nq, q0, dq,
                        mode, out.ctypes.data_as(_D))
    return out.reshape(nq, U)


def mc_directions(seed, D):
    out = np.zeros((D, 2))
    lib().orc_mc_directions(seed & 0xFFFFFFFF, D, out.ctypes.data_as(_D))
    return out


def layer_seeds(master, nq, n_layers):
    out = np.zeros(n_layers + 1, dtype=np.uint32)
    lib().orc_layer_seeds(master & 0xFFFFFFFF, nq, n_layers, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def q_brackets(grid_size, qmax, Q):
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    out = np.zeros(len(Q), dtype=np.int32)
    lib().orc_q_brackets(grid_size, qmax, len(Q), Q.ctypes.data_as(_D), out.ctypes.data_as(_I))
    return out


def make_leaf(data, coeffs, rot=(0, 0, 0), tr=(0, 0, 0), copy_rot=None, copy_tr=None, sym_scale=1.0, keep=None):
    """Build an oracle leaf; ``keep`` collects arrays that must outlive the call."""
    keep = keep if keep is not None else []
    data = np.ascontiguousarray(data, dtype=np.float64)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    keep += [data, coeffs]
    lf = Leaf()
    lf.data = data.ctypes.data_as(_D)
    lf.coeffs = coeffs.ctypes.data_as(_D)
    lf.rot[:] = list(rot)
    lf.tr[:] = list(tr)
    if copy_rot is not None:
        cr = np.ascontiguousarray(copy_rot, dtype=np.float64).ravel()
        ct = np.ascontiguousarray(copy_tr, dtype=np.float64).ravel()
        keep += [cr, ct]
        lf.n_copies = len(cr) // 3
        lf.copy_rot = cr.ctypes.data_as(_D)
        lf.copy_tr = ct.ctypes.data_as(_D)
    else:
        lf.n_copies = 0
    lf.sym_scale = sym_scale
    return lf


def integrate_layers(grid_size, qmax, leaves, Q, dirs, dir_layer_stride, max_iter, eps, nthreads=0):
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    dirs = np.ascontiguousarray(dirs, dtype=np.float64)
    arr = (Leaf * len(leaves))(*leaves)
    res = np.zeros(len(Q))
    lib().orc_integrate_layers(grid_size, qmax, len(leaves), arr, len(Q), Q.ctypes.data_as(_D),
                               dirs.ctypes.data_as(_D), dir_layer_stride, max_iter, eps, nthreads,
                               res.ctypes.data_as(_D))
    return res


def integrate_layers_gpu_rule(grid_size, qmax, leaves, Q, dirs, dir_layer_stride, max_iter, eps, samples_per_step,
                              nthreads=0):
    """integrate_layers with the reference GPU averages' convergence test."""
    L = lib()
    L.orc_integrate_layers_gpu_rule.restype = C.c_int
    L.orc_integrate_layers_gpu_rule.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(Leaf), C.c_int, _D, _D,
                                                C.c_int64, C.c_int64, C.c_double, C.c_int64, C.c_int, _D]
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    dirs = np.ascontiguousarray(dirs, dtype=np.float64)
    arr = (Leaf * len(leaves))(*leaves)
    res = np.zeros(len(Q))
    L.orc_integrate_layers_gpu_rule(grid_size, qmax, len(leaves), arr, len(Q), Q.ctypes.data_as(_D),
                                    dirs.ctypes.data_as(_D), dir_layer_stride, max_iter, eps, samples_per_step,
                                    nthreads, res.ctypes.data_as(_D))
    return res


def direct_intensity(s: Struct, Q, dirs, copy_rot=None, copy_tr=None, nthreads=0):
    """FP64 direct sum (no grid) at the given directions, with the leaf's
    solvent boxes and optional docked copies (radians, nm)."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    dirs = np.ascontiguousarray(dirs, dtype=np.float64)
    res = np.zeros(len(Q))
    nc = 0 if copy_rot is None else len(np.ravel(copy_rot)) // 3
    nb = 0 if s.boxes is None else len(s.boxes)
    bx = None if s.boxes is None else s.boxes.ctypes.data_as(_F)
    lib().orc_direct_intensity(len(s.xyz), _d(s.xyz), len(s.api), s.api.ctypes.data_as(_I), _d(s.coeffs),
                               _d(s.rads), s.flags, s.sol_ed, s.c1, s.scale, nb, bx, nc, _d(copy_rot), _d(copy_tr),
                               len(Q),
                               Q.ctypes.data_as(_D), len(dirs), dirs.ctypes.data_as(_D), nthreads,
                               res.ctypes.data_as(_D))
    return res


def debye(s: Struct, Q, bfactor=None, anom=None, mode=FP64, nthreads=0):
    """Debye I(q) of a leaf (DebyeCalTester::Calculate); bfactor [N] and
    anom [N, 2] (f', f'') per atom in the leaf's (ion-sorted) order."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    out = np.zeros(len(Q))
    b = None if bfactor is None else np.ascontiguousarray(bfactor, dtype=np.float64)
    a = None if anom is None else np.ascontiguousarray(anom, dtype=np.float64).reshape(-1)
    lib().orc_debye(len(s.xyz), _d(s.xyz), len(s.api), s.api.ctypes.data_as(_I), _d(s.coeffs), _d(s.rads), s.flags,
                    s.sol_ed, s.c1, _d(b), _d(a), len(Q), _d(Q), mode, nthreads, out.ctypes.data_as(_D))
    return out


def gk_intensity(grid_size, qmax, leaves, q, eps, max_depth):
    arr = (Leaf * len(leaves))(*leaves)
    return lib().orc_gk_intensity(grid_size, qmax, len(leaves), arr, q, eps, max_depth)


def assemble_grid(grid_size, qmax, leaves, lattice=None, scale=1.0, out=None):
    L = lib()
    L.orc_assemble_grid.restype = None
    L.orc_assemble_grid.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(Leaf), _D, C.c_double, C.c_int, _D]
    if out is None:
        out = np.zeros(2 * grid_cells(grid_size))
    arr = (Leaf * len(leaves))(*leaves)
    lat = None if lattice is None else np.ascontiguousarray(lattice, dtype=np.float64)
    L.orc_assemble_grid(grid_size, qmax, len(leaves), arr, _d(lat), scale, 0, out.ctypes.data_as(_D))
    return out


def vegas_intensity(grid_size, qmax, leaves, Q, seed, points_per_iter, max_points, eps):
    L = lib()
    if not getattr(L, "_vegas_typed", False):
        L.orc_vegas_intensity.restype = C.c_int
        L.orc_vegas_intensity.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(Leaf), C.c_int, _D, C.c_uint64,
                                          C.c_int, C.c_int64, C.c_double, _D]
        L.orc_uniform.restype = C.c_double
        L.orc_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L._vegas_typed = True
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    arr = (Leaf * len(leaves))(*leaves)
    res = np.zeros(len(Q))
    rc = L.orc_vegas_intensity(grid_size, qmax, len(leaves), arr, len(Q), Q.ctypes.data_as(_D), seed,
                               points_per_iter, max_points, eps, res.ctypes.data_as(_D))
    if rc != 0:
        raise ValueError("bad VEGAS arguments")
    return res
