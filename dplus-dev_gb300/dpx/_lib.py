"""ctypes binding of libdpx.so (the C-ABI declared in include/dpx.h).

The library is the only compute path: if it is missing, every entry point
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

from ._build import LIB_PATH

_lib = None

DPX_OK = 0
DPX_FP64 = 0
DPX_FP32 = 1
DPX_CALC_ATOMIC_FORMFACTORS = 1
DPX_CALC_DUMMY_SOLVENT = 2
DPX_FILL_DIRECT, DPX_FILL_HARMONIC = 0, 1
DPX_CONV_CPU, DPX_CONV_GPU = 0, 1
DPX_MOMENTS_TCGEN05, DPX_MOMENTS_MMA_SYNC, DPX_MOMENTS_MMA_F16 = 0, 1, 2
DPX_OA_MC, DPX_OA_VEGAS = 0, 1

_STATUS = {-1: "DPX_ERR_ARG", -2: "DPX_ERR_CUDA", -3: "DPX_ERR_OOM", -4: "DPX_ERR_STOPPED",
           -5: "DPX_ERR_NODEVICE"}


class DpxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)
_U32 = C.POINTER(C.c_uint32)


class PdbDesc(C.Structure):
    """dpx_pdb_desc: one leaf of dpx_grid_fill_pdb_batch."""
    _fields_ = [("n_atoms", C.c_int64), ("atoms", _P), ("atoms_on_device", C.c_int), ("n_ions", C.c_int),
                ("atoms_per_ion", _I), ("coeffs", _D), ("ion_rads", _D), ("flags", C.c_int),
                ("solvent_ed", C.c_double), ("c1", C.c_double), ("scale", C.c_double), ("center", _D),
                ("n_boxes", C.c_int64), ("boxes", _F), ("voxel_step", C.c_double), ("aff", _F), ("aff_n", C.c_int)]

class SolveDesc(C.Structure):
    """dpx_solve_desc: one solve of a dpx_batch."""
    _fields_ = [("pdb", PdbDesc), ("grid_size", C.c_int), ("qmax", C.c_double), ("nq", C.c_int), ("Q", _D)]


class Request(C.Structure):
    """dpx_request: one I(q) solve submitted to a dpx_server."""
    _fields_ = [("n_leaves", C.c_int), ("leaves", C.POINTER(PdbDesc)), ("leaf_keys", C.POINTER(C.c_uint64)),
                ("n_models", C.c_int), ("model_leaf", _I), ("rot", _D), ("tr", _D), ("n_copies", _I),
                ("copy_rot", _D), ("copy_tr", _D), ("sym_scale", _D), ("grid_size", C.c_int), ("qmax", C.c_double),
                ("precision", C.c_int), ("nq", C.c_int), ("Q", _D), ("n_samples", C.c_int64), ("eps", C.c_double)]


class ServerStats(C.Structure):
    """dpx_server_stats."""
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "grid_fills", "grid_hits",
                                         "fill_launches", "steps", "evictions", "bytes_in_use", "bytes_peak",
                                         "budget", "cached_grids")]


_SIGS = {
    "dpx_last_error": (C.c_char_p, []),
    "dpx_version": (C.c_int, []),
    "dpx_ctx_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "dpx_ctx_destroy": (C.c_int, [_P]),
    "dpx_ctx_set_stream": (C.c_int, [_P, _P]),
    "dpx_ctx_get_stream": (_P, [_P]),
    "dpx_ctx_synchronize": (C.c_int, [_P]),
    "dpx_ctx_set_fill_shape": (C.c_int, [_P, C.c_int, C.c_int]),
    "dpx_ctx_set_fill_schedule": (C.c_int, [_P, C.c_int]),
    "dpx_set_average_shape": (C.c_int, [C.c_int]),
    "dpx_ctx_set_fill_poly": (C.c_int, [_P, C.c_int]),
    "dpx_ctx_set_fill_method": (C.c_int, [_P, C.c_int]),
    "dpx_set_moments_kernel": (C.c_int, [C.c_int]),
    "dpx_get_moments_kernel": (C.c_int, []),
    "dpx_take_device_faults": (C.c_int, [C.POINTER(C.c_uint)]),
    "dpx_ctx_get_fill_method": (C.c_int, [_P]),
    "dpx_ctx_set_convergence": (C.c_int, [_P, C.c_int, C.c_int64]),
    "dpx_ctx_set_timing": (C.c_int, [_P, C.c_int]),
    "dpx_ctx_stage_times": (C.c_int, [_P, _D]),
    "dpx_ctx_average_kernel_ms": (C.c_int, [_P, _D]),
    "dpx_ctx_get_fill_shape": (C.c_int, [_P, _I]),
    "dpx_fill_shapes": (C.c_int, [_I]),
    "dpx_grid_cells": (C.c_int64, [C.c_int]),
    "dpx_grid_bytes": (C.c_int64, [C.c_int, C.c_int]),
    "dpx_grid_create": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.POINTER(_P)]),
    "dpx_grid_destroy": (C.c_int, [_P]),
    "dpx_grid_device_ptr": (_P, [_P]),
    "dpx_grid_info": (C.c_int, [_P, _I, _D, _I, C.POINTER(C.c_int64)]),
    "dpx_grid_fill_pdb": (C.c_int, [_P, C.c_int64, _P, C.c_int, C.c_int, _I, _D, _D, C.c_int, C.c_double,
                                    C.c_double, C.c_double, _D]),
    "dpx_grid_fill_pdb_batch": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(PdbDesc)]),
    "dpx_autotune_fill": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(PdbDesc), C.c_int, _I, _F]),
    "dpx_leaf_create": (C.c_int, [_P, C.POINTER(PdbDesc), C.POINTER(_P)]),
    "dpx_leaf_fill": (C.c_int, [_P]),
    "dpx_leaf_info": (C.c_int, [_P, _I, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "dpx_leaf_destroy": (C.c_int, [_P]),
    "dpx_grid_compute_splines": (C.c_int, [_P]),
    "dpx_grid_read": (C.c_int, [_P, _D, _D]),
    "dpx_grid_write": (C.c_int, [_P, _D, _D]),
    "dpx_orientation_average": (C.c_int, [_P, C.c_int, C.POINTER(_P), _D, _D, _I, _D, _D, _D, C.c_int, _D, _P,
                                          C.c_int, C.c_int64, C.c_int64, C.c_double, _D]),
    "dpx_vegas_intensity": (C.c_int, [_P, C.c_int, C.POINTER(_P), _D, _D, _I, _D, _D, _D, C.c_int, _D, C.c_uint64,
                                      C.c_int, C.c_int64, C.c_double, _D]),
    "dpx_grid_assemble": (C.c_int, [_P, C.c_int, C.POINTER(_P), _D, _D, _I, _D, _D, _D, _D, C.c_double]),
    "dpx_gk_intensity": (C.c_int, [_P, C.c_int, C.POINTER(_P), _D, _D, _I, _D, _D, _D, C.c_int, _D, C.c_double,
                                   C.c_int64, _D]),
    "dpx_mc_directions": (C.c_int, [C.c_uint32, C.c_int64, _D]),
    "dpx_layer_seeds": (C.c_int, [C.c_uint32, C.c_int, C.c_int, _U32]),
    "dpx_q_brackets": (C.c_int, [C.c_int, C.c_double, C.c_int, _D, _I]),
    "dpx_make_globule": (C.c_int, [C.c_int64, C.c_double, C.c_uint64, _F, _I]),
    "dpx_pdb_jacobian_grid_amplitude": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.c_double, _D, _F, C.c_int64,
                                                  C.c_int, _I, _F, _F, C.c_int, C.c_float, C.c_float, _F, _I,
                                                  C.c_int64, C.c_double, _F, _I, C.c_int64, C.c_double, C.c_double,
                                                  C.c_int, _I]),
    "dpx_pdb_jacobian_grid_amplitude_aff": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.c_double, _D, _F, C.c_int64,
                                                      C.c_int, _I, _F, C.c_int, C.c_int, C.c_float, _F, _I,
                                                      C.c_int64, C.c_double, _F, _I, C.c_int64, C.c_double,
                                                      C.c_double, C.c_int, _I]),
    "dpx_calc_mcoa_jacob_sphr": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_double, _D, _D, _D, _D, C.c_int,
                                           C.c_int64, C.c_double, _D, C.c_int64, C.c_int, _I]),
    "dpx_calc_man_sym_jacob_sphr": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, _D, _D, _D, _D, _D,
                                              _D, _D, _D, _D, C.c_double, C.c_int, _I]),
    "dpx_calc_spc_fill_sym_jacob_sphr": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_double, _D, _D, _D, _D, _D, _D,
                                                   _D, C.c_double, C.c_int, _I]),
    "dpx_sum_grids_jacob_sphr": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_double, C.POINTER(_D), C.POINTER(_D),
                                           _D, _D, C.c_int, _D, C.c_int, _I]),
    "dpx_batch_create": (C.c_int, [_P, C.c_int, C.POINTER(SolveDesc), C.c_int, _D, C.c_int64, C.c_double,
                                   C.c_int64, C.POINTER(_P)]),
    "dpx_batch_launch": (C.c_int, [_P]),
    "dpx_batch_run": (C.c_int, [_P]),
    "dpx_batch_result": (C.c_int, [_P, C.c_int, _D]),
    "dpx_batch_info": (C.c_int, [_P, _I, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "dpx_batch_destroy": (C.c_int, [_P]),
    "dpx_server_create": (C.c_int, [_P, C.c_int64, C.c_int, C.c_int, _D, C.c_int64, C.POINTER(_P)]),
    "dpx_server_submit": (C.c_int, [_P, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "dpx_server_poll": (C.c_int, [_P, C.c_uint64]),
    "dpx_server_wait": (C.c_int, [_P, C.c_uint64, _D, _D]),
    "dpx_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "dpx_server_destroy": (C.c_int, [_P]),
    "dpx_voxel_solvent": (C.c_int, [C.c_int64, _F, _F, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.POINTER(_P)]),
    "dpx_boxes_count": (C.c_int64, [_P, C.c_int]),
    "dpx_boxes_get": (C.c_int, [_P, C.c_int, _F, _I]),
    "dpx_boxes_space": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "dpx_boxes_free": (C.c_int, [_P]),
    "dpx_hybrid_create": (C.c_int, [_P, C.c_int, _F, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_int, C.POINTER(_P)]),
    "dpx_hybrid_set_num_children": (C.c_int, [_P, C.c_int]),
    "dpx_hybrid_child_pdb": (C.c_int, [_P, C.c_int, C.POINTER(PdbDesc)]),
    "dpx_hybrid_child_amp": (C.c_int, [_P, C.c_int, _D]),
    "dpx_hybrid_add_rotations": (C.c_int, [_P, C.c_int, C.c_int, _F]),
    "dpx_hybrid_add_translations": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _F]),
    "dpx_hybrid_compute_intensity": (C.c_int, [_P, C.c_int, _D, C.c_double, C.c_int64, C.c_uint64, _I]),
    "dpx_hybrid_destroy": (C.c_int, [_P]),
    "dpx_measure_sfu_peak": (C.c_int, [_P, _D]),
    "dpx_measure_pipe_peaks": (C.c_int, [_P, _D]),
    "dpx_measure_tcgen05_issue": (C.c_int, [_P, _D]),
    "dpx_debye_intensity": (C.c_int, [_P, C.POINTER(PdbDesc), _F, _F, C.c_int, _D, C.c_int, _D]),
    "dpx_direct_intensity": (C.c_int, [_P, C.POINTER(PdbDesc), C.c_int, _D, _D, C.c_int, _D, C.c_int64, _D, _D]),
    "dpx_calc_debye_v2": (C.c_int, [C.c_int, C.c_float, C.c_float, _D, C.c_int, _I, _F, C.POINTER(C.c_uint8), _F,
                                    C.c_int, _F, _F, C.c_int, C.c_int, C.POINTER(C.c_char), _F, C.c_float, C.c_float,
                                    C.c_int, _I]),
    "dpx_amp_write": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_double, _D]),
    "dpx_amp_read_info": (C.c_int, [C.c_char_p, _I, _D, C.c_char_p, C.c_int64]),
    "dpx_amp_read": (C.c_int, [C.c_char_p, _D]),
    "dpx_mc_average_noalloc": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.c_int, _D, _P, C.c_int64, C.c_double,
                                         _P, _P]),
}

EXPORTED = sorted(_SIGS)


def lib() -> C.CDLL:
    """Load libdpx.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libdpx.so is not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != DPX_OK:
        raise DpxError(rc, lib().dpx_last_error().decode(errors="replace"))


def dptr(a):
    """double* of a contiguous float64 numpy array (or None)."""
    return None if a is None else a.ctypes.data_as(_D)


def fptr(a):
    return None if a is None else a.ctypes.data_as(_F)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_I)
