"""Host-side mirror of D+'s operator interface for the scattering hot path.

The classes keep the reference's names and argument meaning so that a caller
of D+'s backend finds the same operations:

* ``PDBAmplitude``  — PDBAmplitude::PreCalculate / calculateGrid
  (Backend/Backend/PDBAmplitude.cpp:1199-1336, 319-435)
* ``ManualSymmetry`` — explicit docked copies (Backend/DefaultModels/Symmetries.cpp:670-716, 1079-1166)
* ``DomainModel``   — DomainModel::CalculateIntensityVector with the Monte Carlo
  orientation average between layers (Backend/Backend/Amplitude.cpp:701-842, 1168-1247, 2746-2822)

All arithmetic runs in libdpx on the GPU; nothing here computes amplitudes or
intensities.
"""
from __future__ import annotations

import ctypes as C
import os
import hashlib
import math
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr, lib
from .elements import ion

# radius types (Common/Common.h:371-378)
RAD_UNINITIALIZED, RAD_VDW, RAD_EMP, RAD_CALC, RAD_DUMMY_ATOMS_ONLY, RAD_DUMMY_ATOMS_RADII = range(6)

FP64 = _lib.DPX_FP64
FP32 = _lib.DPX_FP32


class Context:
    """One device + one stream + the library's grow-only device scratch."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().dpx_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None) -> None:
        check(lib().dpx_ctx_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def set_fill_schedule(self, persistent: bool) -> None:
        check(lib().dpx_ctx_set_fill_schedule(self.handle, int(bool(persistent))))

    def fill_shape(self):
        """(cells_per_thread, threads, persistent, poly_columns) of the FP32 fill."""
        out = np.zeros(4, dtype=np.int32)
        check(lib().dpx_ctx_get_fill_shape(self.handle, iptr(out)))
        return tuple(int(v) for v in out)

    def set_fill_shape(self, cells_per_thread: int, threads: int, poly_columns: int = 0) -> None:
        check(lib().dpx_ctx_set_fill_shape(self.handle, cells_per_thread, threads))
        check(lib().dpx_ctx_set_fill_poly(self.handle, poly_columns))

    def set_fill_method(self, method: int) -> None:
        """FP32 fill method: _lib.DPX_FILL_DIRECT or _lib.DPX_FILL_HARMONIC."""
        check(lib().dpx_ctx_set_fill_method(self.handle, int(method)))

    def fill_method(self) -> int:
        return int(lib().dpx_ctx_get_fill_method(self.handle))

    def set_convergence(self, rule: int, samples_per_step: int = 8192) -> None:
        """Monte Carlo convergence test: _lib.DPX_CONV_CPU (the reference's CPU
        rule) or _lib.DPX_CONV_GPU (its GPU averages' rule, samples_per_step
        samples a step: 8192 on the grid path, 4096 on the hybrid path)."""
        check(lib().dpx_ctx_set_convergence(self.handle, rule, samples_per_step))

    def synchronize(self) -> None:
        check(lib().dpx_ctx_synchronize(self.handle))

    def close(self) -> None:
        if self.handle:
            lib().dpx_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Grid:
    """Device-resident JacobianSphereGrid (values + phi-spline derivatives)."""

    def __init__(self, ctx: Context, grid_size: int, qmax: float, precision: int = FP32):
        h = C.c_void_p()
        check(lib().dpx_grid_create(ctx.handle, grid_size, float(qmax), precision, C.byref(h)))
        self.handle = h
        self.ctx = ctx
        self.grid_size = grid_size
        self.qmax = float(qmax)
        self.precision = precision
        self.cells = lib().dpx_grid_cells(grid_size)

    @property
    def device_ptr(self) -> int:
        return lib().dpx_grid_device_ptr(self.handle)

    def compute_splines(self) -> None:
        check(lib().dpx_grid_compute_splines(self.handle))

    def read(self, values: bool = True, coeffs: bool = True):
        v = np.empty(2 * self.cells) if values else None
        d = np.empty(2 * self.cells) if coeffs else None
        check(lib().dpx_grid_read(self.handle, dptr(v), dptr(d)))
        return v, d

    def write(self, values: np.ndarray, coeffs: np.ndarray | None = None) -> None:
        values = np.ascontiguousarray(values, dtype=np.float64)
        coeffs = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.float64)
        check(lib().dpx_grid_write(self.handle, dptr(values), dptr(coeffs)))

    def save_amp(self, path: str, header: str = "") -> None:
        """D+'s binary .amp (version 13, Grid.cpp:847-891): the amplitudes only."""
        v, _ = self.read(True, False)
        check(lib().dpx_amp_write(os.fsencode(path), header.encode(), self.grid_size,
                                  self.qmax / (self.grid_size // 2), dptr(v)))

    def save_ampj(self, path: str, params: Sequence[float] = (), header: str = "") -> None:
        """D+'s zipped grid (Amplitude::WriteAmplitudeToFile, Amplitude.cpp:3120-3212):
        grid.dat (the raw amplitudes), criticalinfo.json and header.json, stored."""
        import json
        import zipfile
        v, _ = self.read(True, False)
        info = {"qmax": self.qmax, "qmin": 0, "gridSize": self.grid_size,
                "stepSize": self.qmax / (self.grid_size // 2), "Params": [float(x) for x in params]}
        with zipfile.ZipFile(path, "w", zipfile.ZIP_STORED) as z:
            z.writestr("grid.dat", np.ascontiguousarray(v, dtype="<f8").tobytes())
            z.writestr("criticalinfo.json", json.dumps(info))
            z.writestr("header.json", json.dumps({"Old Header:": header, "Header": {}}))

    def close(self) -> None:
        if self.handle:
            lib().dpx_grid_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_amp(path: str):
    """(grid_size, qmax, header, values) of a .amp (binary v13) or .ampj (zip) file."""
    if zipfile_like(path):
        import json
        import zipfile
        with zipfile.ZipFile(path) as z:
            info = json.loads(z.read("criticalinfo.json"))
            values = np.frombuffer(z.read("grid.dat"), dtype="<f8").astype(np.float64)
            header = ""
            if "header.json" in z.namelist():
                header = json.loads(z.read("header.json")).get("Old Header:", "")
        gs, qmax = int(info["gridSize"]), float(info["qmax"])
        if len(values) != 2 * lib().dpx_grid_cells(gs):
            raise ValueError(f"{path}: grid.dat holds {len(values)} doubles, not 2 x {lib().dpx_grid_cells(gs)}")
        return gs, qmax, header, values
    gs, step = C.c_int(), C.c_double()
    head = C.create_string_buffer(1 << 16)
    check(lib().dpx_amp_read_info(os.fsencode(path), C.byref(gs), C.byref(step), head, len(head)))
    values = np.empty(2 * lib().dpx_grid_cells(gs.value))
    check(lib().dpx_amp_read(os.fsencode(path), dptr(values)))
    return gs.value, step.value * (gs.value // 2), head.value.decode(errors="replace"), values


def zipfile_like(path: str) -> bool:
    with open(path, "rb") as f:
        return f.read(4) == b"PK\x03\x04"


class AmpGridAmplitude:
    """A leaf read from a D+ amplitude file (AmpGridAmplitude, Amplitude.cpp:3682-3720,
    3955-3970): the stored amplitudes times ``scale``, splines recomputed on
    the device, placed by ``location`` like any leaf."""

    def __init__(self, path: str, scale: float = 1.0, location: Sequence[float] = (0, 0, 0, 0, 0, 0)):
        self.path = path
        self.grid_size, self.qmax, self.header, self.values = read_amp(path)
        self.scale = float(scale)
        self.location = tuple(float(v) for v in location)
        self._grid = None
        self._grid_key = None

    def calculateGrid(self, ctx: Context, qmax: float, gridSize: int, precision: int = FP32) -> Grid:
        if int(gridSize) != self.grid_size or abs(float(qmax) - self.qmax) > 1e-12 * self.qmax:
            raise ValueError(f"{self.path} holds a grid of size {self.grid_size}, qmax {self.qmax}; "
                             f"the model asks for {gridSize}, {qmax}")
        key = (self.scale, int(precision), ctx.device)
        if self._grid is not None and self._grid_key == key:
            return self._grid
        g = Grid(ctx, self.grid_size, self.qmax, precision)
        g.write(self.values * self.scale)
        g.compute_splines()
        self._grid, self._grid_key = g, key
        return g


def euler_deg_to_rad(a, b, g):
    return (math.radians(a), math.radians(b), math.radians(g))


class PDBAmplitude:
    """A PDB leaf: atoms, form factors and Gaussian dummy-atom solvent.

    ``extra`` follows D+'s 10 PDB ExtraParameters (PDBAmplitude.cpp:1205-1214):
    [scale, solventED, c1, voxelStep, solventRad, solvationThickness,
    outerSolventED, fillHoles, solventOnly, radType].
    """

    def __init__(self, symbols: Sequence[str], xyz_nm: np.ndarray, extra: Sequence[float] | None = None,
                 centered: bool = False, location: Sequence[float] = (0, 0, 0, 0, 0, 0),
                 bfactors: Sequence[float] | None = None):
        xyz = np.asarray(xyz_nm, dtype=np.float64).reshape(-1, 3)
        if len(symbols) != len(xyz):
            raise ValueError("symbols and coordinates differ in length")
        if len(xyz) == 0:
            raise ValueError("a PDB leaf needs at least one atom")
        ions = [ion(s) for s in symbols]
        if centered:  # moveCOMToOrigin (PDBReaderLib.cpp:271-293), on the coordinates as read
            w = np.array([i.weight for i in ions])
            com = (xyz * w[:, None]).sum(0) / w.sum()
            xyz = xyz - com
        # coordinates are stored as float, as the reference does (PDBAmplitude.h:15)
        xyz = xyz.astype(np.float32).astype(np.float64)
        order = sorted(range(len(ions)), key=lambda k: ions[k].ion_key)  # stable, as std::sort by ion index
        self.symbols = [ions[k].symbol for k in order]
        self.xyz = xyz[order]
        # B factors (Debye-Waller, used by the Debye sum), in the sorted order
        self.bfactors = None if bfactors is None else np.asarray(bfactors, dtype=np.float64)[order]
        keys = [ions[k].ion_key for k in order]
        uniq, self.atoms_per_ion = [], []
        for k, s in zip(keys, self.symbols):
            if not uniq or uniq[-1][0] != k:
                uniq.append((k, s))
                self.atoms_per_ion.append(0)
            self.atoms_per_ion[-1] += 1
        self.unique = [ion(s) for _, s in uniq]
        self.atoms_per_ion = np.array(self.atoms_per_ion, dtype=np.int32)
        U = len(self.unique)
        self.coeffs = np.zeros(9 * U)
        for u, io in enumerate(self.unique):
            for k in range(9):
                self.coeffs[u + k * U] = io.coeffs[k]
        self.ion_rads = np.array([io.dummy_radius for io in self.unique])
        self.location = tuple(float(v) for v in location)  # x, y, z (nm), alpha, beta, gamma (radians)
        self.set_extra(extra if extra is not None else [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0])
        self._grid = None
        self._grid_key = None

    def set_extra(self, p: Sequence[float]) -> None:
        """PreCalculate's parameter unpacking and flag logic (PDBAmplitude.cpp:1205-1272)."""
        p = list(p) + [0] * (10 - len(p))
        self.scale, self.solventED, self.c1 = float(p[0]), float(p[1]), float(p[2])
        self.voxelStep, self.solventRad, self.solvationThickness = float(p[3]), float(p[4]), float(p[5])
        self.outerSolventED = float(p[6])
        self.fillHoles = abs(p[7] - 1.0) < 1e-6
        self.solventOnly = abs(p[8] - 1.0) < 1e-6
        self.radType = int(p[9] + 0.1)
        flags = 0
        if not self.solventOnly:
            flags |= _lib.DPX_CALC_ATOMIC_FORMFACTORS
        if self.radType == RAD_DUMMY_ATOMS_ONLY and self.solventED != 0.0:
            flags |= _lib.DPX_CALC_DUMMY_SOLVENT
        # voxelized solvent (PDBAmplitude.cpp:1248-1256): excluded-volume boxes
        # for the radius-table types, solvation-layer boxes when outerSolventED != 0
        self.voxel_excluded = self.solventED != 0.0 and self.radType in (RAD_CALC, RAD_EMP, RAD_DUMMY_ATOMS_RADII,
                                                                          RAD_VDW)
        self.voxel_layer = self.outerSolventED != 0.0 and self.radType in (RAD_CALC, RAD_EMP, RAD_DUMMY_ATOMS_RADII,
                                                                            RAD_VDW, RAD_DUMMY_ATOMS_ONLY)
        if (self.voxel_excluded or self.voxel_layer) and self.radType not in (RAD_DUMMY_ATOMS_ONLY,
                                                                             RAD_DUMMY_ATOMS_RADII):
            raise NotImplementedError("voxelized solvent needs the dummy-atom radius table (radius types 4, 5); "
                                      "the van der Waals / empirical / calculated tables are not carried")
        self.flags = flags
        self._boxes_key = None
        self._boxes = None

    def atom_radii(self) -> np.ndarray:
        """Per-atom radius (nm) of the leaf's radius type (svgRad for types 4, 5)."""
        return np.array([ion(sym).dummy_radius for sym in self.symbols], dtype=np.float32)

    def voxel_boxes(self):
        """dpx_voxel_solvent on the leaf's atoms: (excluded com, excluded dims,
        layer com, layer dims), centres in nm, extents in voxels."""
        xyz = np.ascontiguousarray(self.xyz, dtype=np.float32)
        rad = self.atom_radii()
        h = C.c_void_p()
        check(lib().dpx_voxel_solvent(len(xyz), xyz.ctypes.data_as(C.POINTER(C.c_float)),
                                      rad.ctypes.data_as(C.POINTER(C.c_float)), self.voxelStep, self.solventRad,
                                      self.solvationThickness, int(self.fillHoles), C.byref(h)))
        out = []
        try:
            for which in (0, 1):
                n = lib().dpx_boxes_count(h, which)
                com = np.zeros((n, 3), dtype=np.float32)
                dims = np.zeros((n, 3), dtype=np.int32)
                if n:
                    check(lib().dpx_boxes_get(h, which, com.ctypes.data_as(C.POINTER(C.c_float)), iptr(dims)))
                out += [com, dims]
        finally:
            lib().dpx_boxes_free(h)
        return tuple(out)

    def solvent_boxes(self):
        """[n, 8] float32 {cx, cy, cz, weight, Lx, Ly, Lz, 0} of the voxelized
        solvent (PDBAmplitude.cpp:277-314): excluded volume at -solventED,
        solvation layer at outerSolventED - solventED; None without voxels."""
        if not (self.voxel_excluded or self.voxel_layer):
            return None
        key = (self.voxelStep, self.solventRad, self.solvationThickness, self.fillHoles, self.radType,
               self.solventED, self.outerSolventED, self.voxel_excluded, self.voxel_layer)
        if self._boxes_key != key:
            ec, ed, lc, ld = self.voxel_boxes()
            step = np.float32(self.voxelStep)
            parts = []
            for on, com, dims, w in ((self.voxel_excluded, ec, ed, -self.solventED),
                                     (self.voxel_layer, lc, ld, self.outerSolventED - self.solventED)):
                if on and len(com):
                    b = np.zeros((len(com), 8), dtype=np.float32)
                    b[:, :3] = com
                    b[:, 3] = np.float32(w)
                    b[:, 4:7] = step * dims.astype(np.float32)
                    parts.append(b)
            self._boxes = np.ascontiguousarray(np.concatenate(parts)) if parts else None
            self._boxes_key = key
        return self._boxes

    def atoms_float4(self) -> np.ndarray:
        a = np.zeros((len(self.xyz), 4), dtype=np.float32)
        a[:, :3] = self.xyz
        return a

    def hash(self) -> str:
        h = hashlib.sha1()
        for arr in (self.xyz, self.coeffs, self.ion_rads, self.atoms_per_ion):
            h.update(np.ascontiguousarray(arr).tobytes())
        h.update(repr((self.scale, self.solventED, self.c1, self.flags, self.voxel_excluded, self.voxel_layer,
                       self.voxelStep, self.solventRad, self.solvationThickness, self.outerSolventED,
                       self.fillHoles)).encode())
        return h.hexdigest()

    def _key(self, ctx: Context, qmax: float, gridSize: int, precision: int):
        return (self.hash(), int(gridSize), float(qmax), int(precision), ctx.device)

    def calculateGrid(self, ctx: Context, qmax: float, gridSize: int, precision: int = FP32) -> Grid:
        """Fill (or reuse) the device-resident amplitude grid and its splines."""
        return calculate_grids(ctx, [self], qmax, gridSize, precision)[0]


def pdb_descs(leaves: Sequence[PDBAmplitude]):
    """dpx_pdb_desc array of PDB leaves (host atoms, centroid centring) and the
    numpy arrays it points into, which must outlive the call."""
    keep, descs = [], (_lib.PdbDesc * len(leaves))()
    for d, a in zip(descs, leaves):
        at = a.atoms_float4()
        keep += [at, a.atoms_per_ion, a.coeffs, a.ion_rads]
        d.n_atoms, d.atoms, d.atoms_on_device, d.n_ions = len(at), at.ctypes.data, 0, len(a.unique)
        d.atoms_per_ion, d.coeffs, d.ion_rads = iptr(a.atoms_per_ion), dptr(a.coeffs), dptr(a.ion_rads)
        d.flags, d.solvent_ed, d.c1, d.scale, d.center = a.flags, a.solventED, a.c1, a.scale, None
        boxes = a.solvent_boxes()
        if boxes is not None:
            keep.append(boxes)
            d.n_boxes, d.boxes = len(boxes), boxes.ctypes.data_as(C.POINTER(C.c_float))
            d.voxel_step = a.voxelStep
    return descs, keep


def set_average_shape(directions_per_thread: int) -> None:
    """Directions per thread (1 or 2) of the FP32 average of one undocked leaf
    over a shared direction set, process-wide (dpx_set_average_shape)."""
    check(lib().dpx_set_average_shape(int(directions_per_thread)))


def autotune_fill(ctx: Context, leaves: Sequence[PDBAmplitude], qmax: float, gridSize: int, repeats: int = 2):
    """Project autotuner: time every FP32 fill shape on these leaves and keep
    the fastest in the context.  Returns (best (cpt, threads, persistent,
    poly_columns), {shape: ms})."""
    n_shapes = lib().dpx_fill_shapes(None)
    shapes = np.zeros(4 * n_shapes, dtype=np.int32)
    lib().dpx_fill_shapes(iptr(shapes))
    grids = [Grid(ctx, gridSize, qmax, FP32) for _ in leaves]
    descs, keep = pdb_descs(leaves)
    handles = (C.c_void_p * len(grids))(*[g.handle.value for g in grids])
    best = np.zeros(4, dtype=np.int32)
    times = np.zeros(n_shapes, dtype=np.float32)
    check(lib().dpx_autotune_fill(len(grids), handles, descs, int(repeats), iptr(best),
                                  times.ctypes.data_as(C.POINTER(C.c_float))))
    for g in grids:
        g.close()
    table = {tuple(int(v) for v in shapes[4 * k:4 * k + 4]): float(times[k]) for k in range(n_shapes)}
    return tuple(int(v) for v in best), table


def calculate_grids(ctx: Context, leaves: Sequence[PDBAmplitude], qmax: float, gridSize: int,
                    precision: int = FP32) -> list:
    """Grids of several PDB leaves; the ones not cached are filled by ONE
    dpx_grid_fill_pdb_batch call (a single persistent launch for FP32)."""
    todo, seen = [], set()
    for a in leaves:
        key = a._key(ctx, qmax, gridSize, precision)
        if (a._grid is None or a._grid_key != key) and id(a) not in seen:
            todo.append((a, key))
            seen.add(id(a))
    if todo:
        grids = [Grid(ctx, gridSize, qmax, precision) for _ in todo]
        descs, keep = pdb_descs([a for a, _ in todo])
        handles = (C.c_void_p * len(todo))(*[g.handle.value for g in grids])
        check(lib().dpx_grid_fill_pdb_batch(len(todo), handles, descs))
        for g, (a, key) in zip(grids, todo):
            g.compute_splines()
            a._grid, a._grid_key = g, key
    return [a._grid for a in leaves]


class SolveBatch:
    """Many independent I(q) solves, one PDB leaf each (dpx_batch): every leaf
    on its own grid (gridSize, qMax) with its own q list, Monte Carlo over one
    shared direction set.  Built once (inputs uploaded, CUDA graphs recorded),
    then ``run()`` replays it."""

    def __init__(self, ctx: Context, leaves: Sequence[PDBAmplitude], grid_sizes: Sequence[int],
                 qmaxes: Sequence[float], Qs: Sequence[np.ndarray], dirs: np.ndarray, n_samples: int | None = None,
                 eps: float = 0.0, precision: int = FP32, grid_budget_bytes: int = 0):
        n = len(leaves)
        if not (len(grid_sizes) == len(qmaxes) == len(Qs) == n):
            raise ValueError("leaves, grid_sizes, qmaxes and Qs must have the same length")
        self.ctx = ctx
        self._Qs = [np.ascontiguousarray(q, dtype=np.float64) for q in Qs]
        pdbs, keep = pdb_descs(leaves)
        descs = (_lib.SolveDesc * n)()
        for d, pd, gs, qm, q in zip(descs, pdbs, grid_sizes, qmaxes, self._Qs):
            d.pdb, d.grid_size, d.qmax, d.nq, d.Q = pd, int(gs), float(qm), len(q), dptr(q)
        dirs = np.ascontiguousarray(dirs, dtype=np.float64)
        n_samples = len(dirs) if n_samples is None else int(n_samples)
        h = C.c_void_p()
        check(lib().dpx_batch_create(ctx.handle, n, descs, int(precision), dptr(dirs), n_samples, float(eps),
                                     int(grid_budget_bytes), C.byref(h)))
        self.handle = h

    def run(self) -> None:
        check(lib().dpx_batch_run(self.handle))

    def launch(self) -> None:
        check(lib().dpx_batch_launch(self.handle))

    def result(self, j: int) -> np.ndarray:
        out = np.zeros(len(self._Qs[j]))
        check(lib().dpx_batch_result(self.handle, int(j), dptr(out)))
        return out

    def results(self) -> list:
        return [self.result(j) for j in range(len(self._Qs))]

    def info(self):
        """(waves, kernel launches per run, grid-pool bytes)."""
        w, k, b = C.c_int(), C.c_int64(), C.c_int64()
        check(lib().dpx_batch_info(self.handle, C.byref(w), C.byref(k), C.byref(b)))
        return w.value, k.value, b.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().dpx_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _pdb_leaves(node, out: list) -> list:
    """Every PDBAmplitude under a model tree node."""
    if isinstance(node, PDBAmplitude):
        out.append(node)
    for c in ([node.child] if hasattr(node, "child") else []) + list(getattr(node, "children", [])):
        _pdb_leaves(c, out)
    return out


def _pack_models(placements):
    """C-ABI model arrays from (grid, location[6], copies or None, sym_scale) tuples."""
    n = len(placements)
    rot = np.zeros(3 * n)
    tr = np.zeros(3 * n)
    ncop = np.zeros(n, dtype=np.int32)
    crot, ctr, sscale = [], [], np.ones(n)
    for m, (g, loc, copies, sc) in enumerate(placements):
        tr[3 * m:3 * m + 3] = loc[:3]
        rot[3 * m:3 * m + 3] = loc[3:]
        if copies is not None:
            ncop[m] = len(copies[1])
            crot.append(np.ravel(copies[0]))
            ctr.append(np.ravel(copies[1]))
        sscale[m] = sc
    crot = np.ascontiguousarray(np.concatenate(crot) if crot else np.zeros(3))
    ctr = np.ascontiguousarray(np.concatenate(ctr) if ctr else np.zeros(3))
    gh = (C.c_void_p * n)(*[p[0].handle.value for p in placements])
    return n, gh, rot, tr, ncop, crot, ctr, sscale


class ManualSymmetry:
    """Docked copies of one child: rows (x, y, z [nm], alpha, beta, gamma [degrees]),
    as ManualSymmetry::PreCalculate reads them (Symmetries.cpp:670-695).  The
    child is a PDB leaf or another ManualSymmetry that uses its grid.

    ``use_grid=False`` is the hybrid path: the docked sum is evaluated per
    orientation sample (HybridOA.cu, Symmetries.cpp:1079-1166).  ``use_grid=True``
    builds the assembly grid once (ManualSymmetry::calculateGrid,
    Symmetries.cpp:879-962) and averages it like a leaf."""

    def __init__(self, child, rows: Sequence[Sequence[float]], scale: float = 1.0,
                 use_grid: bool = False, location: Sequence[float] = (0, 0, 0, 0, 0, 0)):
        r = np.asarray(rows, dtype=np.float64).reshape(-1, 6)
        self.child = child
        self.trans = np.ascontiguousarray(r[:, :3])
        self.rot = np.ascontiguousarray(np.radians(r[:, 3:6]))
        self.scale = float(scale)
        self.use_grid = bool(use_grid)
        self.location = tuple(float(v) for v in location)
        self._grid = None
        self._grid_key = None

    def hash(self) -> str:
        """Content key of the assembly: the child's, the rows, scale and placement."""
        h = hashlib.sha1(self.child.hash().encode())
        h.update(np.ascontiguousarray(self.trans).tobytes())
        h.update(np.ascontiguousarray(self.rot).tobytes())
        h.update(repr((self.scale, self.use_grid, self.location, self.child.location)).encode())
        return h.hexdigest()

    def calculateGrid(self, ctx: Context, qmax: float, gridSize: int, precision: int = FP32) -> Grid:
        child = self.child.calculateGrid(ctx, qmax, gridSize, precision)
        key = (self.child.hash(), self.child.location, self.trans.tobytes(), self.rot.tobytes(), self.scale,
               int(gridSize), float(qmax), int(precision))
        if self._grid is not None and self._grid_key == key:
            return self._grid
        g = Grid(ctx, gridSize, qmax, precision)
        n, gh, rot, tr, ncop, crot, ctr, sscale = _pack_models(
            [(child, self.child.location, (self.rot, self.trans), self.scale)])
        check(lib().dpx_grid_assemble(g.handle, n, gh, dptr(rot), dptr(tr), iptr(ncop), dptr(crot), dptr(ctr),
                                      dptr(sscale), None, 1.0))
        g.compute_splines()
        self._grid, self._grid_key = g, key
        return g

    def placement(self, ctx, qmax, gridSize, precision):
        if self.use_grid:
            return (self.calculateGrid(ctx, qmax, gridSize, precision), self.location, None, 1.0)
        return (self.child.calculateGrid(ctx, qmax, gridSize, precision), self.child.location,
                (self.rot, self.trans), self.scale)


class SpaceFillingSymmetry:
    """GridSymmetry (Symmetries.cpp:30-137): children repeated on a lattice of
    Na x Nb x Nc cells with edges da, db, dc (nm) and angles alpha, beta, gamma
    (degrees); evaluated on the grid path."""

    def __init__(self, children: Sequence, da, db, dc, alpha, beta, gamma, Na, Nb, Nc, scale: float = 1.0,
                 location: Sequence[float] = (0, 0, 0, 0, 0, 0)):
        a, b, c = (math.radians(x) for x in (alpha, beta, gamma))
        if (a == 0 or b == 0 or c == 0 or any(abs(abs(x) - math.pi) < 1e-6 for x in (a, b, c))):
            raise ValueError("Angles in a Space-filling Symmetry cannot be zero or 180.")
        if abs(a) + abs(b) <= abs(c) or abs(c) + abs(b) <= abs(a) or abs(a) + abs(c) <= abs(b):
            raise ValueError("In the Space-filling Symmetry, the sum of any two angles must be greater than the third.")
        sa, sb, sc = math.sin(a), math.sin(b), math.sin(c)
        ca, cb, cc = math.cos(a), math.cos(b), math.cos(c)
        cat = (ca - cb * cc) / (sb * sc)
        if abs(cat) > 1.0:
            raise ValueError("In the Space-filling Symmetry, the angles don't form a valid basis.")
        # GridSymmetry::PreCalculate (Symmetries.cpp:89-101)
        self.lattice = np.array([da, 0.0, 0.0, db * cc, db * sc, 0.0, dc * cb, dc * sb * cat,
                                 dc * sb * math.sin(math.acos(cat)), Na, Nb, Nc], dtype=np.float64)
        self.children = list(children)
        self.scale = float(scale)
        self.location = tuple(float(v) for v in location)
        self._grid = None
        self._grid_key = None

    def calculateGrid(self, ctx: Context, qmax: float, gridSize: int, precision: int = FP32) -> Grid:
        placements = [c.placement(ctx, qmax, gridSize, precision) if hasattr(c, "placement")
                      else (c.calculateGrid(ctx, qmax, gridSize, precision), c.location, None, 1.0)
                      for c in self.children]
        key = (tuple(id(p[0]) for p in placements), self.lattice.tobytes(), self.scale)
        if self._grid is not None and self._grid_key == key:
            return self._grid
        g = Grid(ctx, gridSize, qmax, precision)
        n, gh, rot, tr, ncop, crot, ctr, sscale = _pack_models(placements)
        check(lib().dpx_grid_assemble(g.handle, n, gh, dptr(rot), dptr(tr), iptr(ncop), dptr(crot), dptr(ctr),
                                      dptr(sscale), dptr(self.lattice), self.scale))
        g.compute_splines()
        self._grid, self._grid_key = g, key
        return g

    def placement(self, ctx, qmax, gridSize, precision):
        return (self.calculateGrid(ctx, qmax, gridSize, precision), self.location, None, 1.0)


class DebyeCalTester:
    """Debye sum of a PDB leaf (DebyeCalTester, PDBAmplitude.cpp:1586-1967; the
    standalone DebyeCalculator, DebyeCalculator/DebyeCalculator.cpp:83-311): the
    exact orientation average, no grid.  ``p`` = [solventED, Debye-Waller
    flag, c1] as the reference's parameter vector (DebyeCalculator.cpp:239-243):
    dummy-atom solvent when solventED != 0 (with the dummy-atom radii, as
    PreCalculate selects RAD_DUMMY_ATOMS_ONLY), the leaf's B factors when the
    flag is above 0.1.  ``anomalous``: [N, 2] (f', f'') per atom in the leaf's
    ion-sorted order, or None (AnomDebyeCalTester)."""

    def __init__(self, leaf: PDBAmplitude, anomalous: np.ndarray | None = None):
        self.leaf = leaf
        self.anomalous = None if anomalous is None else \
            np.ascontiguousarray(anomalous, dtype=np.float32).reshape(len(leaf.xyz), 2)

    def CalculateVector(self, ctx: Context, q, p: Sequence[float] = (0.0, 0.0, 1.0), precision: int = FP32):
        pv = list(p) + [0.0, 0.0, 1.0][len(p):]
        a = self.leaf
        bf = None
        if pv[1] > 0.1:
            if a.bfactors is None:
                raise ValueError("the Debye-Waller flag needs B factors on the leaf")
            bf = np.ascontiguousarray(a.bfactors, dtype=np.float32)
        at = a.atoms_float4()
        d = _lib.PdbDesc()
        d.n_atoms, d.atoms, d.atoms_on_device, d.n_ions = len(at), at.ctypes.data, 0, len(a.unique)
        d.atoms_per_ion, d.coeffs, d.ion_rads = iptr(a.atoms_per_ion), dptr(a.coeffs), dptr(a.ion_rads)
        d.flags = _lib.DPX_CALC_ATOMIC_FORMFACTORS | (_lib.DPX_CALC_DUMMY_SOLVENT if pv[0] != 0.0 else 0)
        d.solvent_ed, d.c1, d.scale, d.center = float(pv[0]), float(pv[2]), 1.0, None
        Q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(len(Q))
        fptr = C.POINTER(C.c_float)
        check(lib().dpx_debye_intensity(ctx.handle, C.byref(d), None if bf is None else bf.ctypes.data_as(fptr),
                                        None if self.anomalous is None else self.anomalous.ctypes.data_as(fptr),
                                        len(Q), dptr(Q), int(precision), dptr(out)))
        return out


class DomainModel:
    """DomainModel::CalculateIntensityVector over its top-level amplitudes."""

    def __init__(self, amps: Sequence, gridSize: int, qMax: float, precision: int = FP32):
        self.amps = list(amps)
        self.gridSize = int(gridSize)
        self.qMax = float(qMax)
        self.precision = precision

    def placements(self, ctx: Context):
        leaves = []
        for a in self.amps:
            _pdb_leaves(a, leaves)
        if leaves:  # fill every missing leaf grid in one batched launch
            calculate_grids(ctx, leaves, self.qMax, self.gridSize, self.precision)
        out = []
        for a in self.amps:
            if hasattr(a, "placement"):
                out.append(a.placement(ctx, self.qMax, self.gridSize, self.precision))
            else:
                out.append((a.calculateGrid(ctx, self.qMax, self.gridSize, self.precision), a.location, None, 1.0))
        return out

    def _model_args(self, ctx: Context):
        placements = self.placements(ctx)
        # the arrays must stay alive for the call: return them together
        return _pack_models(placements), (placements,)

    def CalculateIntensityVector(self, ctx: Context, Q: Sequence[float], epsi: float, iterations: int,
                                 dirs: np.ndarray | None = None, dir_layer_stride: int = 0, method: str = "MC",
                                 seed: int = 0, points_per_iter: int = 4096) -> np.ndarray:
        """I(q) by the orientation method of Amplitude.cpp:736-842: "MC" averages
        over the given directions (``iterations`` per bracket); "VEGAS" iterates
        ``points_per_iter`` points until ``iterations`` points or convergence."""
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        (n, gh, rot, tr, ncop, crot, ctr, sscale), keep = self._model_args(ctx)
        res = np.zeros(len(Q))
        if method == "MC":
            d = np.ascontiguousarray(dirs, dtype=np.float64)
            check(lib().dpx_orientation_average(ctx.handle, n, gh, dptr(rot), dptr(tr), iptr(ncop), dptr(crot),
                                                dptr(ctr), dptr(sscale), len(Q), dptr(Q),
                                                d.ctypes.data_as(C.c_void_p), 0, dir_layer_stride, iterations, epsi,
                                                dptr(res)))
        elif method == "GK":  # iterations is the depth budget, as in the reference
            check(lib().dpx_gk_intensity(ctx.handle, n, gh, dptr(rot), dptr(tr), iptr(ncop), dptr(crot), dptr(ctr),
                                         dptr(sscale), len(Q), dptr(Q), epsi, iterations, dptr(res)))
        elif method == "VEGAS":
            check(lib().dpx_vegas_intensity(ctx.handle, n, gh, dptr(rot), dptr(tr), iptr(ncop), dptr(crot), dptr(ctr),
                                            dptr(sscale), len(Q), dptr(Q), seed, points_per_iter, iterations, epsi,
                                            dptr(res)))
        else:
            raise ValueError(f"unknown orientation method {method!r}")
        del keep
        return res


# ---- seeded inputs -------------------------------------------------------

def mc_directions(seed: int, D: int) -> np.ndarray:
    """(theta, phi) pairs of the reference's mt19937 draw order."""
    out = np.empty((D, 2))
    check(lib().dpx_mc_directions(seed & 0xFFFFFFFF, D, dptr(out)))
    return out


def layer_seeds(master: int, nq: int, n_layers: int) -> np.ndarray:
    out = np.empty(n_layers + 1, dtype=np.uint32)
    check(lib().dpx_layer_seeds(master & 0xFFFFFFFF, nq, n_layers, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out


def layer_directions(master: int, nq: int, n_layers: int, D: int) -> np.ndarray:
    """Per-layer direction streams [n_layers, D, 2] as IntegrateLayersTogether draws them."""
    seeds = layer_seeds(master, nq, n_layers)
    return np.stack([mc_directions(int(seeds[l]), D) for l in range(n_layers)])


def make_globule(n_atoms: int, radius_nm: float, seed: int):
    xyz = np.empty((n_atoms, 3), dtype=np.float32)
    el = np.empty(n_atoms, dtype=np.int32)
    check(lib().dpx_make_globule(n_atoms, radius_nm, seed, xyz.ctypes.data_as(C.POINTER(C.c_float)), iptr(el)))
    from .elements import GLOBULE_CODES
    return [GLOBULE_CODES[e] for e in el], xyz.astype(np.float64)
