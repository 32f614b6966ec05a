"""Oracle (test infrastructure only): a numpy / scipy restatement of D+'s
voxelized solvent, used to check the library's C++ voxelizer.

Follows PDBAmplitude::FindPDBRanges (Backend/Backend/PDBAmplitude.cpp:710-749)
and PDBAmplitude::CalculateSolventSpace with its helpers
(Backend/Backend/VoxelizedSolvent.cpp:4-440): the reference's voxel space is
x-major with z padded to a multiple of 16 (SolventSpace::allocate,
Backend/Backend/Amplitude.cpp:4095-4109).  The marking steps are written as
whole-array operations (distance masks, connected components, ball
dilations) instead of the reference's per-voxel loops; the box reduction is
the reference's greedy scan, with faces tested as array slices.

Parity of this restatement is checked against the library; the reference's
own voxelizer needs Eigen / Boost sources that do not build here, so no
reference output pins it.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage

BLUE, GREEN, RED, LIGHT_BLUE, PINK, YELLOW, GREY, MARKER = 0, 1, 2, 3, 4, 5, 6, 8


def _ranges(xyz32, rad32, step, probe, thick):
    dist = max(probe, thick) + 2.0 * step
    lo = (xyz32 - rad32[:, None]).min(axis=0)  # float32 arithmetic, as the reference
    hi = (xyz32 + rad32[:, None]).max(axis=0)
    mins = lo.astype(np.float64) - dist
    maxs = hi.astype(np.float64) + dist
    maxs = np.array([mins[a] + float(int(2.0 + (maxs[a] - mins[a]) / step)) * step for a in range(3)])
    return mins, maxs


def _mark_near_atoms(S, mins, step, xyz32, rad32, r_sol, frm, to):
    dims = S.shape
    for i in range(len(xyz32)):
        p = xyz32[i].astype(np.float64)
        dd = float(rad32[i]) + r_sol
        reach = 2 + int(dd / step)
        c = [int((p[a] - mins[a]) / step) for a in range(3)]
        lo = [max(0, c[a] - reach) for a in range(3)]
        hi = [min(c[a] + reach, dims[a]) for a in range(3)]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        g = [mins[a] + np.arange(lo[a], hi[a], dtype=np.float64) * step - p[a] for a in range(3)]
        d = np.sqrt(g[0][:, None, None] ** 2 + g[1][None, :, None] ** 2 + g[2][None, None, :] ** 2)
        sub = S[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[(sub == frm) & (d <= dd)] = to


def _ball(r):
    a = np.arange(-r, r + 1)
    return np.sqrt(a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2) <= r


def _mark_layer(S, step, radius, typ, neighbor, to_type, from_type):
    disc = int(0.5 + radius / step)
    near = ndimage.binary_dilation(S == neighbor, structure=np.ones((3, 3, 3), bool))
    seeds = np.zeros(S.shape, bool)
    seeds[1:-1, 1:-1, 1:-1] = ((S == typ) & near)[1:-1, 1:-1, 1:-1]
    if disc > 0:
        reach = ndimage.binary_dilation(seeds, structure=_ball(disc))
    else:
        reach = seeds
    S[reach & (S == from_type)] = to_type


def _reduce(S, mins, step, designation, used):
    xs, ys, zs = S.shape
    com, dims = [], []
    cand = np.argwhere(S == designation)  # x, y, z scan order
    for xb, yb, zb in cand:
        if S[xb, yb, zb] != designation:
            continue
        lx = ly = lz = 0
        dx = dy = dz = False
        while not (dx and dy and dz):
            if not dx:
                lx += 1
                ok = xb + lx < xs and bool(np.all(S[xb + lx, yb:yb + ly + 1, zb:zb + lz + 1] == designation))
                if not ok:
                    dx, lx = True, lx - 1
            if not dy:
                ly += 1
                ok = yb + ly < ys and bool(np.all(S[xb:xb + lx + 1, yb + ly, zb:zb + lz + 1] == designation))
                if not ok:
                    dy, ly = True, ly - 1
            if not dz:
                lz += 1
                ok = zb + lz < zs and bool(np.all(S[xb:xb + lx + 1, yb:yb + ly + 1, zb + lz] == designation))
                if not ok:
                    dz, lz = True, lz - 1
        com.append([np.float32(mins[0] + (float(xb) + lx / 2.0) * step),
                    np.float32(mins[1] + (float(yb) + ly / 2.0) * step),
                    np.float32(mins[2] + (float(zb) + lz / 2.0) * step)])
        dims.append([lx + 1, ly + 1, lz + 1])
        S[xb:xb + lx + 1, yb:yb + ly + 1, zb:zb + lz + 1] = used
    return np.array(com, dtype=np.float32).reshape(-1, 3), np.array(dims, dtype=np.int32).reshape(-1, 3)


def voxel_solvent(xyz, radii, step, probe, thick, fill_holes):
    """(excluded com, excluded dims, layer com, layer dims, space dims)."""
    xyz32 = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    rad32 = np.ascontiguousarray(radii, dtype=np.float32)
    mins, maxs = _ranges(xyz32, rad32, step, probe, thick)
    n = [int((maxs[a] - mins[a]) / step) for a in range(3)]
    zs = n[2] + (15 - (n[2] + 15) % 16)
    S = np.zeros((n[0], n[1], zs), dtype=np.int8)
    _mark_near_atoms(S, mins, step, xyz32, rad32, 0.0, BLUE, GREEN)
    if probe > 0:
        _mark_near_atoms(S, mins, step, xyz32, rad32, probe, BLUE, RED)
    if fill_holes:
        lab, _ = ndimage.label(S == BLUE, structure=np.ones((3, 3, 3), bool))
        if S[0, 0, 0] == BLUE:
            S[lab == lab[0, 0, 0]] = LIGHT_BLUE
        S[S == BLUE] = GREEN
    else:
        S[S == BLUE] = LIGHT_BLUE
    if probe > 0:
        _mark_layer(S, step, probe, LIGHT_BLUE, RED, PINK, RED)
        if probe < thick:
            _mark_layer(S, step, abs(thick - probe), PINK, LIGHT_BLUE, PINK, LIGHT_BLUE)
        else:
            _mark_layer(S, step, abs(thick - probe), PINK, LIGHT_BLUE, LIGHT_BLUE, PINK)
        _mark_near_atoms(S, mins, step, xyz32, rad32, 0.0, PINK, -1)
        S[S == RED] = GREEN
        flat = S.reshape(-1)
        per_nm = int(1.0 / step)
        plane = n[1] * zs
        for x in range(n[0]):
            for i in range(per_nm):
                for z in range(1, 5):
                    at = x * plane + (1 + i) * zs + z
                    if at < flat.size:
                        flat[at] = MARKER
    ec, ed = _reduce(S, mins, step, GREEN, YELLOW)
    lc, ld = _reduce(S, mins, step, PINK, GREY)
    return ec, ed, lc, ld, (n[0], n[1], zs)
