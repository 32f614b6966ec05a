"""Shared builders for the parity tests (seeded inputs; the oracle is the checker)."""
import contextlib

import numpy as np

import oracle as O
from dpx import models as M

SOLVENT = [1, 333, 1, 0.05, 0.14, 0.28, 0, 0, 0, 4]
VACUUM = [1, 0, 1, 0.05, 0.14, 0.28, 0, 0, 0, 0]
# dummy-atom solvent plus a 0.3 nm voxelized solvation layer at 400 e/nm^3
LAYER = [1, 333, 1, 0.05, 0.14, 0.3, 400, 0, 0, 4]
# radius-table solvent (type 5): excluded-volume boxes and the layer, cavities filled
BOXES5 = [1, 334, 1, 0.05, 0.14, 0.28, 364, 1, 0, 5]


def globule(n, radius, seed, extra=SOLVENT, centered=False):
    sym, xyz = M.make_globule(n, radius, seed)
    return M.PDBAmplitude(sym, xyz, extra, centered=centered)


def oracle_grid(amp, gs, qmax, mode=O.FP64):
    s = O.Struct.from_pdb(amp)
    data = O.grid_fill(s, gs, qmax, mode)
    return data, O.grid_splines(gs, data, mode)


@contextlib.contextmanager
def fill_method(ctx, method):
    """Run a block with the context's FP32 fill method set (the batched-solve
    and serving engines fill with the direct sum)."""
    before = ctx.fill_method()
    ctx.set_fill_method(method)
    try:
        yield ctx
    finally:
        ctx.set_fill_method(before)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def rel_to_max(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
