"""Serving engine binding (dpx_server): continuous batching of I(q) requests.

A request is a set of PDB leaves and models placed on one grid:
``models = [(leaf_index, location, copies, sym_scale), ...]`` with
``location = (x, y, z [nm], alpha, beta, gamma [rad])`` and ``copies`` either
None or ``(rot [K, 3] rad, tr [K, 3] nm)`` — the same placement vocabulary as
``DomainModel`` (ManualSymmetry rows become copies).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr, lib
from .models import FP32, Context, ManualSymmetry, PDBAmplitude, pdb_descs


class Server:
    def __init__(self, ctx: Context, dirs: np.ndarray, hbm_budget_bytes: int = 0, max_inflight: int = 32,
                 n_streams: int = 8):
        self.ctx = ctx
        d = np.ascontiguousarray(dirs, dtype=np.float64)
        self.n_dirs = len(d)
        h = C.c_void_p()
        check(lib().dpx_server_create(ctx.handle, int(hbm_budget_bytes), int(max_inflight), int(n_streams), dptr(d),
                                      len(d), C.byref(h)))
        self.handle = h
        self._nq = {}

    def submit(self, leaves: Sequence[PDBAmplitude], models, grid_size: int, qmax: float, Q,
               n_samples: int | None = None, eps: float = 0.0, precision: int = FP32,
               leaf_keys: Sequence[int] | None = None) -> int:
        """Queue a request; returns its ticket (inputs are copied)."""
        descs, keep = pdb_descs(leaves)
        nm = len(models)
        model_leaf = np.array([m[0] for m in models], dtype=np.int32)
        loc = np.array([list(m[1]) for m in models], dtype=np.float64).reshape(nm, 6)
        tr = np.ascontiguousarray(loc[:, :3])
        rot = np.ascontiguousarray(loc[:, 3:])
        ncop = np.array([0 if m[2] is None else len(m[2][1]) for m in models], dtype=np.int32)
        crot = [np.asarray(m[2][0], dtype=np.float64).reshape(-1, 3) for m in models if m[2] is not None]
        ctr = [np.asarray(m[2][1], dtype=np.float64).reshape(-1, 3) for m in models if m[2] is not None]
        crot = np.ascontiguousarray(np.concatenate(crot)) if crot else None
        ctr = np.ascontiguousarray(np.concatenate(ctr)) if ctr else None
        ssc = np.array([m[3] for m in models], dtype=np.float64)
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        keys = None if leaf_keys is None else (C.c_uint64 * len(leaves))(*[int(k) for k in leaf_keys])
        r = _lib.Request()
        r.n_leaves, r.leaves, r.leaf_keys = len(leaves), descs, keys
        r.n_models, r.model_leaf, r.rot, r.tr = nm, iptr(model_leaf), dptr(rot), dptr(tr)
        r.n_copies = iptr(ncop) if ncop.any() else None
        r.copy_rot, r.copy_tr, r.sym_scale = dptr(crot), dptr(ctr), dptr(ssc)
        r.grid_size, r.qmax, r.precision = int(grid_size), float(qmax), int(precision)
        r.nq, r.Q = len(Q), dptr(Q)
        r.n_samples = self.n_dirs if n_samples is None else int(n_samples)
        r.eps = float(eps)
        t = C.c_uint64()
        check(lib().dpx_server_submit(self.handle, C.byref(r), C.byref(t)))
        self._nq[t.value] = len(Q)
        return t.value

    def submit_models(self, amps, grid_size: int, qmax: float, Q, **kw) -> int:
        """A request from top-level amplitudes: PDBAmplitude leaves and hybrid
        ManualSymmetry nodes (docked copies of one leaf)."""
        leaves, models = [], []
        for a in amps:
            if isinstance(a, ManualSymmetry):
                leaf = a.child
                copies, ssc = (a.rot, a.trans), a.scale
            else:
                leaf, copies, ssc = a, None, 1.0
            if not any(leaf is x for x in leaves):
                leaves.append(leaf)
            idx = next(i for i, x in enumerate(leaves) if x is leaf)
            models.append((idx, leaf.location, copies, ssc))
        return self.submit(leaves, models, grid_size, qmax, Q, **kw)

    def done(self, ticket: int) -> bool:
        rc = lib().dpx_server_poll(self.handle, int(ticket))
        if rc < 0:
            check(rc)
        return rc == 1

    def wait(self, ticket: int):
        """(I(q), latency in ms from submission to completion)."""
        out = np.zeros(self._nq.pop(ticket))
        lat = C.c_double()
        check(lib().dpx_server_wait(self.handle, int(ticket), dptr(out), C.byref(lat)))
        return out, lat.value

    def stats(self) -> dict:
        st = _lib.ServerStats()
        check(lib().dpx_server_stats_get(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            check(lib().dpx_server_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
