"""I(q) solves/s of the D+ scattering hot path on GB300.

Workload (one "step" = one I(q) solve): a 20,000-atom synthetic globule
(radius 5 nm, seeded C/N/O/S draw, self-avoiding walk), Gaussian dummy-atom
excluded solvent at 333 e/nm^3, JacobianSphereGrid with 200 radial layers and
qmax = 7.5 nm^-1, I(q) at 500 q in [0, 7.5] averaged by Monte Carlo over a fixed
seeded set of directions per layer bracket.  A solve is amplitude-grid fill +
periodic phi splines + orientation average, FP32 bulk with FP64 centring
phases and FP64 reductions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {dpx,reference}]

``--impl reference`` times the reference's CPU algorithm (the oracle's
reference-exact restatement, all host threads) on a bounded sample of the same
workload.  Under torchrun every rank solves its own replica (no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "dplus-dev_gb300"))

N_ATOMS, RADIUS, SEED = 20000, 5.0, 20251
GRID_SIZE, QMAX, NQ = 400, 7.5, 500
N_DIRS, DIR_SEED = 100_000, 1234
# ncu dram__bytes_read+write of fill_f32_kernel on the profile shape (2,000 atoms,
# 120 layers, 11.3 M cells): 335 MB, i.e. 29.6 B per cell; scaled to 50.7 M cells
FILL_TRAFFIC = 29.6 * 50688289
# ncu dram__bytes_read+write of the moments launch (hm_moments_jobs<FP16>, atoms
# and voxels in one launch) at full size: 137.3 MB read + 144.1 MB written for
# 2,006,280 points, i.e. 140.3 B per point (each point read once, the moments of
# every unit written once); scaled to the points of the workload
MOMENTS_BYTES_PER_POINT = 140.3
# scale, solventED, c1, voxelStep, probe radius, solvation thickness, outer (layer) ED, fillHoles,
# solventOnly, radius type 4 (dummy atoms): dummy-atom solvent at 333 e/nm^3 and a 0.3 nm voxelized
# solvation layer at 400 e/nm^3
EXTRA = [1, 333, 1, 0.05, 0.14, 0.3, 400, 0, 0, 4]
CONFIG = {"workload": "single subunit, 20,000-atom globule r=5 nm, dummy-atom solvent 333 e/nm^3, 0.3 nm "
                      "voxelized solvation layer at 400 e/nm^3 (0.05 nm voxels), L=200 (50,688,289 cells), "
                      "qmax 7.5, 500 q, MC 1e5 fixed directions",
          "atoms": N_ATOMS, "grid_layers": GRID_SIZE // 2, "qmax": QMAX, "q_points": NQ, "mc_directions": N_DIRS,
          "precision": "fp32-bulk", "solvation_layer": "0.3 nm at 400 e/nm^3, voxel 0.05 nm",
          "l2": "grid 811 MB written and read per step (> 129 MB L2)"}


def rank_info():
    r = int(os.environ.get("RANK", 0))
    w = int(os.environ.get("WORLD_SIZE", 1))
    lr = int(os.environ.get("LOCAL_RANK", 0))
    return r, w, lr


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def apply_profile_shape(spec: str) -> None:
    """--profile-shape atoms,layers,dirs,nq: a reduced case for ncu captures
    (never a bench line: the JSON says so)."""
    global N_ATOMS, RADIUS, GRID_SIZE, N_DIRS, NQ, CONFIG
    a, l, d, q = (int(x) for x in spec.split(","))
    N_ATOMS, GRID_SIZE, N_DIRS, NQ = a, 2 * l, d, q
    RADIUS = 5.0 * (a / 20000.0) ** (1.0 / 3.0)
    CONFIG = dict(CONFIG, workload=f"profile shape: {a} atoms, {l} layers, {d} directions, {q} q",
                  atoms=a, grid_layers=l, mc_directions=d, q_points=q)


def build_inputs():
    from dpx import models as M
    sym, xyz = M.make_globule(N_ATOMS, RADIUS, SEED)
    amp = M.PDBAmplitude(sym, xyz, EXTRA)
    Q = np.linspace(0.0, QMAX, NQ)
    dirs = M.mc_directions(DIR_SEED, N_DIRS)
    return amp, Q, dirs


def fill_launches(ctx, n_boxes):
    """Kernel launches of one leaf's fill with its spline derivatives, planned
    and launched in one call.  Harmonic fill: the plan's radial tables (2) and,
    with solvent voxels, their preparation, expansion and binning (7); the
    launch: moments, group sums, contraction, synthesis (4, the synthesis also
    writes the spline derivatives); direct fill: one launch (the boxes are
    sorted on the host), then the spline pass (1)."""
    from dpx import _lib
    if ctx.fill_method() == _lib.DPX_FILL_HARMONIC:
        return 2 + 4 + (7 if n_boxes else 0)
    return 1 + 1


# one average: the angular order of the directions (keys, totals, offsets,
# scatter: eps = 0 and one direction set), bracket tables, average, finalize
AVERAGE_LAUNCHES = 4 + 3


def launches_per_solve(ctx, n_boxes):
    """One solve: the fill and the average."""
    return fill_launches(ctx, n_boxes) + AVERAGE_LAUNCHES


def shape_label(shape) -> str:
    """'CxT' + 'kN' (N phi columns on the FMA pipe) + 'p' (persistent);
    (0, 0, 0, 0) is the harmonic method."""
    c, t, persistent = shape[0], shape[1], shape[2]
    if c == 0:
        return "harmonic"
    poly = shape[3] if len(shape) > 3 else 0
    return "%dx%d%s%s" % (c, t, "k%d" % poly if poly else "", "p" if persistent else "")


def apply_fill_shape(ctx, spec: str) -> None:
    """Set the FP32 fill shape from a shape_label string, e.g. 8x128k2."""
    persistent = spec.endswith("p")
    body = spec.rstrip("p")
    poly = 0
    if "k" in body:
        body, k = body.split("k")
        poly = int(k)
    c, t = (int(x) for x in body.split("x"))
    ctx.set_fill_shape(c, t, poly)
    ctx.set_fill_schedule(persistent)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def run_dpx(args):
    import ctypes as C
    import torch
    import dpx
    from dpx import _lib
    from dpx import models as M

    rank, world, lrank = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(lrank)
    L = dpx.lib()
    ctx = M.Context(lrank)
    stream = torch.cuda.Stream()  # a real stream: CUDA events on it see every libdpx launch
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    if args.fill_shape:
        apply_fill_shape(ctx, args.fill_shape)
    ctx.set_fill_method(_lib.DPX_FILL_HARMONIC if args.fill_method == "harmonic" else _lib.DPX_FILL_DIRECT)
    moments_tc = args.moments == "tcgen05"
    _lib.check(L.dpx_set_moments_kernel({"tcgen05": _lib.DPX_MOMENTS_TCGEN05, "mma": _lib.DPX_MOMENTS_MMA_SYNC,
                                         "mma16": _lib.DPX_MOMENTS_MMA_F16}[args.moments]))

    amp, Q, dirs = build_inputs()
    sfu_c = C.c_double()
    _lib.check(L.dpx_measure_sfu_peak(ctx.handle, C.byref(sfu_c)))
    sfu_measured = sfu_c.value
    pipes = np.zeros(4)  # FP32 FMA scalar, FP32 FMA f32x2, TF32 and FP16 mma.sync: flops/s on this GPU
    _lib.check(L.dpx_measure_pipe_peaks(ctx.handle, _lib.dptr(pipes)))
    tune = None
    if args.autotune:  # sweep every fill shape on this workload's leaf, keep the fastest
        best, table = M.autotune_fill(ctx, [amp], QMAX, GRID_SIZE, repeats=1)
        tune = {"best": shape_label(best), "fill_ms": {shape_label(k): round(v, 3) for k, v in table.items()}}
    t_vox = time.perf_counter()
    boxes = amp.solvent_boxes()  # voxelization: host, once per structure (PreCalculate)
    voxelize_s = time.perf_counter() - t_vox
    n_boxes = 0 if boxes is None else len(boxes)
    atoms_h = amp.atoms_float4()
    # device-resident inputs for the kernel-level number (centred on the host once)
    cen = amp.xyz.mean(0)
    atoms_c = atoms_h.copy()
    atoms_c[:, :3] = (amp.xyz - cen).astype(np.float32)
    d_atoms = torch.from_numpy(atoms_c).cuda()
    d_dirs = torch.from_numpy(np.ascontiguousarray(dirs)).cuda()
    grid = M.Grid(ctx, GRID_SIZE, QMAX, M.FP32)
    gh = (C.c_void_p * 1)(grid.handle.value)
    res = np.zeros(NQ)
    api, co, rads = amp.atoms_per_ion, amp.coeffs, amp.ion_rads
    cen_arr = np.ascontiguousarray(cen)

    ev = {k: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for k in ("fill", "splines", "average")}
    times = {k: [] for k in ev}

    desc_dev, keep_dev = M.pdb_descs([amp])
    desc_dev[0].atoms, desc_dev[0].atoms_on_device = d_atoms.data_ptr(), 1  # centred, resident
    desc_dev[0].center = _lib.dptr(cen_arr)
    # the leaf prepared once, as D+'s PDBAmplitude::PreCalculate (points grouped,
    # solvent voxels binned, tables): outside the timed steps, like the voxelization
    t_prep = time.perf_counter()
    leaf = C.c_void_p()
    _lib.check(L.dpx_leaf_create(grid.handle, desc_dev, C.byref(leaf)))
    prepare_s = time.perf_counter() - t_prep
    leaf_harm, leaf_launches, leaf_bytes = C.c_int(), C.c_int64(), C.c_int64()
    _lib.check(L.dpx_leaf_info(leaf, C.byref(leaf_harm), C.byref(leaf_launches), C.byref(leaf_bytes)))

    def solve(device_inputs: bool, timed_parts: bool = False):
        if timed_parts:
            ev["fill"][0].record(stream)
        if device_inputs:
            # the prepared leaf: queue-only fill (atoms centred and resident; the
            # centring phase is restored per cell)
            _lib.check(L.dpx_leaf_fill(leaf))
        else:
            desc_h, keep_h = M.pdb_descs([amp])  # host atoms and boxes, staged by the call
            _lib.check(L.dpx_grid_fill_pdb_batch(1, gh, desc_h))
        if timed_parts:
            ev["fill"][1].record(stream)
            ev["splines"][0].record(stream)
        _lib.check(L.dpx_grid_compute_splines(grid.handle))
        if timed_parts:
            ev["splines"][1].record(stream)
            ev["average"][0].record(stream)
        if device_inputs:
            _lib.check(L.dpx_orientation_average(ctx.handle, 1, gh, None, None, None, None, None, None, NQ,
                                                 _lib.dptr(Q), C.c_void_p(d_dirs.data_ptr()), 1, 0, N_DIRS, 0.0,
                                                 _lib.dptr(res)))
        else:
            _lib.check(L.dpx_orientation_average(ctx.handle, 1, gh, None, None, None, None, None, None, NQ,
                                                 _lib.dptr(Q), dirs.ctypes.data_as(C.c_void_p), 0, 0, N_DIRS, 0.0,
                                                 _lib.dptr(res)))
        if timed_parts:
            ev["average"][1].record(stream)

    for _ in range(args.warmup):
        solve(True)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    with ClockSampler(lrank) as clk:
        barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            solve(True)
        t1.record(stream)
        barrier()
        dev_ms = t0.elapsed_time(t1)
        # per-kernel split (separate pass so that the timed loop has no extra events);
        # the harmonic fill's own stage events give its moments kernels' time
        _lib.check(L.dpx_ctx_set_timing(ctx.handle, 1))
        stages, avg_kernel = [], []
        for _ in range(max(1, min(3, args.steps))):
            solve(True, timed_parts=True)
            torch.cuda.synchronize()
            for k, (a, b) in ev.items():
                times[k].append(a.elapsed_time(b))
            st5 = np.zeros(5)
            _lib.check(L.dpx_ctx_stage_times(ctx.handle, _lib.dptr(st5)))
            stages.append(st5)
            ak = np.zeros(1)
            _lib.check(L.dpx_ctx_average_kernel_ms(ctx.handle, _lib.dptr(ak)))
            avg_kernel.append(float(ak[0]))
        _lib.check(L.dpx_ctx_set_timing(ctx.handle, 0))
        # end-to-end through the C-ABI with host buffers (atoms in, I(q) out)
        barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            solve(False)
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - w0) * 1e3
        barrier()
    I_fp32 = res.copy()

    dev_ms, e2e_ms = max_over_ranks([dev_ms, e2e_ms], world)

    out = None
    if rank == 0:
        steps_total = args.steps * world
        value = steps_total / (dev_ms / 1e3)
        e2e = steps_total / (e2e_ms / 1e3)
        peaks, peak_kind = measured_peaks()
        clocks = clk.summary()
        fill_ms = float(np.median(times["fill"]))
        avg_ms = float(np.median(times["average"]))
        avg_kernel_ms = float(np.median(avg_kernel))
        spl_ms = float(np.median(times["splines"]))
        P = L.dpx_grid_cells(GRID_SIZE)
        lp = GRID_SIZE // 2 + 3
        cpt, kp = ctx.fill_shape()[0], ctx.fill_shape()[3]
        # row-factored fill: per work item (CPT cells of a theta row, each with its
        # z-mirror) and atom, 1 + CPT sincos = 2 (1 + CPT) sin/cos evaluations
        # (solvent boxes cost the same per work item: their extent factors are cached)
        items = 1 + sum((3 * i // 2 + 1) * ((3 * i + cpt - 1) // cpt) for i in range(1, lp + 1))
        sfu_ops = float(N_ATOMS + n_boxes) * items * 2 * (1 + cpt)
        # SFU roofline: the MUFU throughput this GPU sustains on a calibration
        # kernel of independent sincos chains (measured here, with the clocks above).
        # With kp of the 1 + CPT sincos per item on the FMA pipe, the SFU carries
        # (1 + CPT - kp) of them, so the evaluation rate it allows is
        # peak x (1 + CPT) / (1 + CPT - kp).
        sfu_peak = sfu_measured / 1e12 * (1 + cpt) / (1 + cpt - kp)  # T evaluations/s
        sfu_nominal = 152 * 16 * (peaks.get("sm_max_mhz", 2070.0) * 1e6) / 1e12
        achieved = sfu_ops / (fill_ms / 1e3) / 1e12
        n_brackets = GRID_SIZE // 2
        # the average keeps each direction's radial planes in a sliding window: one
        # new plane (4 rows x 2 nodes x 16 B) per (direction, bracket), read mostly
        # from L2; the grid itself is read from HBM about once
        interp_bytes = float(N_DIRS) * n_brackets * (4 * 2 * 16)
        grid_bytes = float(P) * 16
        if ctx.fill_method() == _lib.DPX_FILL_HARMONIC and stages and stages[-1][2] > 0:
            st5 = np.median(np.array(stages), axis=0)
            mom_ms, syn_ms, harm_ms, n_pts, kk = (float(v) for v in st5)
            # moments: per point and (l, m) six weights times a complex basis value = 24 flops
            flops = n_pts * kk * 24.0
            fp32_peak = float(max(pipes[0], pipes[1])) / 1e12
            # executed on the tensor path, 128 flops per point-(l, m) either way: mma.sync, per
            # 32 points, order l and quartet of 4 m, 8 m16n8k8 TF32 MMAs (hi and remainder of
            # both operands); tcgen05, per 64 points and 128 rows (64 (l, m)), 8 M128 N16 K16
            # FP16 MMAs (hi and remainder of the basis; the weights' halves in N)
            mma_flops = n_pts * kk * 128.0
            tensor_peak = {"tcgen05": peaks["bf16_tflops"] * 1e12, "mma": pipes[2], "mma16": pipes[3]}[args.moments]
            roofline = {"bound": "fp32", "kernel": {"tcgen05": "hm_moments_tc_jobs", "mma": "hm_moments_jobs<TF32>",
                                                   "mma16": "hm_moments_jobs<FP16>"}[args.moments],
                        "method": "harmonic",
                        "achieved": flops / (mom_ms / 1e3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": flops / (mom_ms / 1e3) / 1e12 / fp32_peak,
                        "traffic": MOMENTS_BYTES_PER_POINT * n_pts,
                        "peak_kind": "measured on this GPU (dpx_measure_pipe_peaks: independent FP32 FMA chains, "
                                     "the faster of scalar and packed f32x2)",
                        "pipes_measured_tflops": {"fp32_fma": pipes[0] / 1e12, "fp32_fma_f32x2": pipes[1] / 1e12,
                                                  "tf32_mma_sync": pipes[2] / 1e12,
                                                  "fp16_mma_sync": pipes[3] / 1e12},
                        "tensor_path": {"executed_tflops": mma_flops / (mom_ms / 1e3) / 1e12,
                                        "peak": tensor_peak / 1e12,
                                        "peak_kind": {"tcgen05": "dense bf16/fp16 tcgen05 rate, MEASURED_PEAKS "
                                                                     "bf16_tflops",
                                                      "mma": "TF32 mma.sync m16n8k8, dpx_measure_pipe_peaks",
                                                      "mma16": "FP16 mma.sync m16n8k16, dpx_measure_pipe_peaks"
                                                      }[args.moments],
                                        "frac": mma_flops / (mom_ms / 1e3) / tensor_peak},
                        "note": "flops = points (atoms + solvent voxels) x K x 6 moments x 4 (complex "
                                "multiply-add), K the mean over the points of the (l, m) their radial bins "
                                "carry; time = the hm_moments launches alone (stage events around them); the "
                                "fill also holds the synthesis and the radial tables",
                        "points": n_pts, "K": kk,
                        "stage_ms": {"moments": mom_ms, "synthesis": syn_ms, "harmonic_fill": harm_ms},
                        "equivalent_direct_pairs_per_s": float(N_ATOMS + n_boxes) * P / (fill_ms / 1e3)}
        else:
            roofline = {"bound": "sfu",
                        "kernel": "fill_f32_%s" % ("persistent" if ctx.fill_shape()[2] and not n_boxes else "flat"),
                        "method": "direct", "fill_shape": shape_label(ctx.fill_shape()),
                        "achieved": achieved, "peak": sfu_peak,
                        "unit": "T sin/cos-eval/s", "frac": achieved / sfu_peak, "traffic": FILL_TRAFFIC,
                        "peak_kind": "measured (sincos calibration kernel, dpx_measure_sfu_peak)"
                                     + (", x (1+CPT)/(1+CPT-k): k sincos per item on the FMA pipe" if kp else ""),
                        "sfu_measured": sfu_measured / 1e12,
                        "peak_nominal_16_per_sm_clk": sfu_nominal,
                        "note": "SFU ops = (atoms + solvent boxes) x work items x 2(1+CPT) (row-factored fill); "
                                "traffic = ncu dram bytes of the profile shape scaled by cells",
                        "algorithmic_pairs_per_s": float(N_ATOMS + n_boxes) * P / (fill_ms / 1e3)}
        out = {
            "metric": "I(q) solves/s (FP32-bulk, 20k-atom subunit, L=200, 500 q)",
            "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded globule)", "config": CONFIG,
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(atoms_h.nbytes + Q.nbytes +
                                                                               dirs.nbytes + 32 * n_boxes),
                    "d2h_bytes_per_step": int(res.nbytes),
                    "note": "voxelization (host, once per structure) excluded: voxelize_s"},
            "voxelize_s": voxelize_s, "prepare_s": prepare_s, "solvent_boxes": n_boxes,
            "leaf": {"harmonic": bool(leaf_harm.value), "fill_launches": int(leaf_launches.value),
                     "device_bytes": int(leaf_bytes.value),
                     "note": "prepared once (dpx_leaf_create, the PreCalculate step) outside the timed steps; "
                             "e2e prepares from host arrays in every step"},
            "gpu_launches": args.steps * (int(leaf_launches.value) + AVERAGE_LAUNCHES),
            "roofline": roofline,
            "roofline_average": {"bound": "hbm", "kernel": "average_slide_f32_kernel",
                                 "achieved": grid_bytes / (avg_kernel_ms / 1e3) / 1e9, "peak": peaks["hbm_gbs"],
                                 "unit": "GB/s",
                                 "frac": grid_bytes / (avg_kernel_ms / 1e3) / 1e9 / peaks["hbm_gbs"],
                                 "peak_kind": peak_kind, "kernel_ms": avg_kernel_ms, "call_ms": avg_ms,
                                 "note": "algorithmic bytes = the grid read once (cells x 16 B: the sliding "
                                         "plane window and L2 reuse read each cell from HBM about once); the "
                                         "plane gathers (one plane of 8 cells per direction and bracket) run "
                                         "from L1/L2; kernel_ms = CUDA events around the average kernel alone "
                                         "(dpx_ctx_average_kernel_ms), call_ms = the whole average call",
                                 "gather_gbs": interp_bytes / (avg_kernel_ms / 1e3) / 1e9},
            "split_ms": {"fill": fill_ms, "splines": spl_ms, "average": avg_ms, "average_kernel": avg_kernel_ms},
            "clocks": clocks,
        }
        if tune:
            out["autotune"] = tune
        if not args.no_error:
            out.update(error_report(ctx, stream, amp, Q, dirs, d_dirs, I_fp32, grid, dev_ms / args.steps))
        if not args.no_cpu_baseline and world == 1:
            out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    _lib.check(L.dpx_leaf_destroy(leaf))
    grid.close()
    ctx.close()
    if out is not None and world == 1 and not args.no_extras:
        out.update(headline_extras(args))
    return out


def headline_extras(args):
    """The metric's other two workloads, as keys of the default line: the
    uneven batch of 512 structures (one graph per wave) and the served Poisson
    stream, each FP32-bulk against the plain FP64 GPU path on a seeded
    subsample of the same work (solves/s ratio and max relative I(q) error),
    the stream with its p50 / p99 latency.  Each runs on its own context after
    the subunit's is closed."""
    import argparse as _ap
    import torch
    torch.cuda.synchronize()
    b = run_batch(_ap.Namespace(**dict(vars(args), steps=min(args.steps, 5), warmup=1, fp64_sample=8,
                                       autotune=False, e2e_steps=1, batch_size=512)))
    torch.cuda.synchronize()
    v = run_serve(_ap.Namespace(**dict(vars(args), requests=200, rate=200.0, fp64_sample=8, warmup=3)))
    f64b, f64s = b.get("fp64_plain", {}), v.get("fp64_plain", {})
    return {
        "batch": {"workload": b["config"]["workload"], "value": b["value"], "unit": "solves/s", "steps": b["steps"],
                  "ms_per_step": b["ms_per_step"], "e2e": b["e2e"]["value"], "waves": b["config"]["waves"],
                  "gpu_launches_per_step": b["gpu_launches"] // max(1, b["steps"]),
                  "fp64_plain_solves_per_s_on_sample": f64b.get("fp64_solves_per_s"),
                  "speedup_fp32_vs_fp64_same_sample": f64b.get("speedup_fp32_vs_fp64"),
                  "max_rel_err_vs_fp64": f64b.get("max_rel_err_fp32_vs_fp64"),
                  "fp64_sample": f64b.get("sample"), "clocks": b["clocks"]},
        "serve": {"workload": v["config"]["workload"], "value": v["value"], "unit": "solves/s",
                  "arrival_rate_hz": 200.0, "latency_ms": v["latency_ms"], "server": v["server"],
                  "fp64_plain_solves_per_s_on_sample": f64s.get("fp64_solves_per_s"),
                  "speedup_served_vs_fp64": f64s.get("speedup_served_vs_fp64"),
                  "max_rel_err_vs_fp64": f64s.get("max_rel_err_fp32_vs_fp64"),
                  "fp64_sample": f64s.get("sample"), "clocks": v["clocks"]},
    }


BATCH_NQ, BATCH_DIRS = 200, 100_000


def run_batch(args):
    """Independent solves of uneven size in one batch (dpx_batch: one CUDA graph
    per wave with the harmonic fills planned at creation); FP32-bulk for the whole mix, the
    plain FP64 path on a seeded subsample of it for the speed ratio and the
    error."""
    import torch
    from dpx import models as M
    from dpx import workloads as W

    rank, world, lrank = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(lrank)
    ctx = M.Context(lrank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    mix = W.batch_mix(args.batch_size)
    # every rank solves its own copy of the mix (replicas: no exchange on this path)
    t0 = time.perf_counter()
    leaves = [s.leaf() for s in mix]
    gen_s = time.perf_counter() - t0
    Qs = [np.linspace(0.0, s.qmax, BATCH_NQ) for s in mix]
    dirs = M.mc_directions(DIR_SEED, BATCH_DIRS)
    gss = [s.grid_size for s in mix]
    qms = [s.qmax for s in mix]
    tune = None
    if args.autotune:  # on a seeded sample of four mid-sized structures of the mix
        rng = np.random.default_rng(7)
        mids = sorted(range(len(mix)), key=lambda j: mix[j].pairs())[len(mix) // 4: 3 * len(mix) // 4]
        pick = [mids[k] for k in rng.choice(len(mids), size=min(4, len(mids)), replace=False)]
        # the sample shares one grid: the largest of the four
        j0 = max(pick, key=lambda j: mix[j].layers)
        best, table = M.autotune_fill(ctx, [leaves[j] for j in pick], mix[j0].qmax, mix[j0].grid_size, repeats=1)
        tune = {"best": "%dx%d%s" % (best[0], best[1], "p" if best[2] else ""), "sample": pick,
                "fill_ms": {"%dx%d%s" % (k[0], k[1], "p" if k[2] else ""): round(v, 3) for k, v in table.items()}}

    def build(idx, prec):
        return M.SolveBatch(ctx, [leaves[j] for j in idx], [gss[j] for j in idx], [qms[j] for j in idx],
                            [Qs[j] for j in idx], dirs, precision=prec)

    allidx = list(range(len(mix)))
    b = build(allidx, M.FP32)
    waves, launches, pool = b.info()
    for _ in range(args.warmup):
        b.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(lrank) as clk:
        barrier_sync(world)
        e0.record(stream)
        for _ in range(args.steps):
            b.launch()
        e1.record(stream)
        torch.cuda.synchronize()
        dev_ms = e0.elapsed_time(e1)
    dev_ms = max_over_ranks(dev_ms, world)
    I32 = b.results()
    b.close()
    # end to end: build from host leaves (upload, graph recording), run, read back
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        b = build(allidx, M.FP32)
        b.run()
        _ = b.results()
        b.close()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    n_tot = len(mix) * world
    value = n_tot * args.steps / (dev_ms / 1e3)
    pairs = float(sum(s.pairs() for s in mix))
    out = {
        "metric": "I(q) solves/s (FP32-bulk, uneven batch of independent structures)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded globules)",
        "config": {"workload": "batch of %d independent structures: atoms log-uniform [500, 200000], qmax U[2,10], "
                               "layers U[40,250], half with dummy-atom solvent; %d q in [0, qmax], MC %d shared "
                               "directions" % (len(mix), BATCH_NQ, BATCH_DIRS),
                   "structures": len(mix), "atom_cell_pairs": pairs, "waves": waves, "grid_pool_bytes": pool,
                   "l2": "every grid >= 8 MB and the wave's grids together >> 129 MB L2"},
        "e2e": {"value": n_tot / e2e_s, "unit": "solves/s",
                "h2d_bytes_per_step": int(sum(16 * s.atoms for s in mix) + dirs.nbytes + sum(q.nbytes for q in Qs)
                                          + sum(0 if lf.solvent_boxes() is None else lf.solvent_boxes().nbytes
                                                for lf in leaves)),
                "d2h_bytes_per_step": int(sum(q.nbytes for q in Qs)),
                "note": "per step: the batch created from host leaves (upload, harmonic plans, graph recording), "
                        "run, and its I(q) read back"},
        "gpu_launches": int(launches) * args.steps,
        "fill_method": "harmonic" if ctx.fill_method() == 1 else "direct",
        "roofline": {"note": "whole-batch time (fill + average per structure); per-kernel rooflines in the "
                             "subunit line", "equivalent_direct_pairs_per_s": pairs * args.steps / (dev_ms / 1e3)},
        "generation_s": gen_s,
    }
    if tune:
        out["autotune"] = tune
    out["clocks"] = clk.summary()
    if args.fp64_sample > 0 and rank == 0:
        rng = np.random.default_rng(11)
        sub = sorted(rng.choice(len(mix), size=min(args.fp64_sample, len(mix)), replace=False).tolist())
        b32, b64 = build(sub, M.FP32), build(sub, M.FP64)
        b32.run()
        b64.run()
        torch.cuda.synchronize()
        t = {}
        for name, bb in (("fp32", b32), ("fp64", b64)):
            e0.record(stream)
            bb.launch()
            e1.record(stream)
            torch.cuda.synchronize()
            t[name] = e0.elapsed_time(e1)
        r32, r64 = b32.results(), b64.results()
        err = max(float(np.max(np.abs(x - y) / np.abs(y))) for x, y in zip(r32, r64))
        out["fp64_plain"] = {"sample": sub, "atom_cell_pairs": float(sum(mix[j].pairs() for j in sub)),
                             "fp32_ms": t["fp32"], "fp64_ms": t["fp64"], "speedup_fp32_vs_fp64": t["fp64"] / t["fp32"],
                             "fp64_solves_per_s": len(sub) / (t["fp64"] / 1e3),
                             "max_rel_err_fp32_vs_fp64": err}
        b32.close()
        b64.close()
    ctx.close()
    return out if rank == 0 else None


ASM_NQ, ASM_DIRS, ASM_GRID, ASM_QMAX = 400, 1_000_000, 300, 4.0


def run_assembly(args):
    """Symmetry-docked assemblies of one 5,000-atom subunit (r = 3 nm, vacuum),
    hybrid docked sum per orientation sample: the 60 rotations of the
    icosahedral group with translations R_k (0, 0, 12 nm), and a 1,300-copy
    helix (radius 12 nm, 13 per 8 nm turn, seeded subunit orientation turned
    by each copy's azimuth).  150 layers, qmax 4, 400 q, FP32 bulk.  A step is
    the subunit grid fill plus both MC averages over 1e6 fixed directions (two
    solves); VEGAS (5 x 2e5 points) and Gauss-Kronrod (1e-5) are timed once
    on the icosahedral assembly, and the plain FP64 path on 1e5 directions."""
    import torch
    from dpx import models as M
    from dpx import workloads as W

    rank, world, lrank = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(lrank)
    ctx = M.Context(lrank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    sym, xyz = M.make_globule(5000, 3.0, 2020)
    leaf = M.PDBAmplitude(sym, xyz, W.VACUUM)
    ir, it = W.icosahedral_copies(12.0)
    hr, ht = W.helix_copies(1300, 12.0, 13, 8.0, seed=77)
    rows_ico = np.concatenate([it, np.degrees(ir)], axis=1)
    rows_hel = np.concatenate([ht, np.degrees(hr)], axis=1)
    Q = np.linspace(0.0, ASM_QMAX, ASM_NQ)
    dirs = M.mc_directions(DIR_SEED, ASM_DIRS)
    d_dirs = torch.from_numpy(dirs).cuda()

    def dom(rows, prec=M.FP32):
        return M.DomainModel([M.ManualSymmetry(leaf, rows, use_grid=False)], ASM_GRID, ASM_QMAX, prec)

    import ctypes as C
    from dpx import _lib
    L = M.lib()

    def mc(d, ndirs=ASM_DIRS):
        (n, gh, rot, tr, ncop, crot, ctr, sscale), keep = d._model_args(ctx)
        res = np.zeros(len(Q))
        _lib.check(L.dpx_orientation_average(ctx.handle, n, gh, _lib.dptr(rot), _lib.dptr(tr), _lib.iptr(ncop),
                                             _lib.dptr(crot), _lib.dptr(ctr), _lib.dptr(sscale), len(Q),
                                             _lib.dptr(Q), C.c_void_p(d_dirs.data_ptr()), 1, 0, ndirs, 0.0,
                                             _lib.dptr(res)))
        return res

    d_ico, d_hel = dom(rows_ico), dom(rows_hel)

    def step():
        leaf._grid = None  # the subunit grid is refilled every step
        return mc(d_ico), mc(d_hel)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(lrank) as clk:
        barrier_sync(world)
        e0.record(stream)
        for _ in range(args.steps):
            I_ico, I_hel = step()
        e1.record(stream)
        torch.cuda.synchronize()
        dev_ms = e0.elapsed_time(e1)
    dev_ms = max_over_ranks(dev_ms, world)
    # end to end: host directions in, I(q) out, through DomainModel
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        leaf._grid = None
        d_ico.CalculateIntensityVector(ctx, Q, 0.0, ASM_DIRS, dirs)
        d_hel.CalculateIntensityVector(ctx, Q, 0.0, ASM_DIRS, dirs)
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    solves = 2 * args.steps * world
    value = solves / (dev_ms / 1e3)
    out = {
        "metric": "I(q) solves/s (FP32-bulk, symmetry-docked assemblies, hybrid MC 1e6 directions)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded globule, icosahedral and helical copies)",
        "config": {"workload": "5,000-atom subunit r=3 nm; icosahedral 60 copies at 12 nm; helix 1,300 copies, "
                               "r=12 nm, 13 per 8 nm turn; 150 layers, qmax 4, 400 q, MC 1e6 directions; a step "
                               "= subunit fill + both averages (2 solves)",
                   "copies": [60, 1300], "rotation_groups": [60, 13],
                   "l2": "subunit grid 350 MB (> 129 MB L2) gathered per sample"},
        "e2e": {"value": 2 * world / e2e_s, "unit": "solves/s",
                "h2d_bytes_per_step": int(2 * dirs.nbytes + 16 * len(xyz) + 48 * (60 + 1300)),
                "d2h_bytes_per_step": int(2 * Q.nbytes)},
        # the subunit fill, then two averages
        "gpu_launches": (fill_launches(ctx, 0) + 2 * AVERAGE_LAUNCHES) * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_extras:
        t0 = time.perf_counter()
        d_ico.CalculateIntensityVector(ctx, Q, 0.0, 5 * 200704, method="VEGAS", seed=11, points_per_iter=200704)
        out["vegas_s"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        Qg = np.linspace(0.05, ASM_QMAX, 40)
        d_ico.CalculateIntensityVector(ctx, Qg, 1e-5, 6, method="GK")
        out["gk_s_40q_depth6"] = time.perf_counter() - t0
        errs = []
        for rows, I32 in ((rows_ico, None), (rows_hel, None)):
            leaf._grid = None
            a32 = mc(dom(rows, M.FP32), 100_000)
            leaf._grid = None
            a64 = mc(dom(rows, M.FP64), 100_000)
            errs.append(float(np.max(np.abs(a32 - a64) / np.abs(a64))))
        out["max_rel_err_vs_fp64_1e5_dirs"] = errs
        leaf._grid = None
    ctx.close()
    return out if rank == 0 else None


SERVE_DIRS, SERVE_NQ = 10_000, 100


def run_serve(args):
    """Serving: a seeded Poisson request stream through the serving engine
    (continuous batching, HBM-budget admission, resident grids for repeats).
    value / e2e = completed requests per second of wall clock from the first
    submission to the last completion (host inputs in, I(q) out: the served
    path is end to end by construction); p50 / p99 latency from submission to
    completion.  The plain FP64 path (one request at a time, no grid reuse) is
    timed on the first requests of the stream for the ratio and the error."""
    import threading as th
    import torch
    from dpx import models as M
    from dpx import workloads as W
    from dpx.serve import Server

    rank, world, lrank = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(lrank)
    ctx = M.Context(lrank)
    t0 = time.perf_counter()
    stream = W.request_stream(args.requests, rate_hz=args.rate, nq=SERVE_NQ)
    gen_s = time.perf_counter() - t0
    dirs = M.mc_directions(DIR_SEED, SERVE_DIRS)

    def submit(srv, r, prec=M.FP32):
        return srv.submit([r.leaf], r.models(), r.grid_size, r.qmax, r.Q, precision=prec)

    # warm-up on a separate server (its grid cache does not carry over)
    srv = Server(ctx, dirs, max_inflight=args.inflight, n_streams=8)
    for r in stream[:args.warmup]:
        srv.wait(submit(srv, r))
    srv.close()
    torch.cuda.synchronize()

    srv = Server(ctx, dirs, max_inflight=args.inflight, n_streams=8)
    tickets = [None] * len(stream)
    ready = [th.Event() for _ in stream]

    def feeder():
        base = time.perf_counter()
        for j, r in enumerate(stream):
            dt = base + r.arrival_s - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets[j] = submit(srv, r)
            ready[j].set()

    with ClockSampler(lrank) as clk:
        barrier_sync(world)
        t_start = time.perf_counter()
        f = th.Thread(target=feeder)
        f.start()
        res, lat = [], []
        for j in range(len(stream)):
            ready[j].wait()
            I, ms = srv.wait(tickets[j])
            res.append(I)
            lat.append(ms)
        f.join()
        wall = time.perf_counter() - t_start
    st = srv.stats()
    srv.close()
    wall = max_over_ranks(wall * 1e3, world) / 1e3
    n_tot = len(stream) * world
    value = n_tot / wall
    kinds = {k: sum(r.kind == k for r in stream) for k in ("subunit", "assembly", "helix")}
    out = {
        "metric": "served I(q) solves/s (FP32-bulk), Poisson request stream; p50/p99 latency",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": 1, "warmup": args.warmup,
        "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded globules, helical copies)",
        "config": {"workload": "Poisson stream of %d requests at %.0f req/s: 70%% 20k-atom solvated subunits, 25%% "
                               "5k-atom subunit x 60-5000 helical copies, 5%% 2k-atom subunit x 1e5 helical copies; "
                               "qmax U[2,8]; 30%% placement-only repeats; %d q, MC %d directions"
                               % (len(stream), args.rate, SERVE_NQ, SERVE_DIRS),
                   "requests": len(stream), "kinds": kinds, "repeats": sum(r.repeat_of >= 0 for r in stream),
                   "arrival_window_s": stream[-1].arrival_s, "max_inflight": args.inflight,
                   "l2": "grids of 2.5 MB - 1.2 GB per request, most above the 129 MB L2"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(np.max(lat))},
        "e2e": {"value": value, "unit": "solves/s",
                "h2d_bytes_per_step": int(sum(16 * len(r.leaf.xyz) + (0 if r.copies is None else 48 * len(r.copies[1]))
                                              for r in stream)),
                "d2h_bytes_per_step": int(sum(r.Q.nbytes for r in stream))},
        # the fills' kernels (harmonic: tables, moments, contractions, the synthesis,
        # which writes the spline derivatives); per request: the average and I(0)
        "gpu_launches": int(st["fill_launches"] + (AVERAGE_LAUNCHES + 1) * st["completed"]),
        "server": st, "generation_s": gen_s, "clocks": clk.summary(),
    }
    if args.fp64_sample > 0 and rank == 0:
        sub = list(range(min(args.fp64_sample, len(stream))))
        errs, t64 = [], 0.0
        for j in sub:
            r = stream[j]
            ts = time.perf_counter()
            s64 = Server(ctx, dirs, max_inflight=1, n_streams=1)
            I64, _ = s64.wait(submit(s64, r, M.FP64))
            s64.close()
            t64 += time.perf_counter() - ts
            errs.append(float(np.max(np.abs(res[j] - I64) / np.abs(I64))))
        out["fp64_plain"] = {"sample": sub, "fp64_solves_per_s": len(sub) / t64,
                             "speedup_served_vs_fp64": value / (len(sub) / t64),
                             "max_rel_err_fp32_vs_fp64": max(errs),
                             "note": "one request at a time, fresh grids (no reuse), FP64 fill and average"}
    ctx.close()
    return out if rank == 0 else None


def barrier_sync(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ms, world):
    """Max over the ranks of a time (or a list of times): replicas report the
    slowest rank.  NCCL ranks reduce on their GPU, gloo ranks on the CPU."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    vals = ms if isinstance(ms, (list, tuple)) else [ms]
    t = torch.tensor(list(vals), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out = [float(x) for x in t.tolist()]
    return out if isinstance(ms, (list, tuple)) else out[0]


DIRECT_Q_STRIDE, DIRECT_DIRS = 25, 2000


def error_report(ctx, stream, amp, Q, dirs, d_dirs, I32, grid32, ms32):
    """The error every result reports, and the plain FP64 GPU path beside it.

    (1) The plain FP64 path on the same inputs (FP64 direct-sum fill with the
    solvent boxes, FP64 splines and Monte Carlo average over the same 1e5
    directions), timed as one solve with CUDA events: max relative I(q) error
    of the FP32-bulk result against it, and its solves/s.
    (2) The FP64 direct sum with no grid (dpx_direct_intensity) at every 25th
    q and the first 2,000 directions, against the FP32 grid and the FP64 grid
    averaged over the same sample: the FP32 figure is what the result reports;
    the FP64 grid's shows how much of it is the grid method's own
    (interpolation) error."""
    import ctypes as C
    import torch
    from dpx import _lib
    from dpx import models as M
    L = M.lib()
    rel = lambda a, b: float(np.max(np.abs(a - b) / np.abs(b)))  # noqa: E731
    g64 = M.Grid(ctx, GRID_SIZE, QMAX, M.FP64)
    gh = (C.c_void_p * 1)(g64.handle.value)
    desc, keep = M.pdb_descs([amp])
    I64 = np.zeros(len(Q))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    _lib.check(L.dpx_grid_fill_pdb_batch(1, gh, desc))
    _lib.check(L.dpx_grid_compute_splines(g64.handle))
    _lib.check(L.dpx_orientation_average(ctx.handle, 1, gh, None, None, None, None, None, None, len(Q), _lib.dptr(Q),
                                         C.c_void_p(d_dirs.data_ptr()), 1, 0, len(dirs), 0.0, _lib.dptr(I64)))
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1)
    Qs = np.ascontiguousarray(Q[12::DIRECT_Q_STRIDE])
    ds = np.ascontiguousarray(dirs[:DIRECT_DIRS])

    def sample_average(g):
        r = np.zeros(len(Qs))
        h = (C.c_void_p * 1)(g.handle.value)
        _lib.check(L.dpx_orientation_average(ctx.handle, 1, h, None, None, None, None, None, None, len(Qs),
                                             _lib.dptr(Qs), ds.ctypes.data_as(C.c_void_p), 0, 0, len(ds), 0.0,
                                             _lib.dptr(r)))
        return r

    a32, a64 = sample_average(grid32), sample_average(g64)
    g64.close()
    direct = np.zeros(len(Qs))
    desc[0].center = None  # the frame as given
    t0 = time.perf_counter()
    _lib.check(L.dpx_direct_intensity(ctx.handle, desc, 0, None, None, len(Qs), _lib.dptr(Qs), len(ds),
                                      _lib.dptr(ds), _lib.dptr(direct)))
    t_direct = time.perf_counter() - t0
    del keep
    return {"max_rel_err_vs_fp64": rel(I32, I64),
            "max_rel_err_vs_direct_sum": rel(a32, direct),
            "error": {"vs_fp64": "FP32-bulk I(q) against the plain FP64 GPU path, all %d q, the same %d directions"
                                 % (len(Q), len(dirs)),
                      "vs_direct_sum": "FP64 direct sum (no grid, dpx_direct_intensity) at %d q (every %dth) x the "
                                       "first %d directions, against the grid averaged over the same sample"
                                       % (len(Qs), DIRECT_Q_STRIDE, len(ds)),
                      "fp32_grid_vs_direct_sum": rel(a32, direct), "fp64_grid_vs_direct_sum": rel(a64, direct),
                      "direct_sum_s": t_direct},
            "fp64_plain": {"ms_per_solve": ms64, "solves_per_s": 1e3 / ms64, "speedup_fp32_vs_fp64": ms64 / ms32,
                           "note": "plain FP64 GPU path (FP64 direct-sum fill, splines, MC average), same inputs, "
                                   "one solve timed with CUDA events"}}


def _every(s, k):
    """Every k-th atom of each ion and every k-th solvent box of an oracle struct."""
    import oracle as O
    xyz, api, start = [], [], 0
    for n in s.api:
        part = s.xyz[start:start + n][::k]
        xyz.append(part)
        api.append(len(part))
        start += n
    boxes = None if s.boxes is None else s.boxes[::k]
    return O.Struct(np.concatenate(xyz), api, s.coeffs, s.rads, s.flags, s.sol_ed, s.c1, s.scale, boxes)


_CPU_STRUCT = None


def cpu_struct():
    """The workload's leaf for the CPU baseline, built without libdpx: the
    oracle's globule generator (the library's dpx_make_globule, bit for bit),
    the form-factor tables of dpx.elements (Python data), and the oracle's
    numpy voxelizer for the solvation layer (box for box the library's C++
    voxelizer).  Built once per process (about 20 s of host work, outside
    every timed sample)."""
    global _CPU_STRUCT
    if _CPU_STRUCT is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        import voxel as OV
        from dpx import models as M
        from dpx.elements import GLOBULE_CODES
        el, xyz = O.make_globule(N_ATOMS, RADIUS, SEED)
        amp = M.PDBAmplitude([GLOBULE_CODES[e] for e in el], xyz.astype(np.float64), EXTRA)
        ec, ed, lc, ld, _ = OV.voxel_solvent(amp.xyz, amp.atom_radii(), amp.voxelStep, amp.solventRad,
                                             amp.solvationThickness, amp.fillHoles)
        step = np.float32(amp.voxelStep)
        parts = []
        for on, com, dims, w in ((amp.voxel_excluded, ec, ed, -amp.solventED),
                                 (amp.voxel_layer, lc, ld, amp.outerSolventED - amp.solventED)):
            if on and len(com):
                b = np.zeros((len(com), 8), dtype=np.float32)
                b[:, :3] = com
                b[:, 3] = np.float32(w)
                b[:, 4:7] = step * dims.astype(np.float32)
                parts.append(b)
        boxes = np.concatenate(parts) if parts else None
        _CPU_STRUCT = O.Struct(amp.xyz, amp.atoms_per_ion, amp.coeffs, amp.ion_rads, amp.flags, amp.solventED,
                               amp.c1, amp.scale, boxes)
    return _CPU_STRUCT


def cpu_baseline(seconds: float):
    """The reference's CPU algorithm (oracle, reference-exact precision, all host
    threads) on a bounded sample: the outermost shell of the grid fill for every
    k-th atom of each ion and every k-th solvent box (k chosen by a short probe
    so that the sample takes about `seconds`), scaled to the full grid and all
    points by point-cell pairs; the splines timed in full.  The orientation
    average is < 1 % of a CPU solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    s = cpu_struct()
    Lp = GRID_SIZE // 2 + 3
    cores = os.cpu_count() or 1
    P = O.grid_cells(GRID_SIZE)
    out = np.zeros(2 * P)
    cells = 6 * Lp * (3 * Lp + 1)

    def points(x):
        return len(x.xyz) + (0 if x.boxes is None else len(x.boxes))

    # probe: 1/256 of the points on the outer shell
    probe = _every(s, 256)
    t0 = time.perf_counter()
    O.grid_fill_shells(probe, GRID_SIZE, QMAX, Lp, Lp, O.REFEXACT, cores, out)
    t_probe = max(time.perf_counter() - t0, 1e-4)
    k = max(1, int(np.ceil(256 * t_probe / seconds)))
    sample = _every(s, k)
    out[:] = 0.0
    t0 = time.perf_counter()
    O.grid_fill_shells(sample, GRID_SIZE, QMAX, Lp, Lp, O.REFEXACT, cores, out)
    dt = time.perf_counter() - t0
    t_fill = dt * (P / cells) * (points(s) / points(sample))
    t0 = time.perf_counter()
    O.grid_splines(GRID_SIZE, out, O.REFEXACT, cores)
    t_spl = time.perf_counter() - t0
    solve_s = t_fill + t_spl
    return {"value": 1.0 / solve_s, "unit": "solves/s", "cores": cores, "kind": "port",
            "measured_s": dt + t_spl, "solve_fraction": (dt + t_spl) / solve_s,
            "sample": f"outer shell of the grid fill ({cells} cells) for every {k}-th atom and solvent box "
                      f"({points(sample)} of {points(s)} points, {dt:.1f} s), scaled by point-cell pairs to "
                      f"{P} cells; splines timed in full ({t_spl:.1f} s); orientation average not included "
                      f"(<1%); voxelization (host, once per structure) not included; inputs built without the "
                      f"library (oracle globule generator and numpy voxelizer)"}


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return None
    cpu_struct()  # inputs built once, outside the timed steps
    solves, measured = [], []
    base = None
    for i in range(args.warmup + args.steps):
        base = cpu_baseline(args.cpu_seconds)
        if i >= args.warmup:
            solves.append(1.0 / base["value"])
            measured.append(base["measured_s"])
    v = len(solves) / sum(solves)
    cb = dict(base)
    cb["value"] = v
    # a step is the bounded sample, timed as run: ms_per_step is its measured
    # time; value extrapolates it to whole solves by point-cell pairs
    return {"impl": "reference", "metric": "I(q) solves/s (FP32-bulk, 20k-atom subunit, L=200, 500 q)",
            "value": v, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(measured)),
            "solve_fraction_per_step": float(np.mean(measured)) * v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded globule)", "config": CONFIG, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="dpx", choices=["dpx", "reference"])
    ap.add_argument("--fill-shape", default="", help="CxT[kN][p]: N phi columns on the FMA pipe, p = persistent")
    ap.add_argument("--fill-method", default="harmonic", choices=["direct", "harmonic"],
                    help="FP32 amplitude fill: direct sum, or multipole expansion")
    ap.add_argument("--autotune", action="store_true", help="sweep the fill shapes first and use the fastest")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-error", action="store_true",
                    help="skip the error report (plain FP64 solve and FP64 direct-sum sample)")
    ap.add_argument("--profile-shape", default="", help="atoms,layers,dirs,nq (ncu captures only)")
    ap.add_argument("--moments", default="mma16", choices=["tcgen05", "mma", "mma16"],
                    help="harmonic moments kernel: mma.sync FP16 (default), mma.sync TF32 or tcgen05.mma")
    ap.add_argument("--workload", default="subunit", choices=["subunit", "batch", "serve", "assembly"])
    ap.add_argument("--no-extras", action="store_true",
                    help="subunit: skip the batch and serving keys; assembly: skip the VEGAS / GK / FP64 extras")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--inflight", type=int, default=32)
    ap.add_argument("--batch-size", type=int, default=512)
    ap.add_argument("--fp64-sample", type=int, default=0, help="batch: FP64 comparison on this many structures")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--average-dpt", type=int, default=0,
                    help="directions per thread of the FP32 average (1 or 2; 0: the library default)")
    args = ap.parse_args()
    if args.profile_shape:
        apply_profile_shape(args.profile_shape)
        args.no_cpu_baseline = True
        args.no_error = True
        args.no_extras = True
    if args.impl == "reference":
        out = run_reference(args)
    else:
        from dpx import _build
        _build.build_libdpx()
        from dpx import models as M
        if args.average_dpt:
            M.set_average_shape(args.average_dpt)
        run = {"batch": run_batch, "serve": run_serve, "assembly": run_assembly}.get(args.workload, run_dpx)
        out = run(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
