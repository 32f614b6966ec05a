"""Build recipe for libdpx.so (sm_103a) and the test-side oracle.

libdpx is compiled in-tree with nvcc for ``sm_103a`` only; the object files are
built in parallel and linked into ``dpx/libdpx.so`` next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(os.path.dirname(PKG_DIR), "csrc")
REPO_DIR = os.path.dirname(os.path.dirname(PKG_DIR))
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(os.path.dirname(PKG_DIR), "_build")
LIB_PATH = os.path.join(PKG_DIR, "libdpx.so")

SOURCES = ["dpx_fill.cu", "dpx_kernels.cu", "dpx_api.cpp", "dpx_batch.cpp", "dpx_server.cpp", "dpx_stage.cpp",
           "dpx_voxel.cpp", "dpx_amp.cpp", "dpx_noalloc.cu", "dpx_debye.cu", "dpx_debye_host.cpp",
           "dpx_harmonic.cu", "dpx_harmonic_host.cpp", "dpx_direct.cu",
           "dpx_leaf.cpp", "dpx_hybrid.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; libdpx needs the CUDA toolkit to build")
    return cand


def _compile(src: str) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    # host code without floating-point contraction: the same results on x86 and Arm hosts
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE_DIR, "-I", SRC_DIR, "-c", os.path.join(SRC_DIR, src),
           "-o", obj]
    if src.endswith(".cu"):
        cmd[3:3] = ["-Xptxas", "-v"] if os.environ.get("DPX_PTXAS_VERBOSE") else []
    subprocess.run(cmd, check=True)
    return obj


def build_libdpx(force: bool = False) -> str:
    """Compile libdpx.so if any source is newer than the library."""
    srcs = [os.path.join(SRC_DIR, s) for s in SOURCES] + [
        os.path.join(SRC_DIR, "dpx_internal.h"), os.path.join(SRC_DIR, "dpx_host.h"),
        os.path.join(SRC_DIR, "dpx_spline.cuh"), os.path.join(INCLUDE_DIR, "dpx.h")]
    if (not force and os.path.exists(LIB_PATH)
            and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in srcs)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB_PATH + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_root() -> str | None:
    """The reference checkout the oracle's pin library is built from:
    DPX_REF_ROOT, else a checkout named ``reference`` beside this repository;
    None where neither exists (the GPU machine runs without it)."""
    for cand in (os.environ.get("DPX_REF_ROOT"), os.path.join(os.path.dirname(REPO_DIR), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "Backend")):
            return cand
    return None


def build_oracle(with_reference: bool = True) -> None:
    """Compile the CPU oracle (test infrastructure) and, where the reference
    checkout exists, the reference-backed pin library."""
    oracle_dir = os.path.join(REPO_DIR, "oracle")
    subprocess.run(["make", "-s", "-C", oracle_dir], check=True)
    ref_root = reference_root()
    if with_reference and ref_root:
        subprocess.run(["make", "-s", "-C", oracle_dir, "ref", f"REF_ROOT={ref_root}"], check=True)
