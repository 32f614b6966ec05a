"""The reference-side binding (dplus-dev_gb300/shims/dplus_gpu_shims.cpp)
compiled against the reference's own headers and linked with libdpx: D+'s GPU
entry points with their reference signatures (PDBJacobianGridAmplitudeCalculation,
GPUCalcMCOAJacobSphrDD, GPUCreateCalculatorHybrid's IGPUGridCalculator and the
GPUHybrid_SetPDB / PDBAmplitude hooks), called from a driver that includes the
reference's headers as its call sites do.  Runs where the reference checkout
and its pin library (the reference's Atomic Form Factor.cpp, for
atomicFFCalculator) are built; without a GPU every call must return libdpx's
no-device status through the reference's failure values."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_root():
    from dpx import _build
    return _build.reference_root()


def test_shims_compile_against_the_reference_headers_and_dispatch(tmp_path):
    import oracle as O
    ref = _reference_root()
    if not ref or not O.have_ref():
        pytest.skip("needs the reference checkout and its pin library (build container only)")
    from dpx import _build
    inc = ["-I" + os.path.join(ref, d) for d in ("Common", "Common/ZipLib/Source", "Backend", "Backend/Backend",
                                                  "Backend/GPU")]
    inc += ["-I/usr/local/cuda/include", "-I" + os.path.join(ROOT, "include")]
    exe = str(tmp_path / "shim_driver")
    libdir = os.path.dirname(_build.LIB_PATH)
    refdir = os.path.dirname(O.REF_LIB)
    cmd = ["g++", "-std=c++17", "-O1", "-w", *inc, os.path.join(ROOT, "tests", "shims", "shim_driver.cpp"),
           os.path.join(ROOT, "dplus-dev_gb300", "shims", "dplus_gpu_shims.cpp"), "-o", exe,
           "-L" + libdir, "-l:libdpx.so", "-L" + refdir, "-l:libdplus_ref.so", "-fopenmp",
           "-Wl,-rpath," + libdir + ":" + refdir]
    subprocess.run(cmd, check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lines = dict(ln.split(" ", 1) for ln in out.strip().splitlines())
    import torch
    if torch.cuda.is_available():
        assert lines["fill"].startswith("0") and lines["mcoa"].startswith("0")
        assert lines["hybrid_init"].startswith("1") and lines["hybrid_run"].startswith("1 1")
    else:  # DPX_ERR_NODEVICE (-5) through the reference's -1000 - err / -3000 - err and false
        assert lines["fill"].startswith("-1005") and "no CUDA device" in lines["fill"]
        assert lines["mcoa"].startswith("-3005")
        assert lines["hybrid_init"].startswith("0")
