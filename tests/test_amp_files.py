"""Amplitude-grid files on the CPU: D+'s binary .amp (version 13) written by
the library and read back, checked field by field with a reader that follows
JacobianSphereGrid::ImportBinaryData (Backend/Backend/Grid.cpp:893-963), and
the zipped .ampj layout of Amplitude::WriteAmplitudeToFile."""
import json
import struct
import zipfile

import numpy as np
import pytest

import dpx
from dpx import _lib
from dpx import models as M


def _values(gs, seed=0):
    P = dpx.lib().dpx_grid_cells(gs)
    return np.random.default_rng(seed).normal(size=2 * P)


def _reference_style_read(path):
    """The reader steps of ImportBinaryData, restated in Python."""
    b = open(path, "rb").read()
    assert b[:2] == b"#@"
    offset = struct.unpack("<I", b[2:6])[0]
    header = b[7:offset - 1].decode()
    rest = b[offset:]
    lines = rest.split(b"\n", 4)
    version, nbytes, dimx, extras = (int(x) for x in lines[:4])
    step = struct.unpack("<d", lines[4][:8])[0]
    data = np.frombuffer(lines[4][8:], dtype="<f8")
    return header, version, nbytes, dimx, extras, step, data


@pytest.mark.parametrize("gs,header", [(20, "made by dpx"), (36, "# two\nlines"), (12, "")])
def test_amp_write_read_round_trip(tmp_path, gs, header):
    v = _values(gs, gs)
    step = 5.0 / (gs // 2)
    p = str(tmp_path / "g.amp")
    _lib.check(dpx.lib().dpx_amp_write(p.encode(), header.encode(), gs, step, _lib.dptr(v)))
    h, version, nbytes, dimx, extras, st, data = _reference_style_read(p)
    assert (h, version, nbytes, dimx, extras, st) == (header, 13, 16, gs // 2 + 3, 3, step)
    assert np.array_equal(data, v)
    g2, qmax, h2, v2 = M.read_amp(p)
    assert (g2, h2) == (gs, header) and abs(qmax - 5.0) < 1e-12 and np.array_equal(v2, v)


def test_amp_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.amp"
    p.write_bytes(b"#@\x10\x00\x00\x00\nhdr\n12\n16\n13\n3\n")
    assert dpx.lib().dpx_amp_read_info(str(p).encode(), _lib.iptr(np.zeros(1, np.int32)),
                                       _lib.dptr(np.zeros(1)), None, 0) == -1
    v = _values(10)
    q = str(tmp_path / "short.amp")
    _lib.check(dpx.lib().dpx_amp_write(q.encode(), b"x", 10, 0.5, _lib.dptr(v)))
    raw = open(q, "rb").read()
    open(q, "wb").write(raw[:-8])  # one double short
    with pytest.raises(_lib.DpxError):
        M.read_amp(q)


def test_ampj_layout_is_read(tmp_path):
    gs, qmax = 16, 3.0
    v = _values(gs, 3)
    p = str(tmp_path / "g.ampj")
    with zipfile.ZipFile(p, "w", zipfile.ZIP_STORED) as z:
        z.writestr("grid.dat", v.astype("<f8").tobytes())
        z.writestr("criticalinfo.json", json.dumps({"qmax": qmax, "qmin": 0, "gridSize": gs,
                                                    "stepSize": qmax / 8, "Params": [1, 0]}))
        z.writestr("header.json", json.dumps({"Old Header:": "hdr", "Header": {}}))
    g2, q2, h2, v2 = M.read_amp(p)
    assert (g2, q2, h2) == (gs, qmax, "hdr") and np.array_equal(v2, v)


def _ref():
    import oracle as O
    if not O.have_ref():
        pytest.skip("the reference's own Grid.cpp pin library is built only where the reference checkout is")
    import ctypes as C
    L = O.ref()
    D = C.POINTER(C.c_double)
    L.ref_amp_write.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_double, D]
    L.ref_amp_read.argtypes = [C.c_char_p, C.c_int, C.c_double, D, D, C.c_char_p, C.c_int]
    return L


@pytest.mark.parametrize("gs,qmax,header", [(20, 5.0, "made by dpx"), (36, 7.5, "a header"), (12, 2.0, "")])
def test_amp_files_pinned_to_the_reference_both_ways(tmp_path, gs, qmax, header):
    """The library's .amp writer and reader against the reference's own
    JacobianSphereGrid::ExportBinaryData / ImportBinaryData (Grid.cpp:847-963),
    compiled from the reference's sources: each reads the other's file to the
    bit, with the same step and header."""
    import ctypes as C
    L = _ref()
    v = _values(gs, 7 + gs)
    step = qmax / (gs // 2)
    ours = str(tmp_path / "dpx.amp")
    _lib.check(dpx.lib().dpx_amp_write(ours.encode(), header.encode(), gs, step, _lib.dptr(v)))
    got = np.zeros_like(v)
    st = C.c_double()
    buf = C.create_string_buffer(256)
    assert L.ref_amp_read(ours.encode(), gs, qmax, _lib.dptr(got), C.byref(st), buf, 256) == 0
    assert np.array_equal(got, v) and st.value == step
    theirs = str(tmp_path / "ref.amp")
    assert L.ref_amp_write(theirs.encode(), header.encode(), gs, qmax, _lib.dptr(v)) == 0
    g2, q2, h2, v2 = M.read_amp(theirs)
    assert g2 == gs and abs(q2 - qmax) < 1e-12 and h2 == header and np.array_equal(v2, v)
    assert open(ours, "rb").read() == open(theirs, "rb").read()  # the same bytes
