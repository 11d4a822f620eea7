"""The C-ABI boundary without a GPU: the library loads, exports every function
include/lsmpqs_gpu.h declares, and the public structs are laid out exactly as
the reference's headers lay them out (FP64 build)."""
import ctypes as C
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import qssgpu as Q
from abi_probe import STRUCTS, probe_source

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
LAYOUT = os.path.join(ROOT, "tests", "golden", "abi_layout.json")


def declared_functions():
    """Function names declared in include/lsmpqs_gpu.h."""
    src = open(os.path.join(INCLUDE, "lsmpqs_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#define[^\n]*\n", "\n", src)
    names = set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src))
    return sorted(n for n in names if n not in {"if", "sizeof"} and not n.isupper())


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(Q.GPU_LIB):
        pytest.fail("libqssgpu.so is not built (run __graft_entry__.build())")
    return C.CDLL(Q.GPU_LIB)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_header_compiles_as_c_and_cxx():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write('#include "lsmpqs_gpu.h"\nint main(void){ return qssgpu_last_error(); }\n')
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I" + INCLUDE, src], check=True)
        subprocess.run(["g++", "-x", "c++", "-Wall", "-Werror", "-fsyntax-only", "-I" + INCLUDE, src], check=True)


def test_struct_layout_matches_reference():
    with open(LAYOUT) as f:
        want = json.load(f)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "p.c")
        with open(src, "w") as f:
            f.write(probe_source('#include "lsmpqs_types.h"\n'))
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I" + INCLUDE, src, "-o", exe], check=True)
        got = json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    assert got == want
    for cname, cls in STRUCTS.items():  # and the Python binding agrees
        assert C.sizeof(cls) == want[f"{cname}.sizeof"]
        for name, *_ in cls._fields_:
            assert getattr(cls, name).offset == want[f"{cname}.{name}"]


def test_no_device_is_reported_not_crashed(lib):
    """On a machine without a GPU every entry point fails loudly and cleanly."""
    L = Q.load(Q.GPU_LIB)
    if L.qssgpu_device_available():
        pytest.skip("a GPU is present")
    g = Q.make_grid(L, 8)
    v = Q.Volume(g)
    o = Q.default_options(L)
    L.qssgpu_clear_error()
    t = L.constCurvModel3d(C.byref(o), C.byref(v.p), C.byref(g), None)
    assert t == -1
    assert L.qssgpu_last_error() != 0
    assert b"CUDA" in L.qssgpu_error_string() or b"device" in L.qssgpu_error_string()
    L.qssgpu_clear_error()


def test_host_side_argument_checks(lib):
    """Checks that run before any device work: the batch rejects volumes that
    share arrays or options or have a NULL pointer, and without a GPU the page-locked allocator and
    the phase-image call fail cleanly with an error code."""
    L = Q.load(Q.GPU_LIB)
    g = Q.make_grid(L, 8)
    v = Q.Volume(g)
    o1, o2 = Q.default_options(L), Q.default_options(L)
    arr_o = (C.POINTER(Q.Options) * 2)(C.pointer(o1), C.pointer(o2))
    arr_p = (C.POINTER(Q.QSSDataArrays) * 2)(C.pointer(v.p), C.pointer(v.p))  # shared arrays
    arr_g = (C.POINTER(Q.Grid) * 2)(C.pointer(g), C.pointer(g))
    L.qssgpu_clear_error()
    assert L.qssgpu_ladder_batch(1, 2, arr_o, arr_p, arr_g, None, None, 0) == 2
    assert b"share" in L.qssgpu_error_string()
    L.qssgpu_clear_error()
    w = Q.Volume(g)
    arr_p = (C.POINTER(Q.QSSDataArrays) * 2)(C.pointer(v.p), C.pointer(w.p))
    arr_g = (C.POINTER(Q.Grid) * 2)(C.pointer(g), None)  # a NULL grid entry
    assert L.qssgpu_ladder_batch(1, 2, arr_o, arr_p, arr_g, None, None, 0) == 2
    assert b"NULL" in L.qssgpu_error_string()
    L.qssgpu_clear_error()
    if L.qssgpu_device_available():
        return
    assert not L.qssgpu_host_alloc(1 << 20)
    assert L.qssgpu_last_error() != 0
    L.qssgpu_clear_error()
    full = np.zeros(v.shape, dtype=np.uint8)
    rc = L.qssgpu_phase_uchar(Q.dptr(v["phi"]), Q.dptr(v["mask"]), C.byref(g), b"n",
                              full.ctypes.data_as(C.POINTER(C.c_ubyte)), None)
    assert rc != 0 and L.qssgpu_last_error() != 0
    L.qssgpu_clear_error()


def test_axis_variant_settings(lib):
    """The axis-pass form setting takes -1 (default: tiles), 0, 1 (window
    forms), 2 (tuned), 3 and 4 (tiles of 16 x 16 and 8 x 27), clamps larger
    values to 4, returns the previous setting, and the tuned shape table
    starts empty and can be cleared."""
    L = Q.load(Q.GPU_LIB)
    prev = L.qssgpu_set_axis_variant(2)
    try:
        assert L.qssgpu_set_axis_variant(7) == 2
        assert L.qssgpu_set_axis_variant(0) == 4
        assert L.qssgpu_set_axis_variant(-5) == 0
    finally:
        L.qssgpu_set_axis_variant(prev)
    L.qssgpu_axis_tuning_reset()
    assert L.qssgpu_axis_tuning(None, 0) == 0


def test_axis_tuning_file_round_trip(lib, tmp_path):
    """Tuned launch shapes saved to a file and loaded back (no GPU needed):
    valid rows are added, a shape already in the table keeps its pick, and a
    file with any invalid row (a segment length of 0 or longer than the line,
    an unknown form, a tile form whose segment is not its 16 voxels, a bad
    level or axis, a short row) adds nothing."""
    L = Q.load(Q.GPU_LIB)
    L.qssgpu_axis_tuning_reset()
    good = tmp_path / "shapes"
    good.write_text("# level axis lanes lines_per_lane line form seg_len\n"
                    "2 0 512 512 512 1 128\n2 1 512 512 512 3 16\n\n  2 2 512 512 512 0 16\n")
    assert L.qssgpu_axis_tuning_load(str(good).encode()) == 3
    rows = (C.c_int * 21)()
    assert L.qssgpu_axis_tuning(rows, 7) == 3
    got = sorted(tuple(rows[7 * i:7 * i + 7]) for i in range(3))
    assert got == [(2, 0, 512, 512, 512, 1, 128), (2, 1, 512, 512, 512, 3, 16), (2, 2, 512, 512, 512, 0, 16)]
    # the first pick of a shape stays
    other = tmp_path / "other"
    other.write_text("2 0 512 512 512 0 64\n1 0 40 40 40 0 20\n")
    assert L.qssgpu_axis_tuning_load(str(other).encode()) == 2
    assert L.qssgpu_axis_tuning(None, 0) == 4
    back = tmp_path / "saved"
    assert L.qssgpu_axis_tuning_save(str(back).encode()) == 4
    assert "2 0 512 512 512 1 128" in back.read_text()
    assert "2 0 512 512 512 0 64" not in back.read_text()
    for bad in ("2 0 512 512 512 1 0", "2 0 512 512 512 1 513", "2 0 512 512 512 2 64", "2 0 512 512 512 3 17",
                "3 0 8 8 8 0 8",
                "2 3 8 8 8 0 8", "2 0 8 8 8 0", "2 0 8 8 8 0 8 9", "2 0 -8 8 8 0 8"):
        f = tmp_path / "bad"
        f.write_text("2 1 64 64 64 0 16\n" + bad + "\n")
        assert L.qssgpu_axis_tuning_load(str(f).encode()) == -1, bad
    assert L.qssgpu_axis_tuning(None, 0) == 4
    assert L.qssgpu_axis_tuning_load(str(tmp_path / "missing").encode()) == -1
    L.qssgpu_axis_tuning_reset()
    assert L.qssgpu_axis_tuning_load(str(back).encode()) == 4
    L.qssgpu_axis_tuning_reset()
