"""Host-side parts of the C API in libqssgpu.so, no GPU needed: the option
file parser, grid construction and the binary grid / data-array formats.
Checked against expected values and, where it was built, against the
reference's own C implementation (oracle/_ref)."""
import ctypes as C
import gzip
import os

import numpy as np
import pytest

import qssgpu as Q

DECK = """\
outfile run/out_file
dx 0.04
a 0.3
amax 2.5
amin 0.2
b 0.05
dc 0.5
tmax 40
tplot 0.25
theta 35
space_accur 5
time_accur 3
eps_stop 0.02
err_check_zone 0.6
eps_coefficient 1.2
check_connectivity 1
checkpoint 1
center_inlet 0
reservoir_inlet 0
mask_reinit 0
init_step 4
vol_frac_max 0.9
use_satn_stop 0
use_var_theta 0
overlap 0.01
save_data 0
print_details 0
accuracy very_high
unknown_key 5
"""

FIELDS = ["dx", "a", "amax", "amin", "b", "dc", "tmax", "tplot", "theta", "order_space_accur", "order_time_accur",
          "eps_stop", "err_check_zone", "eps_coefficient", "check_connectivity", "checkpoint", "center_inlet",
          "reservoir_inlet", "mask_reinit", "init_step", "vol_frac_max", "use_satn_stop", "use_var_theta",
          "overlap", "save_data", "print_details", "accuracy_id", "tmax_r", "cmax"]


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(Q.GPU_LIB):
        pytest.fail("libqssgpu.so is not built")
    lib = Q.load(Q.GPU_LIB)
    lib.createOptionsFromInputFile.restype = C.POINTER(Q.Options)
    lib.createOptionsFromInputFile.argtypes = [C.c_char_p]
    return lib


def _parse(lib, path):
    f = lib.createOptionsFromInputFile
    f.restype = C.POINTER(Q.Options)
    f.argtypes = [C.c_char_p]
    op = f(path.encode())
    o = Q.Options()
    C.pointer(o)[0] = op[0]
    lib.destroyOptions(op)
    return o


def test_option_file(host, tmp_path):
    p = tmp_path / "deck"
    p.write_text(DECK)
    o = _parse(host, str(p))
    assert o.outfile == b"run/out_file" and o.path == b"run/"
    assert (o.a, o.amax, o.amin, o.b, o.dc, o.tmax, o.tplot) == (0.3, 2.5, 0.2, 0.05, 0.5, 40.0, 0.25)
    assert o.theta == 35 * 3.14159 / 180
    assert (o.order_space_accur, o.order_time_accur, o.init_step, o.accuracy_id) == (5, 3, 4, 3)
    assert (o.checkpoint, o.reservoir_inlet, o.mask_reinit, o.save_data, o.print_details) == (1, 0, 0, 0, 0)
    assert o.tmax_r == 10 * 0.04 and o.err_check_zone == 0.6 and o.overlap == 0.01


def test_option_file_matches_reference_parser(host, tmp_path):
    ref_path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                            "libqss_ref.so")
    if not os.path.exists(ref_path):
        pytest.skip("reference C build not present")
    ref = Q.load(ref_path)
    p = tmp_path / "deck"
    p.write_text(DECK)
    a, b = _parse(host, str(p)), _parse(ref, str(p))
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), f
    assert a.outfile == b.outfile and a.path == b.path and a.accuracy == b.accuracy


def test_defaults_match_reference_defaults(host):
    o = Q.default_options(host)
    assert (o.dx, o.tmax, o.tplot, o.a, o.b, o.eps_stop, o.dc, o.amax, o.amin) == \
        (0.04, 150.0, 0.5, 0.15, 0.04, 0.014, 0.1, 10.0, 0.05)
    assert (o.order_space_accur, o.order_time_accur, o.check_connectivity, o.use_satn_stop) == (3, 3, 1, 1)
    assert o.err_check_zone == 20 * 0.04 and o.vol_frac_max == 0.97 and o.eps_coefficient == 1.5


@pytest.mark.parametrize("acc", [0, 1, 2, 3])
def test_grid_and_files(host, oracle, tmp_path, acc):
    dims = (C.c_int * 3)(12, 9, 7)
    lo = (C.c_double * 3)(0.12, 0.12, 0.12)
    hi = (C.c_double * 3)(0.12 + 12 * 0.04, 0.12 + 9 * 0.04, 0.12 + 7 * 0.04)
    gh = host.createGridSetGridDims(3, dims, lo, hi, acc)
    go = oracle.createGridSetGridDims(3, dims, lo, hi, acc)
    assert bytes(C.string_at(gh, C.sizeof(Q.Grid))) == bytes(C.string_at(go, C.sizeof(Q.Grid)))
    g = gh[0]
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        host.writeGridToBinaryFile(gh, b"grid", 1)
        f = host.readGridFromBinaryFile
        f.restype = C.POINTER(Q.Grid)
        f.argtypes = [C.c_char_p]
        g2 = f(b"grid.gz")
        assert bytes(C.string_at(g2, C.sizeof(Q.Grid))) == bytes(C.string_at(gh, C.sizeof(Q.Grid)))
        n = g.num_gridpts
        data = np.random.default_rng(acc).standard_normal(n)
        host.writeDataArrayQSS.argtypes = [Q.c_double_p, C.POINTER(Q.Grid), C.c_char_p, C.c_int]
        host.writeDataArrayQSS(Q.dptr(data), gh, b"arr", 1)
        with gzip.open("arr.gz", "rb") as fh:
            raw = fh.read()
        dims3 = np.frombuffer(raw[:12], dtype=np.int32)
        assert list(dims3) == list(g.grid_dims_ghostbox)
        assert np.array_equal(np.frombuffer(raw[12:], dtype=np.float64), data)
        rd = host.readDataArrayQSS
        rd.restype = Q.c_double_p
        rd.argtypes = [C.POINTER(C.c_int), C.c_char_p]
        d3 = (C.c_int * 3)()
        back = rd(d3, b"arr.gz")
        assert list(d3) == list(g.grid_dims_ghostbox)
        assert np.array_equal(np.ctypeslib.as_array(back, (n,)), data)
    finally:
        os.chdir(cwd)


def test_gzip_members_round_trip(host, tmp_path):
    """A saved array larger than one compression chunk is written as several
    gzip members deflated in parallel; gzip readers (Python's and the
    library's own readDataArrayQSS) return exactly the reference layout:
    int[3] ghost-box dims then the values."""
    dims = (C.c_int * 3)(150, 140, 130)
    lo = (C.c_double * 3)(0.12, 0.12, 0.12)
    hi = (C.c_double * 3)(0.12 + 150 * 0.04, 0.12 + 140 * 0.04, 0.12 + 130 * 0.04)
    gh = host.createGridSetGridDims(3, dims, lo, hi, 1)
    g = gh[0]
    n = g.num_gridpts
    assert n * 8 > (16 << 20)  # at least two data members
    data = np.random.default_rng(5).standard_normal(n)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        (tmp_path / "big").write_bytes(b"stale")  # the reference's gzip -f leaves no raw file behind
        host.writeDataArrayQSS.argtypes = [Q.c_double_p, C.POINTER(Q.Grid), C.c_char_p, C.c_int]
        host.writeDataArrayQSS(Q.dptr(data), gh, b"big", 1)
        assert not os.path.exists("big") and os.path.exists("big.gz")
        with gzip.open("big.gz", "rb") as fh:
            raw = fh.read()
        assert list(np.frombuffer(raw[:12], dtype=np.int32)) == list(g.grid_dims_ghostbox)
        assert np.array_equal(np.frombuffer(raw[12:], dtype=np.float64), data)
        rd = host.readDataArrayQSS
        rd.restype = Q.c_double_p
        rd.argtypes = [C.POINTER(C.c_int), C.c_char_p]
        d3 = (C.c_int * 3)()
        back = rd(d3, b"big.gz")
        assert np.array_equal(np.ctypeslib.as_array(back, (n,)), data)
    finally:
        os.chdir(cwd)


def _reader(host):
    rd = host.readDataArrayQSS
    rd.restype = Q.c_double_p
    rd.argtypes = [C.POINTER(C.c_int), C.c_char_p]
    return rd


def _small_grid(host):
    dims = (C.c_int * 3)(6, 5, 4)
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(0.24, 0.20, 0.16)
    return host.createGridSetGridDims(3, dims, lo, hi, 1)


def test_file_names_passed_to_gzip_as_one_argument(host, tmp_path):
    """Compressed array files whose names hold a space, a single quote or a
    shell metacharacter, or whose path is longer than 256 bytes, are
    decompressed, read and compressed again in place by the gzip programs,
    the name reaching them as one argument."""
    gh = _small_grid(host)
    n = gh[0].num_gridpts
    data = np.random.default_rng(9).standard_normal(n)
    deep = tmp_path / ("d" * 120) / ("e" * 120)
    deep.mkdir(parents=True)
    host.writeDataArrayQSS.argtypes = [Q.c_double_p, C.POINTER(Q.Grid), C.c_char_p, C.c_int]
    rd = _reader(host)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        for path in ("a b", "it's", "x;touch pwned", str(deep / "long")):
            assert len(str(deep / "long")) > 256
            host.writeDataArrayQSS(Q.dptr(data), gh, path.encode(), 1)
            assert os.path.exists(path + ".gz") and not os.path.exists(path)
            d3 = (C.c_int * 3)()
            back = rd(d3, (path + ".gz").encode())
            assert back, path
            assert list(d3) == list(gh[0].grid_dims_ghostbox)
            assert np.array_equal(np.ctypeslib.as_array(back, (n,)), data), path
            assert os.path.exists(path + ".gz") and not os.path.exists(path), path
        assert not os.path.exists("pwned")
    finally:
        os.chdir(cwd)


def test_bad_array_headers_read_as_null(host, tmp_path):
    """An array file without a valid header (too short, or a size that is not
    positive) reads as NULL instead of sizing an allocation from it; a
    payload shorter than the header says leaves the rest zero."""
    rd = _reader(host)
    p = tmp_path / "bad"
    for content in (b"", b"\x01\x00\x00\x00", np.array([4, -1, 2], np.int32).tobytes(),
                    np.array([0, 5, 5], np.int32).tobytes()):
        p.write_bytes(content)
        d3 = (C.c_int * 3)()
        assert not rd(d3, str(p).encode())
    p.write_bytes(np.array([2, 2, 2], np.int32).tobytes() + np.arange(3, dtype=np.float64).tobytes())
    d3 = (C.c_int * 3)()
    back = rd(d3, str(p).encode())
    assert list(d3) == [2, 2, 2]
    assert np.ctypeslib.as_array(back, (8,)).tolist() == [0.0, 1.0, 2.0] + [0.0] * 5


def test_option_file_short_lines(host, tmp_path):
    """Lines shorter than the letter positions that tell keywords apart
    ('c', 'd', 'do 0', 'v 1', 'u 1', 'e 1') set nothing, whatever the lines
    before them held."""
    p = tmp_path / "deck"
    p.write_text("err_check_zone 0.7\nc\nvol_frac_max 0.8\nd\ndo 0\nuse_var_theta 1\nv 1\nu 1\ne 1\na 0.3\n")
    o = _parse(host, str(p))
    d = _parse(host, str(tmp_path / "missing"))  # the defaults
    assert o.a == 0.3 and o.err_check_zone == 0.7 and o.vol_frac_max == 0.8 and o.use_var_theta == 1
    for f in FIELDS:
        if f not in ("a", "err_check_zone", "vol_frac_max", "use_var_theta"):
            assert getattr(o, f) == getattr(d, f), f
