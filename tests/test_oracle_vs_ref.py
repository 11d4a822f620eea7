"""Pins the oracle's restated C drivers to the reference's own C drivers
(src/level_set_evolution, src/connectivity, src/reinitialization,
src/utilities compiled unchanged from the reference tree into oracle/_ref and
linked against the same restated kernels), and the restated pre/post-processing
programs to the reference's own programs built the same way.  Only where that
build exists."""
import ctypes as C
import gzip
import os
import subprocess

import numpy as np
import pytest

import qssgpu as Q
from qss_cases import clone, diff_arrays, in_tmpdir, options, pack_case, prepare_model


def _both(ref, oracle, fn, threads=1):
    out = []
    for lib in (ref, oracle):
        lib.oracle_set_threads(threads)
        try:
            out.append(fn(lib))
        finally:
            lib.oracle_set_threads(1)
    return out


@pytest.mark.parametrize("theta,space,time,threads,n", [
    (0, 2, 2, 1, 20), (0, 3, 3, 2, 20), (0, 5, 1, 3, 20), (10, 2, 2, 1, 20), (30, 5, 3, 4, 20), (40, 3, 3, 1, 20),
    (60, 5, 3, 2, 20),
    # non-cubic fill boxes (the ENO3 x stencil's phi(i+3,j,j) needs y within z)
    (10, 5, 3, 3, (19, 13, 16)), (0, 2, 2, 2, (15, 18, 12)), (20, 3, 3, 2, (14, 11, 17))])
def test_drain_imbibe_drivers(ref, oracle, theta, space, time, threads, n):
    g, v = pack_case(oracle, n, seed=theta + space)

    def run(lib):
        w = clone(v)
        o = options(lib, theta, space, time, tmax=0.04, tplot=0.015, a=1.2)
        o.amax = 1.2 + 2.5 * o.b * o.dc
        o.amin = 1.15

        def go(d):
            fp = Q.libc_fopen("out")
            lib.drain_model3d(C.byref(o), C.byref(w.p), C.byref(g), fp)
            o.a = 1.3
            lib.imbibe_model3d(C.byref(o), C.byref(w.p), C.byref(g), fp)
            Q.libc_fclose(fp)

        in_tmpdir(go)
        return w, (o.b_max_over_dx, o.max_U_over_dx, o.overlap, o.phi_nw_ind, o.phi_w_ind)

    (wr, sr), (wo, so) = _both(ref, oracle, run, threads)
    assert sr == so
    assert diff_arrays(wr, wo) == {}


@pytest.mark.parametrize("center", [0, 1])
def test_trap_and_labels(ref, oracle, center):
    g, v = pack_case(oracle, 22, seed=30 + center)
    rng = np.random.default_rng(center)
    v["phi"][...] = np.maximum(0.03 * rng.standard_normal(v.shape), v["mask"])

    def run(lib):
        w = clone(v)
        o = options(lib)
        o.center_inlet = center
        lib.getMainInd_new(C.byref(o), C.byref(w.p), C.byref(g))
        lib.initializeDisconnectedMasks(w["mask_nw"].ctypes.data_as(Q.c_double_p), C.byref(g))
        lib.trapComponents_mask(C.byref(w.p), C.byref(g), C.byref(o))
        return w

    wr, wo = _both(ref, oracle, run)
    assert diff_arrays(wr, wo) == {}


def test_model_direct_call(ref, oracle):
    g, v = pack_case(oracle, 18, seed=41)

    def run(lib):
        w = clone(v)
        o = options(lib, 25, 5, 3, tmax=0.03, tplot=0.01)
        prepare_model(lib, o, w, 1.25)
        fp_box = []

        def go(d):
            fp = Q.libc_fopen("out")
            t = lib.constCurvModel3d(C.byref(o), C.byref(w.p), C.byref(g), fp)
            Q.libc_fclose(fp)
            return t

        return in_tmpdir(go), w

    (tr, wr), (to, wo) = _both(ref, oracle, run, threads=3)
    assert tr == to
    assert diff_arrays(wr, wo) == {}


def test_reinitialize_mask(ref, oracle):
    """qss_reinitialize_mask: the mask and its side effects on scratch1,
    scratch2, lse_rhs and phi_next."""
    g, v = pack_case(oracle, 18, seed=41)

    def run(lib):
        w = clone(v)
        lib.qss_reinitialize_mask(C.byref(w.p), C.byref(g), C.byref(options(lib)))
        return w

    wr, wo = _both(ref, oracle, run)
    assert diff_arrays(wr, wo) == {}


# ---------------------------------------------------------------------------
# the reference's pre/post-processing programs (src/applications), built from
# their own sources into oracle/_ref/bin, against the oracle's restatements

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "bin")


def _program(name):
    path = os.path.join(BIN, name)
    if not os.path.exists(path):
        pytest.skip(f"reference program {name} not built on this machine")
    return path


def _write_qss(path, g, data):
    """writeDataArrayQSS's layout: ghost-box dims (3 int32) then the doubles, gzipped."""
    with gzip.open(path, "wb") as fh:
        fh.write(np.asarray(list(g.grid_dims_ghostbox), dtype=np.int32).tobytes())
        fh.write(np.ascontiguousarray(data, dtype=np.float64).tobytes())


def _read_qss(path, n):
    with gzip.open(path, "rb") as fh:
        raw = fh.read()
    return np.frombuffer(raw[12:], dtype=np.float64, count=n)


def _write_grid(ref, g):
    ref.writeGridToBinaryFile.argtypes = [C.POINTER(Q.Grid), C.c_char_p, C.c_int]
    ref.writeGridToBinaryFile(C.byref(g), b"grid", 1)


def _run(args):
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]


def test_create_mask_ubc_program(ref, oracle, tmp_path):
    """createMaskUBC (createMaskUBC.c:76-112): the reference program on an 8-bit
    image against oracle_create_mask_ubc, every mask value bit for bit."""
    n = (14, 12, 11)
    prog = _program("createMaskUBC")
    rng = np.random.default_rng(71)
    img = np.where(rng.random(n[::-1]) < 0.4, 255, 0).astype(np.uint8)  # z, y, x: x fastest
    img[2:6, 3:8, 4:9] = 255
    (tmp_path / "img.raw").write_bytes(img.tobytes())
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _run([prog, "img.raw", str(n[0]), str(n[1]), str(n[2])])
    finally:
        os.chdir(cwd)
    g = Q.make_grid(oracle, n)
    v = Q.Volume(g)
    o = Q.default_options(oracle)
    rc = oracle.oracle_create_mask_ubc(img.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(v.p), C.byref(g),
                                       C.byref(o))
    assert rc == 0
    want = _read_qss(tmp_path / "mask.gz", g.num_gridpts)
    assert np.array_equal(v["mask"].ravel(), want)


@pytest.mark.parametrize("center", [0, 1])
def test_create_init_from_mask_program(ref, oracle, tmp_path, center):
    prog = _program("createInitFromMask")
    g, v = pack_case(oracle, 16, seed=72 + center)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _write_grid(ref, g)
        _write_qss("mask.gz", g, v["mask"])
        with open("opts.in", "w") as fh:
            fh.write(f"center_inlet {center}\n")
        _run([prog, "mask.gz", "grid.gz", "opts.in"])
        want = _read_qss("data_init.gz", g.num_gridpts)
    finally:
        os.chdir(cwd)
    o = Q.default_options(oracle)
    o.center_inlet = center
    w = clone(v)
    assert oracle.oracle_create_init_from_mask(C.byref(w.p), C.byref(g), C.byref(o)) == 0
    assert np.array_equal(w["phi"].ravel(), want)


@pytest.mark.parametrize("shift", [0.0, 0.35])
def test_make_diff_steps_program(ref, oracle, tmp_path, shift):
    prog = _program("makeDiffSteps")
    g, v = pack_case(oracle, 18, seed=74)
    rng = np.random.default_rng(75)
    x = np.arange(v.shape[2])[None, None, :] * 0.04
    a = np.ascontiguousarray(np.maximum(v["mask"], x - 0.3 + 0.01 * rng.standard_normal(v.shape)))
    b = np.ascontiguousarray(np.maximum(v["mask"], x - 0.5 - shift + 0.01 * rng.standard_normal(v.shape)))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _write_grid(ref, g)
        _write_qss("data_step_1.gz", g, a)
        _write_qss("data_step_2.gz", g, b)
        _run([prog, "1", "2"])
        want = np.fromfile("diff_steps_1_2.raw", dtype=np.float64)
        conn = "diff_steps_1_2_connected_only.raw"
        want_conn = np.fromfile(conn, dtype=np.float64) if os.path.exists(conn) else None
    finally:
        os.chdir(cwd)
    diff = np.zeros(v.shape)
    connected = np.zeros(v.shape)
    perc = C.c_int(-1)
    assert oracle.oracle_diff_steps(Q.dptr(a), Q.dptr(b), C.byref(g), Q.dptr(diff), Q.dptr(connected),
                                    C.byref(perc)) == 0
    assert np.array_equal(diff.ravel(), want)
    assert perc.value == (want_conn is not None)
    if want_conn is not None:
        assert np.array_equal(connected.ravel(), want_conn)


@pytest.mark.parametrize("phase", ["n", "w"])
def test_make_raw_program(ref, oracle, tmp_path, phase):
    """makeRaw (makeRaw.c:76-135): the mask and phase images against
    oracle_phase_uchar.  The reference writes the phase `_fb` images with the
    ghost-box byte count from a fill-box buffer; only their fill-box bytes
    are defined and compared."""
    prog = _program("makeRaw")
    g, v = pack_case(oracle, 15, seed=76)
    nfb = 15 ** 3
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        _write_grid(ref, g)
        _write_qss("mask.gz", g, v["mask"])
        _write_qss("data_step_3.gz", g, v["phi"])
        _run([prog, "3", "3", phase])
        tag = "nw" if phase == "n" else "w"
        files = {k: open(k, "rb").read() for k in ("mask.raw", "mask_fb.raw", f"data_step_3_{tag}_uchar.raw",
                                                     f"data_step_3_{tag}_uchar_fb.raw")}
    finally:
        os.chdir(cwd)
    n = g.num_gridpts

    def img(ph):
        full = np.zeros(n, dtype=np.uint8)
        fb = np.zeros(nfb, dtype=np.uint8)
        assert oracle.oracle_phase_uchar(Q.dptr(v["phi"]), Q.dptr(v["mask"]), C.byref(g), ph.encode(),
                                         full.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                         fb.ctypes.data_as(C.POINTER(C.c_ubyte))) == 0
        return full, fb

    mfull, mfb = img("m")
    pfull, pfb = img(phase)
    assert files["mask.raw"][12:] == mfull.tobytes()
    assert files["mask_fb.raw"][-nfb:] == mfb.tobytes()
    assert files[f"data_step_3_{tag}_uchar.raw"][12:] == pfull.tobytes()
    assert files[f"data_step_3_{tag}_uchar_fb.raw"][12:12 + nfb] == pfb.tobytes()
