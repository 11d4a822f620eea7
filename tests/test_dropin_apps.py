"""The reference's own application programs (src/applications: drain, imbibe,
createMaskUBC, createInitFromMask, makeDiffSteps, makeRaw, convert2Raw),
unchanged and compiled with the reference's own headers, link against
libqssgpu.so alone (oracle/_ref/dropin, built by `make -C oracle dropin`
where the reference tree is present; skipped elsewhere).  convert2Raw, which
only reads and writes files, runs here end to end: its output files through
the GB300 library equal those of the same program linked against the
reference's own C sources (oracle/_ref/bin).  The drain program, run here
without a GPU, fails loudly through the library's error path."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import qssgpu as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "oracle", "_ref", "dropin")
REFBIN = os.path.join(ROOT, "oracle", "_ref", "bin")
APPS = ["drain", "imbibe", "createMaskUBC", "createInitFromMask", "makeDiffSteps", "makeRaw", "convert2Raw"]

pytestmark = pytest.mark.skipif(not os.path.isdir(DROPIN), reason="reference programs not built on this machine")


def _needed(path):
    out = subprocess.run(["readelf", "-d", path], check=True, capture_output=True, text=True).stdout
    return [line.split("[")[1].rstrip("]") for line in out.splitlines() if "(NEEDED)" in line]


@pytest.mark.parametrize("app", APPS)
def test_links_against_the_gb300_library_alone(app):
    needed = _needed(os.path.join(DROPIN, app))
    assert "libqssgpu.so" in needed
    assert not any("qss_ref" in n or "oracle" in n for n in needed)


def _inputs(lib, d, n=(10, 8, 7), steps=(1, 2)):
    """grid.gz, mask.gz and data_step_<k>.gz written through the library."""
    g = Q.make_grid(lib, n)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    rng = np.random.default_rng(sum(n))
    lib.writeGridToBinaryFile.argtypes = [C.POINTER(Q.Grid), C.c_char_p, C.c_int]
    lib.writeDataArrayQSS.argtypes = [Q.c_double_p, C.POINTER(Q.Grid), C.c_char_p, C.c_int]
    lib.writeGridToBinaryFile(C.byref(g), os.path.join(d, "grid").encode(), 1)
    mask = rng.standard_normal(shape)
    lib.writeDataArrayQSS(Q.dptr(mask), C.byref(g), os.path.join(d, "mask").encode(), 1)
    phis = {}
    for k in steps:
        phis[k] = rng.standard_normal(shape)
        lib.writeDataArrayQSS(Q.dptr(phis[k]), C.byref(g), os.path.join(d, f"data_step_{k}").encode(), 1)
    return g, mask, phis


@pytest.mark.parametrize("phase", ["n", "w"])
def test_convert2raw_output_equals_the_reference_build(tmp_path, phase):
    lib = Q.load(Q.GPU_LIB)
    outs = {}
    for name, exe in (("gb300", os.path.join(DROPIN, "convert2Raw")), ("reference", os.path.join(REFBIN, "convert2Raw"))):
        if not os.path.exists(exe):
            pytest.skip("reference build of convert2Raw not present")
        d = tmp_path / name
        d.mkdir()
        g, mask, phis = _inputs(lib, str(d))
        r = subprocess.run([exe, "1", "2", phase], cwd=d, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        outs[name] = {f: (d / f).read_bytes() for f in sorted(os.listdir(d)) if f.endswith(".raw")}
    assert outs["gb300"].keys() == outs["reference"].keys()
    assert len(outs["gb300"]) == 3
    for f in outs["gb300"]:
        assert outs["gb300"][f] == outs["reference"][f], f
    # and the contents are what the program means: the negated mask, phi itself
    assert np.array_equal(np.frombuffer(outs["gb300"]["mask.raw"], np.float64), -mask.ravel())
    tag = "nw" if phase == "n" else "w"
    assert np.array_equal(np.frombuffer(outs["gb300"][f"data_step_2_{tag}.raw"], np.float64), phis[2].ravel())


def test_drain_program_fails_loudly_without_a_gpu(tmp_path):
    lib = Q.load(Q.GPU_LIB)
    if lib.qssgpu_device_available():
        pytest.skip("a GPU is present")
    _inputs(lib, str(tmp_path), steps=(0,))
    (tmp_path / "input").write_text("a 1.2\namax 1.3\nspace_accur 2\ntime_accur 2\n")
    r = subprocess.run([os.path.join(DROPIN, "drain"), "input", "data_step_0.gz", "grid.gz", "mask.gz"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "qssgpu error" in r.stderr and "no CUDA device" in r.stderr
