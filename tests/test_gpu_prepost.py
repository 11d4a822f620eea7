"""Pre- and post-processing on the GPU against the oracle's restatement of
the reference (qss_general_util.c qss_reinitialize_mask; the createMaskUBC,
createInitFromMask and makeDiffSteps programs), bit for bit on every array
the reference writes."""
import ctypes as C

import numpy as np
import pytest

import qssgpu as Q
import synthetic as S
from qss_cases import clone, diff_arrays, options, pack_case

pytestmark = pytest.mark.gpu


def test_reinitialize_mask(gpu, oracle):
    g, v = pack_case(oracle, 20, seed=51)
    out = []
    for lib in (gpu, oracle):
        w = clone(v)
        lib.qss_reinitialize_mask(C.byref(w.p), C.byref(g), C.byref(options(lib)))
        out.append(w)
    Q.check(gpu)
    assert diff_arrays(out[0], out[1]) == {}


@pytest.mark.parametrize("seed", [1, 2])
def test_create_mask_ubc(gpu, oracle, seed):
    n = 20
    g, v = pack_case(oracle, n, seed=seed)
    m = S.overlapping(n, radius_vox=4.0, porosity=0.4, seed=seed).mask()
    s = slice(3, n + 3)
    img = np.where(m[s, s, s] > 0, 255, 0).astype(np.uint8)
    img[0, 0, :3] = (1, 254, 128)  # only 255 is grain
    img = np.ascontiguousarray(img)
    out = []
    for lib, fn in ((gpu, "qssgpu_create_mask_ubc"), (oracle, "oracle_create_mask_ubc")):
        w = clone(v)
        assert getattr(lib, fn)(img.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(w.p), C.byref(g),
                                C.byref(options(lib))) == 0
        out.append(w)
    Q.check(gpu)
    assert diff_arrays(out[0], out[1]) == {}
    assert np.all(np.sign(out[0]["mask"][s, s, s][img == 255]) >= 0)


@pytest.mark.parametrize("center", [0, 1])
def test_create_init_from_mask(gpu, oracle, center):
    g, v = pack_case(oracle, 24, seed=7)
    out = []
    for lib, fn in ((gpu, "qssgpu_create_init_from_mask"), (oracle, "oracle_create_init_from_mask")):
        w = clone(v)
        o = options(lib)
        o.center_inlet = center
        assert getattr(lib, fn)(C.byref(w.p), C.byref(g), C.byref(o)) == 0
        out.append(w)
    Q.check(gpu)
    assert diff_arrays(out[0], out[1]) == {}


@pytest.mark.parametrize("shift,expect", [(0.0, 0), (0.35, 1)])
def test_diff_steps(gpu, oracle, shift, expect):
    """Two saved steps of a drainage: a = the earlier, b = the later (larger
    non-wetting region); the lens between them, its labels and the
    percolation check, for a case that does not percolate and one that does."""
    g, v = pack_case(oracle, 22, seed=9)
    rng = np.random.default_rng(11)
    x = np.arange(v.shape[2])[None, None, :] * 0.04
    a = np.ascontiguousarray(np.maximum(v["mask"], x - 0.3 + 0.01 * rng.standard_normal(v.shape)))
    b = np.ascontiguousarray(np.maximum(v["mask"], x - 0.6 - shift + 0.01 * rng.standard_normal(v.shape)))
    res = []
    for lib, fn in ((gpu, "qssgpu_diff_steps"), (oracle, "oracle_diff_steps")):
        diff = np.zeros(v.shape)
        conn = np.full(v.shape, 7.0)
        perc = C.c_int(-1)
        assert getattr(lib, fn)(Q.dptr(a), Q.dptr(b), C.byref(g), Q.dptr(diff), Q.dptr(conn), C.byref(perc)) == 0
        res.append((diff, conn, perc.value))
    Q.check(gpu)
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][2] == res[1][2] == expect
    assert np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("phase", ["m", "n", "w"])
def test_phase_uchar(gpu, oracle, phase):
    """makeRaw's 0/1 phase images (ghost box and packed fill box) of the mask,
    the non-wetting phase and the wetting phase, with exact and signed zeros
    in phi and the mask."""
    g, v = pack_case(oracle, 21, seed=13)
    rng = np.random.default_rng(17)
    phi = v["phi"].copy()
    mask = v["mask"].copy()
    for arr in (phi, mask):
        sel = rng.random(arr.shape) < 0.05
        arr[sel] = rng.choice([0.0, -0.0, 1e-300, -1e-300], sel.sum())
    nfb = 21 ** 3
    res = []
    for lib, fn in ((gpu, "qssgpu_phase_uchar"), (oracle, "oracle_phase_uchar")):
        full = np.full(v.shape, 7, dtype=np.uint8)
        fb = np.full(nfb, 7, dtype=np.uint8)
        rc = getattr(lib, fn)(Q.dptr(phi), Q.dptr(mask), C.byref(g), phase.encode(),
                              full.ctypes.data_as(C.POINTER(C.c_ubyte)), fb.ctypes.data_as(C.POINTER(C.c_ubyte)))
        assert rc == 0
        res.append((full, fb))
    Q.check(gpu)
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    assert set(np.unique(res[0][0])) <= {0, 1} and res[0][0].any()
    # the packed image is the fill box of the full one
    assert np.array_equal(res[0][1].reshape(21, 21, 21), res[0][0][3:24, 3:24, 3:24])
