"""Path-level parity: the GB300 implementations of the reference's C entry
points (trapping, labelling, reinitialisation, the constant-curvature model
and the drainage / imbibition ladders) against the oracle on the same seeded
inputs.  Every array of QSS_DataArrays is compared bit for bit; the volume
used for the saturation is summed in the reference's loop order, so the
control flow (number of outer iterations, stopping tests) is identical too."""
import ctypes as C
import os

import numpy as np
import pytest

import qssgpu as Q
from qss_cases import clone, diff_arrays, in_tmpdir, options, pack_case, prepare_model

pytestmark = pytest.mark.gpu


def _label_oracle(bin_):
    """Independent check of the label rule: components of the 26-neighbourhood
    graph named by their largest linear index (scipy), 0 for background."""
    from scipy import ndimage

    lab, n = ndimage.label(bin_, structure=np.ones((3, 3, 3)))
    out = np.zeros(bin_.shape, dtype=np.int32)
    flat = np.arange(bin_.size).reshape(bin_.shape)
    mx = ndimage.maximum(flat, lab, index=np.arange(1, n + 1))
    for i, m in enumerate(mx, start=1):
        out[lab == i] = int(m)
    return out


@pytest.mark.parametrize("density", [0.2, 0.45, 0.7])
def test_find_connectivity_labels(gpu, oracle, density):
    g, v = pack_case(oracle, 24)
    rng = np.random.default_rng(int(density * 100))
    v["phi_bin"][...] = (rng.random(v.shape) < density).astype(np.uint8)
    v["phi_bin"][0, 0, 0] = 1
    a, b = clone(v), clone(v)
    gpu.findConnectivity3d(C.byref(a.p), C.byref(g))
    oracle.findConnectivity3d(C.byref(b.p), C.byref(g))
    Q.check(gpu)
    assert np.array_equal(a["connectivity"], b["connectivity"])
    assert np.array_equal(a["connectivity"], _label_oracle(v["phi_bin"].astype(bool)))


@pytest.mark.parametrize("center", [0, 1])
def test_trap_components(gpu, oracle, center):
    g, v = pack_case(oracle, 24, seed=2)
    rng = np.random.default_rng(5)
    v["phi"][...] = 0.04 * np.sin(np.arange(v["phi"].size).reshape(v.shape) * 0.37) + 0.01 * rng.standard_normal(v.shape)
    v["phi"][...] = np.maximum(v["phi"], v["mask"])
    o = options(oracle)
    o.center_inlet = center
    oracle.getMainInd_new(C.byref(o), C.byref(v.p), C.byref(g))
    oracle.initializeDisconnectedMasks(v["mask_nw"].ctypes.data_as(Q.c_double_p), C.byref(g))
    v["mask_nw"][:, :, :10] = np.where(rng.random((v.shape[0], v.shape[1], 10)) < 0.05, 0.03, v["mask_nw"][:, :, :10])
    a, b = clone(v), clone(v)
    gpu.trapComponents_mask(C.byref(a.p), C.byref(g), C.byref(o))
    oracle.trapComponents_mask(C.byref(b.p), C.byref(g), C.byref(o))
    Q.check(gpu)
    assert diff_arrays(a, b) == {}
    assert (b["mask_w"] > 0).any() or (b["mask_nw"] > 0).any()


@pytest.mark.parametrize("emu", [0, 1, 2])
def test_reinitialize(gpu, oracle, emu):
    g, v = pack_case(oracle, 24, seed=3)
    o = options(oracle)
    outs = []
    prev = gpu.qssgpu_set_emu_level(emu)
    try:
        for lib in (gpu, oracle):
            a = v["mask"].copy()
            lib.reinitializeSubcellFix3d(Q.dptr(a), C.byref(g), C.byref(o))
            outs.append(a)
    finally:
        gpu.qssgpu_set_emu_level(prev)
    Q.check(gpu)
    assert np.array_equal(outs[0], outs[1])


def _model(lib, v, o, var, a0):
    def go(_):
        fp = Q.libc_fopen("out")
        try:
            if var:
                return lib.constCurvModel3d(C.byref(o), C.byref(v.p), C.byref(v.g), fp)
            return lib.constCurvModel3dNoVar(C.byref(o), C.byref(v.p), C.byref(v.g), fp, a0)
        finally:
            Q.libc_fclose(fp)

    return in_tmpdir(go)


@pytest.mark.parametrize("theta,space,time", [(0, 2, 2), (0, 3, 3), (0, 5, 1), (40, 5, 3), (10, 2, 2), (30, 3, 3)])
def test_const_curv_model(gpu, oracle, theta, space, time):
    g, v = pack_case(oracle, 24, seed=1)
    o_g = options(gpu, theta, space, time, tmax=0.03, tplot=0.012)
    o_o = options(oracle, theta, space, time, tmax=0.03, tplot=0.012)
    a0 = 1.25
    vg, vo = clone(v), clone(v)
    prepare_model(oracle, o_g, vg, a0)
    prepare_model(oracle, o_o, vo, a0)
    gpu.setSpaceDerivFunc(C.byref(g), C.byref(o_g))
    tg = _model(gpu, vg, o_g, theta > 0, a0)
    to = _model(oracle, vo, o_o, theta > 0, a0)
    Q.check(gpu)
    assert tg == to
    assert diff_arrays(vg, vo) == {}


@pytest.mark.parametrize("split,emu,variant", [(0, 2, -1), (1, 0, -1), (1, 1, 1), (1, 2, 0), (1, 2, 1),
                                               (1, 2, 2), (1, 2, 3)])
def test_const_curv_model_weno_modes(gpu, oracle, split, emu, variant):
    """WENO5 + TVD-RK3 with variable coefficients through the fused stage
    kernel and through the axis passes (both forms) + combine: all equal the
    oracle."""
    g, v = pack_case(oracle, 22, seed=4)
    o_g = options(gpu, 40, 5, 3, tmax=0.02, tplot=0.01)
    o_o = options(oracle, 40, 5, 3, tmax=0.02, tplot=0.01)
    vg, vo = clone(v), clone(v)
    prepare_model(oracle, o_g, vg, 1.25)
    prepare_model(oracle, o_o, vo, 1.25)
    gpu.setSpaceDerivFunc(C.byref(g), C.byref(o_g))
    prev = gpu.qssgpu_set_weno_split(split)
    prev_emu = gpu.qssgpu_set_emu_level(emu)
    prev_var = gpu.qssgpu_set_axis_variant(variant)
    try:
        tg = _model(gpu, vg, o_g, True, 1.25)
    finally:
        gpu.qssgpu_set_weno_split(prev)
        gpu.qssgpu_set_emu_level(prev_emu)
        gpu.qssgpu_set_axis_variant(prev_var)
    to = _model(oracle, vo, o_o, True, 1.25)
    Q.check(gpu)
    assert tg == to
    assert diff_arrays(vg, vo) == {}


def test_tuned_axis_shapes(gpu, oracle):
    """Tuned axis passes: the first step times the candidate launch shapes of
    each axis and keeps the fastest, later steps reuse it; the model still
    equals the oracle, and the table holds each axis once with a valid form
    and a segment length within the line."""
    g, v = pack_case(oracle, 22, seed=6)
    o_g = options(gpu, 40, 5, 3, tmax=0.02, tplot=0.01)
    o_o = options(oracle, 40, 5, 3, tmax=0.02, tplot=0.01)
    vg, vo = clone(v), clone(v)
    prepare_model(oracle, o_g, vg, 1.25)
    prepare_model(oracle, o_o, vo, 1.25)
    gpu.setSpaceDerivFunc(C.byref(g), C.byref(o_g))
    gpu.qssgpu_axis_tuning_reset()
    prev = gpu.qssgpu_set_weno_split(1)
    prev_emu = gpu.qssgpu_set_emu_level(2)
    prev_var = gpu.qssgpu_set_axis_variant(2)
    try:
        tg = _model(gpu, vg, o_g, True, 1.25)
    finally:
        gpu.qssgpu_set_weno_split(prev)
        gpu.qssgpu_set_emu_level(prev_emu)
        gpu.qssgpu_set_axis_variant(prev_var)
    to = _model(oracle, vo, o_o, True, 1.25)
    Q.check(gpu)
    assert tg == to
    assert diff_arrays(vg, vo) == {}
    n = gpu.qssgpu_axis_tuning(None, 0)
    rows = (C.c_int * (7 * max(n, 1)))()
    assert gpu.qssgpu_axis_tuning(rows, n) == n
    r = np.array(rows[:7 * n]).reshape(n, 7)
    assert sorted(r[:, 1].tolist()) == [0, 1, 2]
    assert set(r[:, 0].tolist()) == {2}
    assert set(r[:, 5].tolist()) <= {0, 1, 3, 4}
    seg_max = np.where(r[:, 5] == 3, 16, np.where(r[:, 5] == 4, 27, r[:, 4]))
    assert ((r[:, 6] >= 1) & (r[:, 6] <= seg_max)).all()
    gpu.qssgpu_axis_tuning_reset()
    assert gpu.qssgpu_axis_tuning(None, 0) == 0


@pytest.mark.parametrize("slabs", [2, 5])
def test_const_curv_model_slabs(gpu, oracle, slabs):
    """The reference's dt uses the last voxel of each OpenMP z-slab; with
    T slabs on the GPU the run equals the oracle run with T threads."""
    g, v = pack_case(oracle, 20, seed=9)
    o_g = options(gpu, 40, 5, 3, tmax=0.02, tplot=0.01)
    o_o = options(oracle, 40, 5, 3, tmax=0.02, tplot=0.01)
    vg, vo = clone(v), clone(v)
    prepare_model(oracle, o_g, vg, 1.25)
    prepare_model(oracle, o_o, vo, 1.25)
    gpu.setSpaceDerivFunc(C.byref(g), C.byref(o_g))
    gpu.qssgpu_set_slabs(slabs)
    oracle.oracle_set_threads(slabs)
    try:
        tg = _model(gpu, vg, o_g, True, 1.25)
        to = _model(oracle, vo, o_o, True, 1.25)
    finally:
        gpu.qssgpu_set_slabs(1)
        oracle.oracle_set_threads(1)
    Q.check(gpu)
    assert tg == to
    assert diff_arrays(vg, vo) == {}


def _ladder(lib, v, o, drain=True, imbibe=False):
    def go(d):
        fp = Q.libc_fopen("out")
        try:
            if drain:
                lib.drain_model3d(C.byref(o), C.byref(v.p), C.byref(v.g), fp)
            if imbibe:
                lib.imbibe_model3d(C.byref(o), C.byref(v.p), C.byref(v.g), fp)
        finally:
            Q.libc_fclose(fp)
        files = {}
        for f in sorted(os.listdir(d)):
            if f.startswith("data_step"):
                import gzip

                with gzip.open(os.path.join(d, f), "rb") as fh:
                    files[f] = fh.read()
        return files

    return in_tmpdir(go)


@pytest.mark.parametrize("theta,space,time,imbibe", [(0, 2, 2, False), (10, 5, 3, True), (40, 3, 3, False)])
def test_drain_imbibe_ladder(gpu, oracle, theta, space, time, imbibe):
    g, v = pack_case(oracle, 24, seed=4)
    kw = dict(theta_deg=theta, space=space, time=time, tmax=0.05, tplot=0.02, a=1.2, amin=1.15)
    o_g, o_o = options(gpu, **kw), options(oracle, **kw)
    o_g.amax = o_o.amax = 1.2 + 2.5 * 0.04 * 0.9722
    vg, vo = clone(v), clone(v)
    fg = _ladder(gpu, vg, o_g, True, imbibe)
    fo = _ladder(oracle, vo, o_o, True, imbibe)
    Q.check(gpu)
    assert list(fg) == list(fo) and len(fo) >= 1
    for k in fo:
        assert fg[k] == fo[k], k
    assert diff_arrays(vg, vo) == {}


def test_model_on_page_locked_arrays(gpu, oracle):
    """constCurvModel3d on arrays from qssgpu_host_alloc (page-locked: the
    uploads run asynchronously) equals the oracle on ordinary arrays."""
    g, v = pack_case(oracle, 20, seed=8)
    ptrs = []

    def pinned(shape, dtype):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        ptr = gpu.qssgpu_host_alloc(nbytes)
        assert ptr
        ptrs.append(ptr)
        raw = (C.c_ubyte * nbytes).from_address(ptr)
        return np.frombuffer(raw, dtype=dtype).reshape(shape)

    vg = Q.Volume(g, alloc=pinned)
    assert all(not a.any() for a in vg.arrays.values())  # zeroed
    vg.copy_from(v)
    vo = clone(v)
    o_g = options(gpu, 30, 5, 3, tmax=0.02, tplot=0.01)
    o_o = options(oracle, 30, 5, 3, tmax=0.02, tplot=0.01)
    prepare_model(oracle, o_g, vg, 1.25)
    prepare_model(oracle, o_o, vo, 1.25)
    gpu.setSpaceDerivFunc(C.byref(g), C.byref(o_g))
    try:
        tg = _model(gpu, vg, o_g, True, 1.25)
        to = _model(oracle, vo, o_o, True, 1.25)
        Q.check(gpu)
        assert tg == to
        assert diff_arrays(vg, vo) == {}
    finally:
        gpu.qssgpu_release(C.byref(vg.p))
        del vg
        for p in ptrs:
            gpu.qssgpu_host_free(p)
