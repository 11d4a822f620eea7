"""Pins the oracle's restated C drivers to the reference's own C drivers
(src/level_set_evolution, src/connectivity, src/reinitialization,
src/utilities compiled unchanged from the reference tree into oracle/_ref and
linked against the same restated kernels).  Only where that build exists."""
import ctypes as C

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


@pytest.mark.parametrize("theta,space,time,threads", [
    (0, 2, 2, 1), (0, 3, 3, 2), (0, 5, 1, 3), (10, 2, 2, 1), (30, 5, 3, 4), (40, 3, 3, 1), (60, 5, 3, 2)])
def test_drain_imbibe_drivers(ref, oracle, theta, space, time, threads):
    g, v = pack_case(oracle, 20, seed=theta + space)

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
