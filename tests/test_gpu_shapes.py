"""Parity on non-cubic grids: fill boxes whose sides differ and are not
multiples of the union-find tile (8) or of the line segments, including a
thin one, through the whole drainage ladder (stage kernels of every axis,
boundary extrapolation, trapping and 26-connected labels, reinitialisation,
loop-order volume sums) and the labelling alone, against the oracle bit for
bit, on one slab and on three."""
import ctypes as C

import numpy as np
import pytest

import qssgpu as Q
import synthetic as S
from qss_cases import clone, diff_arrays, in_tmpdir, options

pytestmark = pytest.mark.gpu

SHAPES = [(21, 17, 26), (33, 12, 10), (9, 14, 19)]


def _pack(lib, n, seed):
    g = Q.make_grid(lib, n)
    v = Q.Volume(g)
    rng = np.random.default_rng(500 + seed)
    for name, arr in v.arrays.items():
        if arr.dtype == np.float64:
            arr[...] = rng.uniform(-2.0, 2.0, arr.shape)
        else:
            arr[...] = rng.integers(0, 2, arr.shape)
    m = S.overlapping(n, radius_vox=3.5, porosity=0.4, seed=seed).mask()
    v["mask"][...] = m
    v["phi"][...] = S.initial_phi(m, n)
    return g, v


def _ladder(lib, v, g, o):
    def go(d):
        import gzip
        import os

        fp = Q.libc_fopen("out")
        try:
            lib.drain_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
        finally:
            Q.libc_fclose(fp)
        files = {}
        for f in sorted(os.listdir(d)):
            if f.startswith("data_step"):
                with gzip.open(os.path.join(d, f), "rb") as fh:
                    files[f] = fh.read()
        return files

    return in_tmpdir(go)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("theta,space,time,slabs", [(30, 5, 3, 1), (0, 2, 2, 3), (10, 5, 3, 3)])
def test_ladder_non_cubic(gpu, oracle, shape, theta, space, time, slabs):
    g, v = _pack(oracle, shape, seed=sum(shape) + theta)
    kw = dict(theta_deg=theta, space=space, time=time, tmax=0.04, tplot=0.02, a=1.2, amin=1.15)
    o_g, o_o = options(gpu, **kw), options(oracle, **kw)
    o_g.amax = o_o.amax = 1.2 + 1.5 * 0.04 * 0.9722
    vg, vo = clone(v), clone(v)
    gpu.qssgpu_set_slabs(slabs)
    oracle.oracle_set_threads(slabs)
    try:
        fg = _ladder(gpu, vg, g, o_g)
        fo = _ladder(oracle, vo, g, o_o)
    finally:
        gpu.qssgpu_set_slabs(1)
        oracle.oracle_set_threads(1)
    Q.check(gpu)
    assert list(fg) == list(fo)
    for k in fo:
        assert fg[k] == fo[k], k
    assert diff_arrays(vg, vo) == {}


@pytest.mark.parametrize("shape", SHAPES)
def test_labels_non_cubic(gpu, oracle, shape):
    g, v = _pack(oracle, shape, seed=7)
    rng = np.random.default_rng(sum(shape))
    for density in (0.3, 0.6):
        v["phi_bin"][...] = (rng.random(v.shape) < density).astype(np.uint8)
        a, b = clone(v), clone(v)
        gpu.findConnectivity3d(C.byref(a.p), C.byref(g))
        oracle.findConnectivity3d(C.byref(b.p), C.byref(g))
        Q.check(gpu)
        assert np.array_equal(a["connectivity"], b["connectivity"])
