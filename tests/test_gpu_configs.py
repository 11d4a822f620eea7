"""Parity at the workloads' own sizes.

* 64^3 plain drainage (overlapping pack, seed 0, radius 5, porosity 0.35;
  ENO2 + TVD-RK2, contact angle 0; curvature ladder 0.05 -> 0.4 per voxel in
  10 steps; a reinitialisation after every 5 nominal time steps): the whole
  ladder against the oracle, every saved ``data_step`` file and every array
  bit for bit.
* 256^3 drainage then imbibition (non-overlapping polydisperse pack, seed 1,
  radii 4-12, porosity 0.38; WENO5 + TVD-RK3, contact angle 10 degrees): the
  first two drainage steps of the 40-step ladder 0.02 -> 0.5 per voxel and one
  imbibition step, with the oracle on T OpenMP threads and the GB300 path on
  the same T z-slabs (the CFL step depends on the slab split), bit for bit.
* 512^3 grain pack (lognormal radii, porosity 0.30, contact angle 40
  degrees): the coefficient kernels, the WENO5 right-hand side over T
  z-slabs and the 26-connected labels of the pore space at full size.  The
  oracle runs the slabs on T host threads; the labels are checked against an
  independent rule (scipy components named by their largest linear index)."""
import ctypes as C
import gzip
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import qssgpu as Q
import synthetic as S
from qss_cases import clone, diff_arrays, in_tmpdir, options

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def _ladder(lib, v, g, o, imbibe_from=None, imbibe_min=None):
    """drain_model3d (and optionally imbibe_model3d) in a scratch directory;
    returns the saved data_step files, decompressed."""

    def go(d):
        fp = Q.libc_fopen("out")
        try:
            lib.drain_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
            for f in os.listdir(d):
                if f.startswith("data_step"):  # imbibition numbers its steps from 1 again
                    os.rename(os.path.join(d, f), os.path.join(d, "drain_" + f))
            if imbibe_from is not None:
                o.a, o.amin = imbibe_from, imbibe_min
                lib.imbibe_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
        finally:
            Q.libc_fclose(fp)
        files = {}
        for f in sorted(os.listdir(d)):
            if "data_step" in f:
                with gzip.open(os.path.join(d, f), "rb") as fh:
                    files[f] = fh.read()
        return files

    return in_tmpdir(go)


def _fresh_volume(g, mask, n):
    v = Q.Volume(g)
    v["mask"][...] = mask
    v["phi"][...] = S.initial_phi(mask, n)
    return v


def test_drainage_64_full_ladder(gpu, oracle):
    n = 64
    g = Q.make_grid(oracle, n)
    mask = S.overlapping(n, radius_vox=5.0, porosity=0.35, seed=0).mask()
    da = 0.97222  # 0.03889 per voxel at dx = 0.04
    kw = dict(theta_deg=0.0, space=2, time=2, tmax=0.1, tplot=0.0167, a=1.25, b=0.04, dc=da / 0.04)
    o_g, o_o = options(gpu, **kw), options(oracle, **kw)
    o_g.amax = o_o.amax = 10.0 + 0.5 * da
    vg, vo = _fresh_volume(g, mask, n), _fresh_volume(g, mask, n)
    fg = _ladder(gpu, vg, g, o_g)
    fo = _ladder(oracle, vo, g, o_o)
    Q.check(gpu)
    assert list(fg) == list(fo) and len(fo) >= 9
    for k in fo:
        assert fg[k] == fo[k], k
    assert diff_arrays(vg, vo) == {}


def test_drain_imbibe_256_first_steps(gpu, oracle):
    n = 256
    g = Q.make_grid(oracle, n)
    mask = S.rsa(n, rmin=4.0, rmax=12.0, porosity=0.38, seed=1).mask()
    da = (12.5 - 0.5) / 39  # 0.02 -> 0.5 per voxel in 40 steps at dx = 0.04
    kw = dict(theta_deg=10.0, space=5, time=3, tmax=0.01, tplot=0.005, a=0.5, b=0.04, dc=da / 0.04)
    o_g, o_o = options(gpu, **kw), options(oracle, **kw)
    o_g.amax = o_o.amax = 0.5 + 1.5 * da
    vg = _fresh_volume(g, mask, n)
    vo = clone(vg)
    gpu.qssgpu_set_slabs(THREADS)
    oracle.oracle_set_threads(THREADS)
    try:
        fg = _ladder(gpu, vg, g, o_g, imbibe_from=0.5, imbibe_min=0.5 - 0.5 * da)
        fo = _ladder(oracle, vo, g, o_o, imbibe_from=0.5, imbibe_min=0.5 - 0.5 * da)
    finally:
        gpu.qssgpu_set_slabs(1)
        oracle.oracle_set_threads(1)
    Q.check(gpu)
    assert list(fg) == list(fo) and len(fo) >= 2, list(fo)
    for k in fo:
        assert fg[k] == fo[k], k
    assert diff_arrays(vg, vo) == {}
    # the ladder moved the front
    assert not np.array_equal(vg["phi"], S.initial_phi(mask, n))


@pytest.fixture(scope="module")
def pack512(oracle):
    n = 512
    g = Q.make_grid(oracle, n)
    mask = S.lognormal(n, porosity=0.30).mask()
    return n, g, mask


def _slabs(g):
    ks = np.array_split(np.arange(g.klo_fb, g.khi_fb + 1), THREADS)
    return [(int(k[0]), int(k[-1])) for k in ks if len(k)]


def _coefficients(lib, g, mask, theta, a0, b):
    gx, gy, gz = (np.zeros_like(mask) for _ in range(3))
    lib.getcentralgrad3dorder2_(Q.dptr(gx), Q.dptr(gy), Q.dptr(gz), *Q.gb_args(g), Q.dptr(mask), *Q.gb_args(g),
                                *Q.fb_args(g), Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]))
    curv, vx, vy, vz, vel = (np.zeros_like(mask) for _ in range(5))
    bm, um = C.c_double(0), C.c_double(0)
    lib.setvarcurvadv3d_(Q.dptr(mask), Q.dptr(gx), Q.dptr(gy), Q.dptr(gz), Q.dptr(curv), Q.dptr(vx), Q.dptr(vy),
                         Q.dptr(vz), C.byref(bm), C.byref(um), Q.dref(b), *Q.gb_args(g), *Q.fb_args(g),
                         Q.dref(g.dx[0]))
    lib.setvarnorm3d_(Q.dptr(mask), Q.dptr(gx), Q.dptr(gy), Q.dptr(gz), Q.dptr(vel), Q.dref(a0), Q.dref(theta),
                      *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
    return dict(mask_x=gx, mask_y=gy, mask_z=gz, curvature_coeff=curv, vx=vx, vy=vy, vz=vz, normal_velocity=vel,
                b_max_over_dx=bm.value, max_U_over_dx=um.value)


def _rhs_slabs(lib, g, phi, c, parallel):
    rhs = np.full_like(phi, 7.0)
    d = [Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2])]

    def one(kr):
        h = C.c_double(-5.0)
        lib.getrhs3d5th_(Q.dptr(phi), Q.dptr(c["normal_velocity"]), Q.dptr(c["curvature_coeff"]), Q.dptr(c["vx"]),
                         Q.dptr(c["vy"]), Q.dptr(c["vz"]), C.byref(h), Q.dptr(rhs), *Q.gb_args(g),
                         *Q.fb_args(g, kr[0], kr[1]), *d)
        return h.value

    if parallel:
        with ThreadPoolExecutor(THREADS) as ex:
            hs = list(ex.map(one, _slabs(g)))
    else:
        hs = [one(kr) for kr in _slabs(g)]
    return rhs, hs


def test_coefficients_and_weno5_rhs_512(gpu, oracle, pack512):
    n, g, mask = pack512
    theta, a0, b = 40.0 * 3.14159 / 180, 1.25, 0.04
    cg = _coefficients(gpu, g, mask, theta, a0, b)
    Q.check(gpu)
    co = _coefficients(oracle, g, mask, theta, a0, b)
    for k in cg:
        assert np.array_equal(cg[k], co[k]), k
    del co
    phi = S.initial_phi(mask, n)
    rg, hg = _rhs_slabs(gpu, g, phi, cg, parallel=False)
    Q.check(gpu)
    ro, ho = _rhs_slabs(oracle, g, phi, cg, parallel=True)
    assert hg == ho
    assert np.array_equal(rg, ro), f"max |d| = {np.abs(rg - ro).max()}"
    assert np.isfinite(rg).all() and hg[0] > 0


def test_labels_512(gpu, pack512):
    from scipy import ndimage

    n, g, mask = pack512
    v = Q.Volume(g)
    v["phi_bin"][...] = (mask < 0).astype(np.uint8)
    gpu.findConnectivity3d(C.byref(v.p), C.byref(g))
    Q.check(gpu)
    lab, count = ndimage.label(v["phi_bin"].astype(bool), structure=np.ones((3, 3, 3)))
    flat = np.arange(lab.size, dtype=np.int64).reshape(lab.shape)
    top = ndimage.maximum(flat, lab, index=np.arange(1, count + 1)).astype(np.int64)
    want = np.concatenate([[0], top]).astype(np.int32)[lab]
    assert count > 1
    assert np.array_equal(v["connectivity"], want)
