"""Input builders shared by the parity tests (seeded synthetic packs on the
reference grid layout) and helpers to run one call on several libraries."""
import ctypes as C
import os
import tempfile

import numpy as np

import qssgpu as Q
import synthetic as S


def pack_case(lib, n, seed=0, radius=4.0, porosity=0.4):
    """Grid + Volume holding a sphere-pack mask and the initial level set."""
    g = Q.make_grid(lib, n)
    v = Q.Volume(g)
    # every array starts with caller data, so a value written where the
    # reference leaves the caller's data untouched shows up as a difference
    rng = np.random.default_rng(1000 + seed)
    for name, arr in v.arrays.items():
        if arr.dtype == np.float64:
            arr[...] = rng.uniform(-2.0, 2.0, arr.shape)
        else:
            arr[...] = rng.integers(0, 2, arr.shape)
    m = S.overlapping(n, radius_vox=radius, porosity=porosity, seed=seed).mask()
    v["mask"][...] = m
    v["phi"][...] = S.initial_phi(m, n)
    return g, v


def clone(v):
    w = Q.Volume(v.g)
    w.copy_from(v)
    return w


def options(lib, theta_deg=0.0, space=2, time=2, tmax=0.05, tplot=0.02, a=1.25, b=0.04, dc=0.9722,
            amax=None, amin=0.5, check_connectivity=1):
    o = Q.default_options(lib)
    o.theta = theta_deg * 3.14159 / 180
    o.order_space_accur, o.order_time_accur = space, time
    o.tmax, o.tplot, o.a, o.b, o.dc = tmax, tplot, a, b, dc
    o.amax = a + 1.5 * b * dc if amax is None else amax
    o.amin = amin
    o.check_connectivity = check_connectivity
    return o


def in_tmpdir(fn):
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            return fn(d)
        finally:
            os.chdir(cwd)


def prepare_model(lib, o, v, a0):
    """The set-up drain_model3d performs before calling constCurvModel3d:
    masks, mask gradient, scheme, overlap, coefficients, inlet/outlet points."""
    g = v.g
    gp = C.byref(g)
    lib.initializeDisconnectedMasks(v["mask_w"].ctypes.data_as(Q.c_double_p), gp)
    lib.initializeDisconnectedMasks(v["mask_nw"].ctypes.data_as(Q.c_double_p), gp)
    lib.getcentralgrad3dorder2_(Q.dptr(v["mask_x"]), Q.dptr(v["mask_y"]), Q.dptr(v["mask_z"]), *Q.gb_args(g),
                                Q.dptr(v["mask"]), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]),
                                Q.dref(g.dx[1]), Q.dref(g.dx[2]))
    lib.setSpaceDerivFunc(gp, C.byref(o))
    lib.setThetaOverlap(C.byref(v.p), gp, C.byref(o))
    lib.getMainInd_new(C.byref(o), C.byref(v.p), gp)
    if o.theta > 0:
        bm, um = C.c_double(0), C.c_double(0)
        lib.setvarcurvadv3d_(Q.dptr(v["mask"]), Q.dptr(v["mask_x"]), Q.dptr(v["mask_y"]), Q.dptr(v["mask_z"]),
                             Q.dptr(v["curvature_coeff"]), Q.dptr(v["external_velocity_x"]),
                             Q.dptr(v["external_velocity_y"]), Q.dptr(v["external_velocity_z"]), C.byref(bm),
                             C.byref(um), Q.dref(o.b), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
        o.b_max_over_dx, o.max_U_over_dx = bm.value, um.value
        lib.setvarnorm3d_(Q.dptr(v["mask"]), Q.dptr(v["mask_x"]), Q.dptr(v["mask_y"]), Q.dptr(v["mask_z"]),
                          Q.dptr(v["normal_velocity"]), Q.dref(a0), Q.dref(o.theta), *Q.gb_args(g),
                          *Q.fb_args(g), Q.dref(g.dx[0]))
    else:
        inv = 1.0 / g.dx[0]
        o.b_max_over_dx = 2 * o.b * (inv * inv + inv * inv + inv * inv)
        o.max_U_over_dx = 0.0


def diff_arrays(va, vb, skip=("theta", "overlap")):
    """Names of arrays that differ bit-wise, with the max abs difference."""
    out = {}
    for k in va.arrays:
        if k in skip:
            continue
        a, b = va[k], vb[k]
        if not np.array_equal(a, b):
            d = np.abs(a.astype(np.float64) - b.astype(np.float64))
            out[k] = float(np.nanmax(d))
    return out
