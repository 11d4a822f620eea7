"""The C restatement of the Fortran kernels (oracle_kernels3d.c) against a
second, independent restatement in numpy (oracle/oracle_np.py), bit for bit
on random inputs: the ENO2, ENO3 and WENO5 right-hand sides of the
variable-coefficient model (with voxels below the speed tolerance, zero and
negative advection speeds, unequal spacings, z-slabs) and the ENO2/ENO3
constant-coefficient ones, the TVD-RK stages and the signed linear
extrapolation of every face.  No GPU."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import qssgpu as Q

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle_np as N  # noqa: E402

# (the ENO3 x stencil reads phi(i+3,j,j): y extents kept within the z extent)
SHAPES = [(14, 11, 9), (7, 12, 16)]


def _fields(g, seed, small):
    rng = np.random.default_rng(seed)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    z, y, x = np.meshgrid(*(np.arange(s) for s in shape), indexing="ij")
    phi = 0.04 * (np.sqrt((x - 6.3) ** 2 + (y - 7.1) ** 2 + (z - 5.7) ** 2) - 4.0) + 0.003 * rng.standard_normal(shape)
    vel = rng.uniform(-1, 1, shape)
    sel = rng.random(shape) < small
    vel[sel] = rng.uniform(-9e-6, 9e-6, sel.sum())
    vel[rng.random(shape) < 0.5 * small] = 0.0
    b = rng.uniform(0, 0.05, shape)
    vx, vy, vz = (rng.uniform(-1, 1, shape) for _ in range(3))
    for v in (vx, vy, vz):
        v[rng.random(shape) < 0.1] = 0.0
    return phi, vel, b, vx, vy, vz


def _fb(g, klo=None, khi=None):
    return (g.ilo_fb, g.ihi_fb, g.jlo_fb, g.jhi_fb, g.klo_fb if klo is None else klo,
            g.khi_fb if khi is None else khi)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("small", [0.0, 0.3])
@pytest.mark.parametrize("spacing", [(0.04, 0.04, 0.04), (0.04, 0.05, 0.03)])
def test_weno5_rhs(oracle, shape, small, spacing):
    g = Q.make_grid(oracle, shape)
    phi, vel, b, vx, vy, vz = _fields(g, sum(shape) + int(10 * small), small)
    dx, dy, dz = spacing
    for klo, khi in ((None, None), (g.klo_fb + 2, g.klo_fb + 4)):
        rhs = np.full_like(phi, 7.0)
        h = C.c_double(-5.0)
        oracle.getrhs3d5th_(Q.dptr(phi), Q.dptr(vel), Q.dptr(b), Q.dptr(vx), Q.dptr(vy), Q.dptr(vz), C.byref(h),
                            Q.dptr(rhs), *Q.gb_args(g), *Q.fb_args(g, klo, khi), Q.dref(dx), Q.dref(dy),
                            Q.dref(dz))
        fb = _fb(g, klo, khi)
        want, want_h = N.rhs_weno5(phi, vel, b, vx, vy, vz, fb, dx, dy, dz)
        got = N._shift(rhs, fb)
        assert np.array_equal(got, want), f"max |d| = {np.abs(got - want).max()}"
        assert h.value == want_h
        # nothing outside the fill box is written
        outside = np.ones(phi.shape, bool)
        outside[fb[4]:fb[5] + 1, fb[2]:fb[3] + 1, fb[0]:fb[1] + 1] = False
        assert (rhs[outside] == 7.0).all()


@pytest.mark.parametrize("scheme,name", [(2, "getrhs3d2nd_"), (3, "getrhs3d3rd_")])
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("small", [0.0, 0.3])
def test_eno_rhs_variable(oracle, scheme, name, shape, small):
    g = Q.make_grid(oracle, shape)
    phi, vel, b, vx, vy, vz = _fields(g, 3 * sum(shape) + scheme, small)
    dx, dy, dz = 0.04, 0.05, 0.03
    for klo, khi in ((None, None), (g.klo_fb + 1, g.klo_fb + 3)):
        rhs = np.full_like(phi, 7.0)
        h = C.c_double(-5.0)
        getattr(oracle, name)(Q.dptr(phi), Q.dptr(vel), Q.dptr(b), Q.dptr(vx), Q.dptr(vy), Q.dptr(vz), C.byref(h),
                              Q.dptr(rhs), *Q.gb_args(g), *Q.fb_args(g, klo, khi), Q.dref(dx), Q.dref(dy),
                              Q.dref(dz))
        fb = _fb(g, klo, khi)
        want, want_h = N.rhs_var(scheme, phi, vel, b, vx, vy, vz, fb, dx, dy, dz)
        got = N._shift(rhs, fb)
        assert np.array_equal(got, want), f"max |d| = {np.abs(got - want).max()}"
        assert h.value == want_h


@pytest.mark.parametrize("scheme,name", [(2, "getrhs3d2ndconst_"), (3, "getrhs3d3rdconst_")])
@pytest.mark.parametrize("a", [1.3, -0.7, 4e-6])
def test_eno_rhs_constant(oracle, scheme, name, a):
    """Constant speed a (below the 1e-5 tolerance the normal term is never
    set and stays 0) and curvature coefficient."""
    g = Q.make_grid(oracle, SHAPES[0])
    phi = _fields(g, 77, 0.0)[0]
    dx, dy, dz = 0.04, 0.045, 0.035
    rhs = np.full_like(phi, 7.0)
    h = C.c_double(-5.0)
    getattr(oracle, name)(Q.dptr(phi), Q.dref(a), Q.dref(0.04), C.byref(h), Q.dptr(rhs), *Q.gb_args(g),
                          *Q.fb_args(g), Q.dref(dx), Q.dref(dy), Q.dref(dz))
    fb = _fb(g)
    want, want_h = N.rhs_const(scheme, phi, a, 0.04, fb, dx, dy, dz)
    got = N._shift(rhs, fb)
    assert np.array_equal(got, want), f"max |d| = {np.abs(got - want).max()}"
    assert h.value == want_h


def test_rk_stages(oracle):
    g = Q.make_grid(oracle, (9, 8, 7))
    rng = np.random.default_rng(12)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    u0, u1, r = (rng.standard_normal(shape) for _ in range(3))
    dt = 0.0037
    fb = _fb(g)
    cases = (("qss3drk1step_", (u0, r), lambda: N.rk1(u0, r, dt)),
             ("qss3dtvdrk2stage2_", (u1, u0, r), lambda: N.tvdrk2_stage2(u1, u0, r, dt)),
             ("qss3dtvdrk3stage3_", (u1, u0, r), lambda: N.tvdrk3_stage3(u1, u0, r, dt)))
    for name, args, ref in cases:
        out = np.full(shape, 2.5)
        ptrs = []
        for arr in args:
            ptrs += [Q.dptr(arr)] + Q.gb_args(g)
        getattr(oracle, name)(Q.dptr(out), *Q.gb_args(g), *ptrs, *Q.fb_args(g), Q.dref(dt))
        assert np.array_equal(N._shift(out, fb), N._shift(ref(), fb)), name


@pytest.mark.parametrize("face", range(6))
def test_signed_linear_extrapolation(oracle, face):
    g = Q.make_grid(oracle, (9, 8, 7))
    rng = np.random.default_rng(40 + face)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    phi = rng.standard_normal(shape)
    phi[rng.random(shape) < 0.05] = -0.0
    phi[rng.random(shape) < 0.05] = 0.0
    a = phi.copy()
    oracle.signedlinearextrapolation3d_(Q.dptr(a), *Q.gb_args(g), *Q.fb_args(g), C.byref(C.c_int(face)))
    b = N.signed_linear_extrapolation(phi.copy(), _fb(g), face)
    assert np.array_equal(a, b)
    assert np.array_equal(np.signbit(a), np.signbit(b))
