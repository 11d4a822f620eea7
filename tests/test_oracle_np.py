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


def _trig(oracle):
    """the oracle's portable sine and cosine, elementwise (the restatements
    are compared with the same sine, so the comparison is of the Fortran
    arithmetic around it)"""
    out = []
    for name in ("oracle_portable_sin", "oracle_portable_cos"):
        f = getattr(oracle, name)
        f.restype = C.c_double
        f.argtypes = [C.c_double]
        out.append(np.vectorize(f, otypes=[float]))
    return out


def _ghost(g):
    return (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])


def _mask_fields(g, seed, dx):
    """a mask straddling +-1.5 dx (the Heaviside band) with exact band edges,
    zeros and its central gradient"""
    rng = np.random.default_rng(seed)
    shape = _ghost(g)
    mask = rng.uniform(-3 * dx, 3 * dx, shape)
    for v in (0.0, -0.0, 1.5 * dx, -1.5 * dx):
        mask[rng.random(shape) < 0.04] = v
    mx, my, mz = (rng.uniform(-1.2, 1.2, shape) for _ in range(3))
    mx[rng.random(shape) < 0.05] = 0.0
    return mask, mx, my, mz


@pytest.mark.parametrize("theta_field", [False, True])
def test_set_var_norm(oracle, theta_field):
    sin, cos = _trig(oracle)
    g = Q.make_grid(oracle, (9, 8, 7))
    dx = g.dx[0]
    mask, mx, my, mz = _mask_fields(g, 5 + theta_field, dx)
    out = np.full(_ghost(g), 3.0)
    a0 = 1.15
    fb = _fb(g)
    if theta_field:
        ca = np.random.default_rng(8).uniform(0, 1.2, _ghost(g))
        oracle.setvarnorm3dtheta_(Q.dptr(mask), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(out), Q.dref(a0),
                                  Q.dptr(ca), *Q.gb_args(g), *Q.fb_args(g), Q.dref(dx))
    else:
        ca = 0.61
        oracle.setvarnorm3d_(Q.dptr(mask), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(out), Q.dref(a0),
                             Q.dref(ca), *Q.gb_args(g), *Q.fb_args(g), Q.dref(dx))
    want = N.set_var_norm(mask, mx, my, mz, a0, ca, fb, dx, sin, cos)
    assert np.array_equal(N._shift(out, fb), want)


def test_set_var_curv_adv(oracle):
    sin, _ = _trig(oracle)
    g = Q.make_grid(oracle, (9, 8, 7))
    dx = g.dx[0]
    mask, mx, my, mz = _mask_fields(g, 21, dx)
    b, vx, vy, vz = (np.full(_ghost(g), 3.0) for _ in range(4))
    bm, um = C.c_double(), C.c_double()
    oracle.setvarcurvadv3d_(Q.dptr(mask), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(b), Q.dptr(vx), Q.dptr(vy),
                            Q.dptr(vz), C.byref(bm), C.byref(um), Q.dref(0.04), *Q.gb_args(g), *Q.fb_args(g),
                            Q.dref(dx))
    fb = _fb(g)
    wb, wx, wy, wz, wbm, wum = N.set_var_curv_adv(mask, mx, my, mz, 0.04, fb, dx, sin)
    for got, want in ((b, wb), (vx, wx), (vy, wy), (vz, wz)):
        assert np.array_equal(N._shift(got, fb), want)
    assert (bm.value, um.value) == (wbm, wum)


def test_central_grad_trap_velocity_mask_and_norm(oracle):
    g = Q.make_grid(oracle, (9, 8, 7))
    rng = np.random.default_rng(31)
    shape = _ghost(g)
    fb = _fb(g)
    phi = rng.standard_normal(shape)
    gx, gy, gz = (np.full(shape, 3.0) for _ in range(3))
    oracle.getcentralgrad3dorder2_(Q.dptr(gx), Q.dptr(gy), Q.dptr(gz), *Q.gb_args(g), Q.dptr(phi), *Q.gb_args(g),
                                   *Q.fb_args(g), Q.dref(0.04), Q.dref(0.05), Q.dref(0.03))
    for got, want in zip((gx, gy, gz), N.central_grad(phi, fb, 0.04, 0.05, 0.03)):
        assert np.array_equal(N._shift(got, fb), want)

    dx = g.dx[0]
    mask_w = rng.uniform(0, 3 * dx, shape)
    mask_w[rng.random(shape) < 0.1] = 1.5 * dx  # the threshold itself keeps the values
    fields = [rng.standard_normal(shape) for _ in range(5)]
    mine = [f.copy() for f in fields]
    oracle.imposetrapvelocity3d_(Q.dptr(mask_w), Q.dptr(mask_w), *[Q.dptr(f) for f in fields], *Q.gb_args(g),
                                 *Q.fb_args(g), Q.dref(dx))
    N.impose_trap_velocity(mask_w, mine, fb, dx)
    for a, b in zip(fields, mine):
        assert np.array_equal(a, b)

    mask = rng.standard_normal(shape)
    for overlap in (0.013, rng.uniform(0, 0.05, shape)):
        out = np.full(shape, 3.0)
        klo, khi = 2, shape[0] - 3
        args = Q.dref(overlap) if np.ndim(overlap) == 0 else Q.dptr(overlap)
        fn = oracle.imposemaskparallel_ if np.ndim(overlap) == 0 else oracle.imposemaskparallelvar_
        fn(Q.dptr(out), Q.dptr(mask), Q.dptr(phi), args, *Q.gb_args(g), C.byref(C.c_int(klo)), C.byref(C.c_int(khi)))
        assert np.array_equal(out[klo:khi + 1], N.impose_mask(mask, phi, overlap, klo, khi))
        assert (out[:klo] == 3.0).all() and (out[khi + 1:] == 3.0).all()

    f2 = phi + rng.uniform(-0.1, 0.1, shape)
    ib = (4, 9, 3, 8, 4, 7)
    for zone in (0.5, 1e-9):
        r = C.c_double()
        oracle.qss3dmaxnormdifflocal_(C.byref(r), Q.dptr(phi), *Q.gb_args(g), Q.dptr(f2), *Q.gb_args(g),
                                      *[C.byref(C.c_int(v)) for v in ib], Q.dref(zone))
        assert r.value == N.max_norm_diff_local(phi, f2, ib, zone)


def test_volume_phi_less_than_zero(oracle):
    sin, _ = _trig(oracle)
    g = Q.make_grid(oracle, (11, 9, 8))
    rng = np.random.default_rng(17)
    eps = 1.5 * g.dx[0]
    phi = rng.uniform(-3 * eps, 3 * eps, _ghost(g))
    for v in (eps, -eps, 0.0):
        phi[rng.random(phi.shape) < 0.05] = v
    ib = _fb(g)
    r = C.c_double()
    oracle.qss3dvolumeregionphilessthanzero_(C.byref(r), Q.dptr(phi), *Q.gb_args(g),
                                             *[C.byref(C.c_int(v)) for v in ib], Q.dref(0.04), Q.dref(0.05),
                                             Q.dref(0.03), Q.dref(eps))
    assert r.value == N.volume_phi_less_than_zero(phi, ib, 0.04, 0.05, 0.03, eps, sin)
    # a one-voxel box returns that voxel's contribution exactly (0 + c), which
    # a sum over many voxels would round away
    for k in range(g.klo_fb, g.klo_fb + 3):
        for j in range(g.jlo_fb, g.jhi_fb + 1):
            for i in range(g.ilo_fb, g.ihi_fb + 1):
                one = (i, i, j, j, k, k)
                oracle.qss3dvolumeregionphilessthanzero_(C.byref(r), Q.dptr(phi), *Q.gb_args(g),
                                                         *[C.byref(C.c_int(v)) for v in one], Q.dref(0.04),
                                                         Q.dref(0.05), Q.dref(0.03), Q.dref(eps))
                assert r.value == N.volume_phi_less_than_zero(phi, one, 0.04, 0.05, 0.03, eps, sin), (i, j, k)


@pytest.mark.parametrize("spacing", [(0.04, 0.04, 0.04), (0.04, 0.05, 0.03)])
def test_reinitialisation_kernels(oracle, spacing):
    g = Q.make_grid(oracle, (10, 9, 8))
    rng = np.random.default_rng(23)
    shape = _ghost(g)
    dx, dy, dz = spacing
    z, y, x = np.meshgrid(*(np.arange(s) for s in shape), indexing="ij")
    phi0 = 0.04 * (np.sqrt((x - 6.2) ** 2 + (y - 5.9) ** 2 + (z - 5.1) ** 2) - 3.3)
    phi0 += 0.01 * rng.standard_normal(shape)
    for v in (0.0, -0.0, 5e-6, -5e-6):
        phi0[rng.random(shape) < 0.03] = v
    fb = _fb(g)
    dist = np.full(shape, 3.0)
    oracle.qss3dcomputedistanceforsubcellfix_(Q.dptr(dist), Q.dptr(phi0), *Q.gb_args(g), *Q.fb_args(g),
                                              Q.dref(dx), Q.dref(dy), Q.dref(dz))
    want = N.distance_for_subcell_fix(phi0, fb, dx, dy, dz)
    assert np.array_equal(N._shift(dist, fb), want)
    assert (want == -1000.0 * max(spacing)).any() and (want != -1000.0 * max(spacing)).any()

    phi = phi0 + 0.02 * rng.standard_normal(shape)
    phi[rng.random(shape) < 0.03] = 0.0
    rhs = np.full(shape, 3.0)
    oracle.qss3dcomputereinitializationeqnrhssubcellfixorder1_(Q.dptr(rhs), Q.dptr(phi), *Q.gb_args(g),
                                                               Q.dptr(phi0), Q.dptr(dist), *Q.fb_args(g),
                                                               Q.dref(dx), Q.dref(dy), Q.dref(dz))
    assert np.array_equal(N._shift(rhs, fb), N.reinit_rhs_subcell_fix(phi, phi0, dist, fb, dx, dy, dz))
