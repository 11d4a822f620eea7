"""Per-kernel parity: each GB300 kernel, called through its Fortran-convention
C entry point, against the oracle's restatement of the same reference
routine.  Integer, index and floating-point outputs are compared bit for bit
(the kernels reproduce the reference's FP64 operation order; tolerance 0)."""
import ctypes as C

import numpy as np
import pytest

import qssgpu as Q
from qss_cases import pack_case

pytestmark = pytest.mark.gpu

N = 20


def _fields(g, seed, small_vel_fraction=0.0):
    rng = np.random.default_rng(seed)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    z, y, x = np.meshgrid(*(np.arange(s) for s in shape), indexing="ij")
    phi = 0.04 * (np.sqrt((x - 9.3) ** 2 + (y - 11.1) ** 2 + (z - 8.7) ** 2) - 6.0) + 0.002 * rng.standard_normal(shape)
    vel = rng.uniform(-1, 1, shape)
    if small_vel_fraction:
        sel = rng.random(shape) < small_vel_fraction
        vel[sel] = rng.uniform(-9e-6, 9e-6, sel.sum())
        vel[:, :, :] = np.where(rng.random(shape) < 0.5 * small_vel_fraction, 0.0, vel)
    b = rng.uniform(0, 0.05, shape)
    vx, vy, vz = (rng.uniform(-1, 1, shape) for _ in range(3))
    return phi, vel, b, vx, vy, vz


def _run_rhs(lib, name, var, g, phi, vel, b, vx, vy, vz, klo=None, khi=None, a=1.3, bconst=0.04):
    rhs = np.full_like(phi, 7.0)
    h = C.c_double(-5.0)
    fn = getattr(lib, name)
    d = [Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2])]
    if var:
        fn(Q.dptr(phi), Q.dptr(vel), Q.dptr(b), Q.dptr(vx), Q.dptr(vy), Q.dptr(vz), C.byref(h), Q.dptr(rhs),
           *Q.gb_args(g), *Q.fb_args(g, klo, khi), *d)
    else:
        fn(Q.dptr(phi), Q.dref(a), Q.dref(bconst), C.byref(h), Q.dptr(rhs), *Q.gb_args(g), *Q.fb_args(g, klo, khi), *d)
    return rhs, h.value


RHS = [("getrhs3d2ndconst_", False), ("getrhs3d3rdconst_", False), ("getrhs3d2nd_", True),
       ("getrhs3d3rd_", True), ("getrhs3d5th_", True)]


@pytest.mark.parametrize("name,var", RHS)
@pytest.mark.parametrize("small", [0.0, 0.05])
def test_rhs_bit_exact(gpu, oracle, name, var, small):
    g, _ = pack_case(oracle, N)
    phi, vel, b, vx, vy, vz = _fields(g, 1, small)
    a = _run_rhs(gpu, name, var, g, phi, vel, b, vx, vy, vz)
    o = _run_rhs(oracle, name, var, g, phi, vel, b, vx, vy, vz)
    Q.check(gpu)
    assert np.array_equal(a[0], o[0]), f"max |d| = {np.abs(a[0] - o[0]).max()}"
    assert a[1] == o[1]


@pytest.mark.parametrize("name,var", RHS)
def test_rhs_slab_and_tiny_speed(gpu, oracle, name, var):
    """A z-slab call (one OpenMP thread's box) restarts the carried normal
    term; a constant speed below 1e-5 leaves only the curvature term."""
    g, _ = pack_case(oracle, N)
    phi, vel, b, vx, vy, vz = _fields(g, 2, 0.2)
    for klo, khi in ((g.klo_fb + 5, g.klo_fb + 11), (g.khi_fb, g.khi_fb)):
        a = _run_rhs(gpu, name, var, g, phi, vel, b, vx, vy, vz, klo, khi, a=3e-6)
        o = _run_rhs(oracle, name, var, g, phi, vel, b, vx, vy, vz, klo, khi, a=3e-6)
        Q.check(gpu)
        assert np.array_equal(a[0], o[0])
        assert a[1] == o[1]


@pytest.mark.parametrize("emu", [0, 2])
def test_weno5_rhs_zero_curvature_coefficient(gpu, oracle, emu):
    """Where the curvature coefficient is +0 the combine kernel skips the
    curvature, except where the normal term is -0 (here: a flat patch of the
    level set under a negative speed), where b * kappa could decide the sign
    of a zero: the right-hand side must equal the oracle's bit for bit, signs
    of zeros included."""
    g, _ = pack_case(oracle, N)
    phi, vel, b, vx, vy, vz = _fields(g, 11)
    nz, ny, nx = phi.shape
    b[:, :, : nx // 2] = 0.0  # half the box without curvature
    phi[4:14, 4:14, 3:12] = 0.37  # a flat patch: zero one-sided derivatives inside it
    vel[4:14, 4:14, 3:12] = -0.5  # ... and a negative speed: temp_norm = -0
    vx[4:14, 4:14, 3:12] = 0.0
    vy[4:14, 4:14, 3:12] = 0.0
    vz[4:14, 4:14, 3:12] = 0.0
    prev_emu = gpu.qssgpu_set_emu_level(emu)
    try:
        a = _run_rhs(gpu, "getrhs3d5th_", True, g, phi, vel, b, vx, vy, vz)
    finally:
        gpu.qssgpu_set_emu_level(prev_emu)
    o = _run_rhs(oracle, "getrhs3d5th_", True, g, phi, vel, b, vx, vy, vz)
    Q.check(gpu)
    assert np.array_equal(a[0].view(np.int64), o[0].view(np.int64))
    assert a[1] == o[1]
    # the flat patch gives exact zeros (normal, advection and curvature terms all zero)
    assert (o[0][7:11, 7:11, 6:9] == 0.0).all()


@pytest.mark.parametrize("split,emu,variant", [(0, 2, -1), (1, 0, -1), (1, 1, 0), (1, 1, 1), (1, 2, 0),
                                               (1, 2, 1), (1, 1, 2), (1, 2, 2), (1, 1, 3), (1, 2, 3), (1, 2, 4)])
@pytest.mark.parametrize("small", [0.0, 0.2])
def test_weno5_split_and_fused(gpu, oracle, split, emu, variant, small):
    """The WENO5 stage runs as one fused kernel (split 0) or as one kernel per
    axis with shared sub-expressions + a combine kernel (split 1), with 0, 1
    or 2 levels of FP64 arithmetic on the integer pipes and the axis passes'
    window in registers (variant 0), partly in shared memory (1), the
    launch shape tuned by timing (2) or tiles of one voxel per thread with
    faces and centres in shared memory (3); all equal the oracle bit for bit,
    on the whole fill box and on a z-slab."""
    g, _ = pack_case(oracle, N)
    phi, vel, b, vx, vy, vz = _fields(g, 5, small)
    prev = gpu.qssgpu_set_weno_split(split)
    prev_emu = gpu.qssgpu_set_emu_level(emu)
    prev_var = gpu.qssgpu_set_axis_variant(variant)
    try:
        for klo, khi in ((None, None), (g.klo_fb + 3, g.klo_fb + 9)):
            a = _run_rhs(gpu, "getrhs3d5th_", True, g, phi, vel, b, vx, vy, vz, klo, khi)
            o = _run_rhs(oracle, "getrhs3d5th_", True, g, phi, vel, b, vx, vy, vz, klo, khi)
            Q.check(gpu)
            assert np.array_equal(a[0], o[0]), f"max |d| = {np.abs(a[0] - o[0]).max()}"
            assert a[1] == o[1]
    finally:
        gpu.qssgpu_set_weno_split(prev)
        gpu.qssgpu_set_emu_level(prev_emu)
        gpu.qssgpu_set_axis_variant(prev_var)


def test_emu_selftest(gpu):
    """Integer-pipe FP64 division, square root, product, sum, difference,
    power-of-two scaling, comparisons and maxima equal the native instructions on 2^24
    generated operand pairs (all classes of doubles)."""
    counts = (C.c_longlong * 9)()
    first = (C.c_double * 3)()
    assert gpu.qssgpu_emu_selftest(1 << 24, 20261203, counts, first) == 0
    Q.check(gpu)
    assert counts[8] == 1 << 24
    assert list(counts[:8]) == [0] * 8, f"mismatch: op {first[0]} x={first[1]!r} y={first[2]!r}"


def test_rk_stages(gpu, oracle):
    g, _ = pack_case(oracle, N)
    rng = np.random.default_rng(3)
    shape = (g.grid_dims_ghostbox[2], g.grid_dims_ghostbox[1], g.grid_dims_ghostbox[0])
    u0, u1, r = (rng.standard_normal(shape) for _ in range(3))
    dt = 0.0033
    for name, args in (("qss3drk1step_", (u0, r)), ("qss3dtvdrk2stage2_", (u1, u0, r)),
                       ("qss3dtvdrk3stage3_", (u1, u0, r))):
        outs = []
        for lib in (gpu, oracle):
            out = np.full(shape, 2.5)
            ptrs = []
            for arr in args:
                ptrs += [Q.dptr(arr)] + Q.gb_args(g)
            getattr(lib, name)(Q.dptr(out), *Q.gb_args(g), *ptrs, *Q.fb_args(g), Q.dref(dt))
            outs.append(out)
        Q.check(gpu)
        assert np.array_equal(outs[0], outs[1]), name


@pytest.mark.parametrize("face", range(6))
def test_bc_face(gpu, oracle, face):
    g, v = pack_case(oracle, N)
    rng = np.random.default_rng(face)
    phi = v["phi"] + 0.01 * rng.standard_normal(v.shape)
    phi[v.shape[0] // 2, 3, 3] = -0.0
    outs = []
    for lib in (gpu, oracle):
        a = phi.copy()
        lib.signedlinearextrapolation3d_(Q.dptr(a), *Q.gb_args(g), *Q.fb_args(g), C.byref(C.c_int(face)))
        outs.append(a)
    Q.check(gpu)
    assert np.array_equal(outs[0], outs[1])


def test_bc_all_faces_c_api(gpu, oracle):
    g, v = pack_case(oracle, N)
    outs = []
    for lib in (gpu, oracle):
        a = v["phi"] + 0.003
        lib.signedLinearExtrapolationBCqss(Q.dptr(a), C.byref(g), 9)
        outs.append(a)
    Q.check(gpu)
    assert np.array_equal(outs[0], outs[1])


def test_coefficients(gpu, oracle):
    g, v = pack_case(oracle, N, seed=4)
    res = []
    for lib in (gpu, oracle):
        mx, my, mz = (np.zeros(v.shape) for _ in range(3))
        lib.getcentralgrad3dorder2_(Q.dptr(mx), Q.dptr(my), Q.dptr(mz), *Q.gb_args(g), Q.dptr(v["mask"]),
                                    *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]))
        vb, vx, vy, vz, vn, vt = (np.zeros(v.shape) for _ in range(6))
        bm, um = C.c_double(0), C.c_double(0)
        lib.setvarcurvadv3d_(Q.dptr(v["mask"]), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(vb), Q.dptr(vx),
                             Q.dptr(vy), Q.dptr(vz), C.byref(bm), C.byref(um), Q.dref(0.04), *Q.gb_args(g),
                             *Q.fb_args(g), Q.dref(g.dx[0]))
        lib.setvarnorm3d_(Q.dptr(v["mask"]), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(vn), Q.dref(1.1),
                          Q.dref(0.6981), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
        theta = np.linspace(0, 1.2, vn.size).reshape(vn.shape)
        lib.setvarnorm3dtheta_(Q.dptr(v["mask"]), Q.dptr(mx), Q.dptr(my), Q.dptr(mz), Q.dptr(vt), Q.dref(1.1),
                               Q.dptr(theta), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
        res.append((mx, my, mz, vb, vx, vy, vz, vn, vt, bm.value, um.value))
    Q.check(gpu)
    for a, b in zip(*res):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("emu", [0, 1, 2])
def test_reinit_kernels(gpu, oracle, emu):
    """Distance function and reinitialisation RHS, with the RHS's tests, square
    root and division natively (0) or on the integer pipes (1, 2); phi0 holds
    values inside the +-1e-5 band (sign 0) and signed zeros, phi holds flat
    patches (zero one-sided differences)."""
    g, v = pack_case(oracle, N, seed=5)
    rng = np.random.default_rng(55)
    phi0 = v["phi"].copy()
    sel = rng.random(phi0.shape) < 0.05
    phi0[sel] = rng.choice([0.0, -0.0, 5e-6, -5e-6, 1e-5, -1e-5], sel.sum())
    phi = phi0 + 0.01 * np.sin(np.arange(phi0.size).reshape(phi0.shape))
    flat = rng.random(phi.shape) < 0.1
    phi[flat] = 0.02
    phi[rng.random(phi.shape) < 0.02] = rng.choice([0.0, -0.0, 1e-5, -1e-5, 3e-6])
    res = []
    prev = gpu.qssgpu_set_emu_level(emu)
    try:
        libs = (gpu, oracle)
        for lib in libs:
            d0 = np.zeros(v.shape)
            lib.qss3dcomputedistanceforsubcellfix_(Q.dptr(d0), Q.dptr(phi0), *Q.gb_args(g), *Q.fb_args(g),
                                                   Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]))
            rhs = np.zeros(v.shape)
            lib.qss3dcomputereinitializationeqnrhssubcellfixorder1_(
                Q.dptr(rhs), Q.dptr(phi), *Q.gb_args(g), Q.dptr(phi0), Q.dptr(d0), *Q.fb_args(g),
                Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]))
            res.append((d0, rhs))
    finally:
        gpu.qssgpu_set_emu_level(prev)
    Q.check(gpu)
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])


def test_reductions_and_imposes(gpu, oracle):
    g, v = pack_case(oracle, N, seed=6)
    rng = np.random.default_rng(6)
    f1 = v["phi"]
    f2 = f1 + 0.01 * rng.standard_normal(v.shape)
    arrs = [rng.standard_normal(v.shape) for _ in range(5)]
    test = (rng.random(v.shape) - 0.5) * 0.2
    res = []
    for lib in (gpu, oracle):
        out = []
        m = C.c_double(0)
        lib.qss3dmaxnormdifflocal_(C.byref(m), Q.dptr(f1), *Q.gb_args(g), Q.dptr(f2), *Q.gb_args(g),
                                   *Q.fb_args(g), Q.dref(0.8))
        out.append(m.value)
        vol = C.c_double(0)
        lib.qss3dvolumeregionphilessthanzero_(C.byref(vol), Q.dptr(f1), *Q.gb_args(g), *Q.fb_args(g),
                                              Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]), Q.dref(0.06))
        out.append(vol.value)
        pm = f2.copy()
        lib.imposemaskparallel_(Q.dptr(pm), Q.dptr(v["mask"]), Q.dptr(f1), Q.dref(0.012), *Q.gb_args(g),
                                C.byref(C.c_int(2)), C.byref(C.c_int(g.khi_gb - 4)))
        out.append(pm)
        arrs_copy = [a.copy() for a in arrs]
        lib.imposetrapvelocity3d_(Q.dptr(test), Q.dptr(test), *[Q.dptr(a) for a in arrs_copy], *Q.gb_args(g),
                                  *Q.fb_args(g), Q.dref(g.dx[0]))
        out += arrs_copy
        res.append(out)
    Q.check(gpu)
    for a, b in zip(*res):
        assert np.array_equal(np.asarray(a), np.asarray(b))
