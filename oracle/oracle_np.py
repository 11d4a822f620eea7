"""oracle_np.py -- TEST INFRASTRUCTURE (oracle), never part of the product.

A second restatement of the 3-D Fortran kernels on the level-set path, in
numpy, written from the Fortran source independently of the C restatement
(oracle_kernels3d.c).  No Fortran compiler exists here, so the Fortran
kernels can only be restated; two restatements that agree bit for bit on
random inputs rule out transcription slips in either.  Only the tests use
it, to check the C restatement.

Arithmetic follows the FP64 build of the reference (default REAL kind 8, so
literals such as 1e-6 and 1.e-5 are doubles).  Every expression is evaluated
in Fortran source order, one IEEE operation at a time (numpy applies each
operator separately and never contracts a product into a sum): a+b+c is
(a+b)+c, x**2 is x*x, unary minus binds looser than '*'.

Arrays are numpy (nz, ny, nx) C-contiguous, i.e. Fortran (i, j, k) with i
fastest, ghost box starting at index 0; `fb` is the fill box
(ilo, ihi, jlo, jhi, klo, khi) in those indices.

"3d.f" is src/spatial_derivatives/qss_spatial_derivatives3d.f and "rk3d.f"
src/time_integration/qss_tvd_runge_kutta3d.f.
"""
import numpy as np

C13 = 1.0 / 3.0
C76 = 7.0 / 6.0
C116 = 11.0 / 6.0
C16 = 1.0 / 6.0
C56 = 5.0 / 6.0
C1312 = 13.0 / 12.0
C14 = 0.25
TINY = 1.0e-35
ZERO_TOL = 1.0e-5


def _shift(a, fb, di=0, dj=0, dk=0):
    """a(i+di, j+dj, k+dk) over the fill box."""
    ilo, ihi, jlo, jhi, klo, khi = fb
    return a[klo + dk:khi + 1 + dk, jlo + dj:jhi + 1 + dj, ilo + di:ihi + 1 + di]


def _axis(d, m):
    """offset (di, dj, dk) of m steps along axis d (0 = x, 1 = y, 2 = z)."""
    o = [0, 0, 0]
    o[d] = m
    return o


def weno5_side(v1, v2, v3, v4, v5):
    """HJ WENO5 reconstruction from five scaled differences (3d.f:1981-2014)."""
    eps = 1e-6 * np.maximum(np.maximum(np.maximum(np.maximum(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5) + TINY
    p1 = (C13 * v1 - C76 * v2) + C116 * v3
    p2 = (-(C16 * v2) + C56 * v3) + C13 * v4
    p3 = (C13 * v3 + C56 * v4) - C16 * v5
    t = (v1 - 2.0 * v2) + v3
    u = (v1 - 4.0 * v2) + 3.0 * v3
    s1 = C1312 * (t * t) + C14 * (u * u)
    t = (v2 - 2.0 * v3) + v4
    u = v2 - v4
    s2 = C1312 * (t * t) + C14 * (u * u)
    t = (v3 - 2.0 * v4) + v5
    u = (3.0 * v3 - 4.0 * v4) + v5
    s3 = C1312 * (t * t) + C14 * (u * u)
    q1, q2, q3 = s1 + eps, s2 + eps, s3 + eps
    a1 = 0.1 / (q1 * q1)
    a2 = 0.6 / (q2 * q2)
    a3 = 0.3 / (q3 * q3)
    inv = 1.0 / ((a1 + a2) + a3)
    a1, a2, a3 = a1 * inv, a2 * inv, a3 * inv
    return (a1 * p1 + a2 * p2) + a3 * p3


def weno5_plus_minus(phi, fb, d, inv):
    """phi_plus and phi_minus along axis d (3d.f:1969-2247): faces
    D(m) = phi(i+m) - phi(i+m-1), scaled by 1/dx."""
    D = {m: _shift(phi, fb, *_axis(d, m)) - _shift(phi, fb, *_axis(d, m - 1)) for m in range(-2, 4)}
    plus = weno5_side(D[3] * inv, D[2] * inv, D[1] * inv, D[0] * inv, D[-1] * inv)
    minus = weno5_side(D[-2] * inv, D[-1] * inv, D[0] * inv, D[1] * inv, D[2] * inv)
    return plus, minus


def eno2_plus_minus(phi, fb, d, inv):
    """ENO2 phi_plus and phi_minus along axis d (3d.f:1113-1182, the same
    text in the constant-coefficient variant 3d.f:394-463): second
    differences taken from phi directly, the smaller one in magnitude
    chosen (ties take the second)."""
    def s(m):
        return _shift(phi, fb, *_axis(d, m))

    D1 = s(0) - s(-1)
    D1p = s(1) - s(0)
    D2 = (s(1) + s(-1)) - 2.0 * s(0)
    D2p = (s(2) + s(0)) - 2.0 * s(1)
    D2m = (s(-2) + s(0)) - 2.0 * s(-1)
    plus = np.where(np.abs(D2) < np.abs(D2p), (D1p - 0.5 * D2) * inv, (D1p - 0.5 * D2p) * inv)
    minus = np.where(np.abs(D2m) < np.abs(D2), (D1 + 0.5 * D2m) * inv, (D1 + 0.5 * D2) * inv)
    return plus, minus


def eno3_plus_minus(phi, fb, d, inv, inv_minus):
    """ENO3 phi_plus and phi_minus along axis d (3d.f:1446-1700, the same
    text in the constant-coefficient variant 3d.f:676-931).  Kept as the
    Fortran has them: the x stencil's outermost plus point is phi(i+3,j,j)
    (3d.f:1454), and the y and z minus derivatives are scaled by 1/dx
    (inv_minus = 1/dx for every axis)."""
    def s(m):
        return _shift(phi, fb, *_axis(d, m))

    if d == 0:
        ilo, ihi, jlo, jhi, klo, khi = fb
        J = np.arange(jlo, jhi + 1)[:, None]
        I = np.arange(ilo, ihi + 1)[None, :]
        far = np.broadcast_to(phi[J, J, I + 3][None, :, :], s(0).shape)
    else:
        far = s(3)
    D1 = s(0) - s(-1)
    D1p = s(1) - s(0)
    D1m = s(-1) - s(-2)
    D1mm = s(-2) - s(-3)
    D1pp = s(2) - s(1)
    D1ppp = far - s(2)
    D2 = D1p - D1
    D2p = D1pp - D1p
    D2m = D1 - D1m
    D2pp = D1ppp - D1pp
    D2mm = D1m - D1mm
    D3 = D2 - D2m
    D3p = D2p - D2
    D3pp = D2pp - D2p
    D3m = D2m - D2mm
    third, sixth = 1.0 / 3.0, 1.0 / 6.0

    a = D1p - 0.5 * D2
    a = np.where(np.abs(D3) < np.abs(D3p), a - sixth * D3, a - sixth * D3p)
    c = D1p - 0.5 * D2p
    c = np.where(np.abs(D3p) < np.abs(D3pp), c + third * D3p, c + third * D3pp)
    plus = np.where(np.abs(D2) < np.abs(D2p), a, c) * inv

    a = D1 + 0.5 * D2m
    a = np.where(np.abs(D3m) < np.abs(D3), a + third * D3m, a + third * D3)
    c = D1 + 0.5 * D2
    c = np.where(np.abs(D3) < np.abs(D3p), c - sixth * D3, c - sixth * D3p)
    minus = np.where(np.abs(D2m) < np.abs(D2), a, c) * inv_minus
    return plus, minus


def _sq(x):
    return x * x


def _assemble(pm, phi, vn, b, adv, fb, dx, dy, dz, norm_sign):
    """The part every right-hand-side variant shares (3d.f:2249-2385 for
    WENO5; the same text for ENO2 3d.f:1183-1320 and ENO3 3d.f:1701-1812,
    and without the advection term for the constant-coefficient variants):
    Godunov normal term (sign +1 for WENO5, -1 otherwise), CFL estimate of
    the last voxel, upwind advection (adv = (vx, vy, vz) or None), central
    curvature.  vn and b are arrays over the fill box."""
    inv = (1.0 / dx, 1.0 / dy, 1.0 / dz)
    fac = (0.5 / dx, 0.5 / dy, 0.5 / dz)
    (pxp, pxm), (pyp, pym), (pzp, pzm) = pm

    # Godunov |grad phi|^2
    zero = 0.0
    pos = ((np.maximum(_sq(np.maximum(pxm, zero)), _sq(np.minimum(pxp, zero)))
            + np.maximum(_sq(np.maximum(pym, zero)), _sq(np.minimum(pyp, zero))))
           + np.maximum(_sq(np.maximum(pzm, zero)), _sq(np.minimum(pzp, zero))))
    neg = ((np.maximum(_sq(np.minimum(pxm, zero)), _sq(np.maximum(pxp, zero)))
            + np.maximum(_sq(np.minimum(pym, zero)), _sq(np.maximum(pyp, zero))))
           + np.maximum(_sq(np.minimum(pzm, zero)), _sq(np.maximum(pzp, zero))))
    ngps = np.where(vn > 0.0, pos, neg)
    set_here = np.abs(vn) >= ZERO_TOL
    signed_vn = vn if norm_sign > 0 else -vn
    norm_here = (signed_vn * np.sqrt(ngps)).ravel()
    # carried temp_norm in loop order (i fastest, then j, then k)
    flat_set = set_here.ravel()
    last = np.maximum.accumulate(np.where(flat_set, np.arange(flat_set.size), -1))
    temp_norm = np.where(last >= 0, norm_here[np.maximum(last, 0)], 0.0).reshape(vn.shape)

    # CFL estimate of the last voxel
    mdx = max(dx, dy, dz)
    max_dx_sq = mdx * mdx
    cx = np.maximum(np.abs(pxp), np.abs(pxm))[-1, -1, -1]
    cy = np.maximum(np.abs(pyp), np.abs(pym))[-1, -1, -1]
    cz = np.maximum(np.abs(pzp), np.abs(pzm))[-1, -1, -1]
    ngp = np.sqrt(((cx * cx + cy * cy) + cz * cz) + max_dx_sq)
    h = abs(vn[-1, -1, -1]) / ngp * ((cx * inv[0] + cy * inv[1]) + cz * inv[2])
    max_h = h if h > -1.0 else -1.0

    # central curvature
    def s(di=0, dj=0, dk=0):
        return _shift(phi, fb, di, dj, dk)

    p0 = s()
    px = (s(1) - s(-1)) * fac[0]
    py = (s(0, 1) - s(0, -1)) * fac[1]
    pz = (s(0, 0, 1) - s(0, 0, -1)) * fac[2]
    pxx = (((s(2) + s(-2)) - 2.0 * p0) * fac[0]) * fac[0]
    pzz = (((s(0, 0, 2) + s(0, 0, -2)) - 2.0 * p0) * fac[2]) * fac[2]
    pyy = (((s(0, 2) + s(0, -2)) - 2.0 * p0) * fac[1]) * fac[1]
    pxy = ((((s(1, 1) + s(-1, -1)) - s(-1, 1)) - s(1, -1)) * fac[0]) * fac[1]
    pxz = ((((s(1, 0, 1) + s(-1, 0, -1)) - s(-1, 0, 1)) - s(1, 0, -1)) * fac[0]) * fac[2]
    pyz = ((((s(0, 1, 1) + s(0, -1, -1)) - s(0, -1, 1)) - s(0, 1, -1)) * fac[1]) * fac[2]
    g2 = (px * px + py * py) + pz * pz
    curv = (pxx * py) * py
    curv = curv + (pyy * px) * px
    curv = curv - ((2.0 * pxy) * px) * py
    curv = curv + (pxx * pz) * pz
    curv = curv + (pzz * px) * px
    curv = curv - ((2.0 * pxz) * px) * pz
    curv = curv + (pyy * pz) * pz
    curv = curv + (pzz * py) * py
    curv = curv - ((2.0 * pyz) * py) * pz
    with np.errstate(divide="ignore", invalid="ignore"):
        curv = np.where(g2 < ZERO_TOL, 0.0, curv / g2)
    temp_curv = b * curv
    if adv is None:
        return temp_norm + temp_curv, max_h

    # upwind advection
    ux, uy, uz = adv
    pxa = np.where(ux >= 0, pxm, pxp)
    pya = np.where(uy >= 0, pym, pyp)
    pza = np.where(uz >= 0, pzm, pzp)
    temp_vel = -((ux * pxa + uy * pya) + uz * pza)
    return (temp_norm + temp_curv) + temp_vel, max_h


def _derivs(scheme, phi, fb, dx, dy, dz):
    inv = (1.0 / dx, 1.0 / dy, 1.0 / dz)
    if scheme == 2:
        return [eno2_plus_minus(phi, fb, d, inv[d]) for d in range(3)]
    if scheme == 3:
        return [eno3_plus_minus(phi, fb, d, inv[d], inv[0]) for d in range(3)]
    return [weno5_plus_minus(phi, fb, d, inv[d]) for d in range(3)]


def rhs_var(scheme, phi, vel_n, b, vx, vy, vz, fb, dx, dy, dz):
    """getRHS3d2nd / getRHS3d3rd / getRHS3d5th (scheme 2, 3, 5; 3d.f:1020,
    1335, 1827) on the fill box: returns (lse_rhs over the fill box,
    max_H_over_dX).

    Kept as the Fortran has them: the normal term is -vel_n*|grad phi|
    except +vel_n*|grad phi| in getRHS3d5th (3d.f:2276); temp_norm keeps the
    previous voxel's value (loop order) where |vel_n| < 1e-5, 0 before the
    first voxel that sets it; max_H_over_dX is reset inside the loop, so the
    last voxel's H is returned."""
    pm = _derivs(scheme, phi, fb, dx, dy, dz)
    adv = (_shift(vx, fb), _shift(vy, fb), _shift(vz, fb))
    return _assemble(pm, phi, _shift(vel_n, fb), _shift(b, fb), adv, fb, dx, dy, dz, 1 if scheme == 5 else -1)


def rhs_weno5(phi, vel_n, b, vx, vy, vz, fb, dx, dy, dz):
    """getRHS3d5th (3d.f:1827-2385), see rhs_var."""
    return rhs_var(5, phi, vel_n, b, vx, vy, vz, fb, dx, dy, dz)


def rhs_const(scheme, phi, a, bconst, fb, dx, dy, dz):
    """getRHS3d2ndConst / getRHS3d3rdConst (scheme 2, 3; 3d.f:302, 572):
    constant normal speed a and curvature coefficient b, no advection;
    returns (lse_rhs over the fill box, max_H_over_dX)."""
    pm = _derivs(scheme, phi, fb, dx, dy, dz)
    shape = _shift(phi, fb).shape
    return _assemble(pm, phi, np.full(shape, float(a)), np.full(shape, float(bconst)), None, fb, dx, dy, dz, -1)


def rk1(u_cur, rhs, dt):
    """qss3dRK1Step (rk3d.f:48), elementwise."""
    return u_cur + dt * rhs


def tvdrk2_stage2(u_stage1, u_cur, rhs, dt):
    """qss3dTVDRK2Stage2 (rk3d.f:117-118), elementwise."""
    return 0.75 * u_cur + 0.25 * (u_stage1 + dt * rhs)


def tvdrk3_stage3(u_stage2, u_cur, rhs, dt):
    """qss3dTVDRK3Stage3 (rk3d.f:190-192), elementwise."""
    return C13 * u_cur + (2.0 / 3.0) * (u_stage2 + dt * rhs)


def signed_linear_extrapolation(phi, fb, face):
    """signedLinearExtrapolation3d (3d.f:3055-3190), in place on phi: face 0/1
    x low/high, 2/3 y, 4/5 z; the ghost layers beyond the fill box continue
    the boundary value with slope sign(phi_b)*|phi_b - phi_inner| per layer,
    over the whole ghost box in the other two directions."""
    ilo, ihi, jlo, jhi, klo, khi = fb
    d = face // 2
    ax = 2 - d  # numpy axis of the Fortran direction d
    lo_side = face % 2 == 0
    b = (ilo, jlo, klo)[d] if lo_side else (ihi, jhi, khi)[d]
    inner = b + 1 if lo_side else b - 1
    pb = np.take(phi, b, axis=ax)
    pin = np.take(phi, inner, axis=ax)
    slope = np.copysign(1.0, pb) * np.abs(pb - pin)
    n = phi.shape[ax]
    layers = range(0, b) if lo_side else range(b + 1, n)
    for m in layers:
        dist = float(b - m) if lo_side else float(m - b)
        idx = [slice(None)] * 3
        idx[ax] = m
        phi[tuple(idx)] = pb + slope * dist
    return phi
