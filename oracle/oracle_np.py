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
    """HJ WENO5 reconstruction from five scaled differences (3d.f:1976-2005)."""
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
    """phi_plus and phi_minus along axis d (3d.f:1962-2250): faces
    D(m) = phi(i+m) - phi(i+m-1), scaled by 1/dx."""
    D = {m: _shift(phi, fb, *_axis(d, m)) - _shift(phi, fb, *_axis(d, m - 1)) for m in range(-2, 4)}
    plus = weno5_side(D[3] * inv, D[2] * inv, D[1] * inv, D[0] * inv, D[-1] * inv)
    minus = weno5_side(D[-2] * inv, D[-1] * inv, D[0] * inv, D[1] * inv, D[2] * inv)
    return plus, minus


def eno2_plus_minus(phi, fb, d, inv):
    """ENO2 phi_plus and phi_minus along axis d (3d.f:1119-1190, the same
    text in the constant-coefficient variant 3d.f:387-458): second
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
    """ENO3 phi_plus and phi_minus along axis d (3d.f:1449-1680, the same
    text in the constant-coefficient variant 3d.f:672-903).  Kept as the
    Fortran has them: the x stencil's outermost plus point is phi(i+3,j,j)
    (3d.f:1454), and the y and z minus derivatives are scaled by 1/dx
    (3d.f:1600, 1677; inv_minus = 1/dx for every axis)."""
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
    """The part every right-hand-side variant shares (3d.f:2251-2379 for
    WENO5; the same text for ENO2 3d.f:1191-1319 and ENO3 3d.f:1681-1809,
    and without the advection term for the constant-coefficient variants
    3d.f:459-560 and 904-1004):
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
    """getRHS3d5th (3d.f:1827-2386), see rhs_var."""
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


# ---------------------------------------------------------------------------
# coefficients of the variable model, "util3d.f" = src/utilities/qss_util3d.f

PI = 3.14159265358979323846
ONE_OVER_PI = 0.31830988618379


def _basic_heaviside(x):
    """basicHeaviside (util3d.f:477-494): 0 below zero, 1 above, 1/2 at zero."""
    return np.where(x < 0, 0.0, np.where(x > 0, 1.0, 0.5))


def heaviside(x, eps, sin=np.sin):
    """qssHeaviside (util3d.f:450-471); `sin` is the sine the caller's build
    uses (the reference's libm, or the oracle's portable one)."""
    v1 = _basic_heaviside(x + eps)
    v2 = _basic_heaviside(eps - x)
    v3 = _basic_heaviside(x - eps)
    return (((0.5 + x / (2.0 * eps)) + (0.5 * ONE_OVER_PI) * sin((PI * x) / eps)) * v1) * v2 + v3


def _mask_terms(mask, mx, my, mz, fb, dx, sin):
    """h1, h2, |grad mask|, s of 3d.f:72-80 (the same text in 3d.f:156-164
    and 3d.f:263-271)."""
    m = _shift(mask, fb)
    gx, gy, gz = _shift(mx, fb), _shift(my, fb), _shift(mz, fb)
    eps_var = 1.5 * dx
    h1 = heaviside(-m, eps_var, sin)
    h2 = heaviside(m, eps_var, sin)
    absgrad = np.sqrt((gx * gx + gy * gy) + gz * gz)
    x = np.sqrt(m * m + ((absgrad * dx) * absgrad) * dx)
    s = m / x
    return h1, h2, absgrad, s, gx, gy, gz


def set_var_norm(mask, mx, my, mz, a0, ca, fb, dx, sin=np.sin, cos=np.cos):
    """setVarNorm3d (3d.f:13-87) with a scalar contact angle ca, or
    setVarNorm3dTheta (3d.f:94-172) with ca an array: the normal speed over
    the fill box, h1*a0 - s*h2*1*cos(ca)*|grad mask|."""
    h1, h2, absgrad, s, *_ = _mask_terms(mask, mx, my, mz, fb, dx, sin)
    c = cos(_shift(ca, fb)) if np.ndim(ca) else cos(np.full(h1.shape, float(ca)))
    return h1 * a0 - (((s * h2) * 1.0) * c) * absgrad


def set_var_curv_adv(mask, mx, my, mz, const_b, fb, dx, sin=np.sin):
    """setVarCurvAdv3d (3d.f:178-298): curvature coefficient b = h1*const_b,
    advection field s*1*grad mask*h2 and the two CFL bounds (true maxima,
    -1 for an empty box): returns (b, vx, vy, vz, b_max_over_dx,
    max_U_over_dx)."""
    h1, h2, absgrad, s, gx, gy, gz = _mask_terms(mask, mx, my, mz, fb, dx, sin)
    inv = 1.0 / dx
    b = h1 * const_b
    vx = ((s * 1.0) * gx) * h2
    vy = ((s * 1.0) * gy) * h2
    vz = ((s * 1.0) * gz) * h2
    u = (np.abs(vx) * inv + np.abs(vy) * inv) + np.abs(vz) * inv
    b_max = max(-1.0, float(b.max())) if b.size else -1.0
    u_max = max(-1.0, float(u.max())) if u.size else -1.0
    return b, vx, vy, vz, (2.0 * b_max) * ((inv * inv + inv * inv) + inv * inv), u_max


def central_grad(phi, fb, dx, dy, dz):
    """getCentralGrad3dOrder2 (3d.f:2987-3048) over the fill box."""
    def s(di=0, dj=0, dk=0):
        return _shift(phi, fb, di, dj, dk)

    return ((s(1) - s(-1)) * (0.5 / dx), (s(0, 1) - s(0, -1)) * (0.5 / dy), (s(0, 0, 1) - s(0, 0, -1)) * (0.5 / dz))


def impose_trap_velocity(mask_w, fields, fb, dx):
    """imposeTrapVelocity3d (util3d.f:499-581), in place: the five fields
    are zeroed on the fill box where the tested array exceeds 1.5*dx."""
    sel = _shift(mask_w, fb) > 1.5 * dx
    for f in fields:
        _shift(f, fb)[sel] = 0.0
    return fields


def impose_mask(mask, phi, overlap, klo, khi):
    """imposeMaskParallel (util3d.f:130-177; scalar overlap: max(mask -
    overlap, phi)) and imposeMaskParallelVar (util3d.f:181-230; array
    overlap: mask itself where mask - overlap > phi) on z-planes klo..khi of
    the whole ghost box."""
    m, p = mask[klo:khi + 1], phi[klo:khi + 1]
    if np.ndim(overlap):
        return np.where(m - overlap[klo:khi + 1] > p, m, p)
    t = m - overlap
    return np.where(t > p, t, p)


def max_norm_diff_local(f1, f2, ib, zone):
    """qss3dMaxNormDiffLocal (util3d.f:65-125): max |f1 - f2| where |f1| <
    zone over the box ib, -1 when no voxel qualifies."""
    a, b = _shift(f1, ib), _shift(f2, ib)
    d = np.abs(a - b)[np.abs(a) < zone]
    return max(-1.0, float(d.max())) if d.size else -1.0


def volume_phi_less_than_zero(phi, ib, dx, dy, dz, eps, sin=np.sin):
    """qss3dVolumeRegionPhiLessThanZero (util3d.f:288-359): the loop-order
    sum of dV (phi < -eps) and (1 - H(phi))*dV (|phi| < eps), added one
    voxel after the other in loop order (i fastest)."""
    dV = (dx * dy) * dz
    p = _shift(phi, ib).ravel()
    x = p / eps
    one_minus_h = 0.5 * ((1.0 - x) - ONE_OVER_PI * sin(PI * x))
    c = np.where(p < -eps, dV, np.where(p < eps, one_minus_h * dV, 0.0))
    return float(np.add.accumulate(np.concatenate(([0.0], c)))[-1])


# ---------------------------------------------------------------------------
# reinitialisation, "reinit3d.f" = src/reinitialization/qss_reinitialization3d.f

def distance_for_subcell_fix(phi0, fb, dx, dy, dz):
    """qss3dComputeDistanceForSubcellFix (reinit3d.f:476-580): phi0/delta at
    voxels with a sign change to a face neighbour (delta the largest of the
    one- and two-sided differences of the three axes and 1e-5), -1000*max
    spacing elsewhere."""
    def s(di=0, dj=0, dk=0):
        return _shift(phi0, fb, di, dj, dk)

    p = s()
    near = np.zeros(p.shape, bool)
    for o in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        q = s(*o)
        near |= ((q > 0.0) & (p <= 0.0)) | ((q <= 0.0) & (p > 0.0))
    delta = np.full(p.shape, ZERO_TOL)
    for d in range(3):
        up, dn = s(*_axis(d, 1)), s(*_axis(d, -1))
        d1 = np.abs(up - dn) / 2.0
        d2 = np.abs(up - p)
        d3 = np.abs(p - dn)
        delta = np.maximum(np.maximum(np.maximum(d1, d2), d3), delta)
    flag = -1000.0 * max(dx, dy, dz)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(near, p / delta, flag)


def reinit_rhs_subcell_fix(phi, phi0, distance0, fb, dx, dy, dz):
    """qss3dComputeReinitializationEqnRHSSubcellFixOrder1 (reinit3d.f:585-742)
    over the fill box: first-order Godunov away from the interface (where
    distance0 holds the flag), the Russo-Smereka subcell term
    distance0 - sgn(phi0)*|phi|/max_dx next to it."""
    def s(a, di=0, dj=0, dk=0):
        return _shift(a, fb, di, dj, dk)

    max_dx = max(dx, dy, dz)
    flag = -1000.0 * max_dx
    inv = (1.0 / dx, 1.0 / dy, 1.0 / dz)
    p = s(phi)
    p0 = s(phi0)
    dist = s(distance0)
    sgn = np.where(np.abs(p0) > ZERO_TOL, np.copysign(1.0, p0), 0.0)
    pos = p > 0.0
    g2 = None
    for d in range(3):
        plus = (s(phi, *_axis(d, 1)) - p) * inv[d]
        minus = (p - s(phi, *_axis(d, -1))) * inv[d]
        gp = np.where(pos, np.maximum(-plus, 0.0), np.maximum(plus, 0.0))
        gm = np.where(pos, np.maximum(minus, 0.0), np.maximum(-minus, 0.0))
        star = np.maximum(gp, gm)
        g2 = star * star if g2 is None else g2 + star * star
    away = np.where(np.abs(p) > ZERO_TOL, sgn - sgn * np.sqrt(g2), 0.0)
    near = dist - (sgn * np.abs(p)) / max_dx
    return np.where(dist == flag, away, near)
