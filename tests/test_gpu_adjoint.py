"""Adjoint mode (qssgpu_adjoint_theta): the gradient of the saturation-mismatch
loss with respect to a spatially varying contact angle.

The angle field is the trilinear interpolation of an 8 x 8 x 8 control grid
(as in the adjoint configuration); the library's per-voxel gradient is
wrapped in a torch.autograd.Function here, composed with the interpolation
in torch, and checked against
  * central finite differences of the library's own forward (h = 1e-6 rad,
    relative error <= 1e-5 on the controls with the largest gradients);
  * an FP64 PyTorch-autograd replica of the same forward model (WENO5 +
    Godunov + curvature + upwind advection, TVD-RK3, signed linear
    extrapolation of the ghost layers, mask imposition);
and the gradient must not depend on the checkpoint interval."""
import ctypes as C
import math

import numpy as np
import pytest

import qssgpu as Q
from qss_cases import pack_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N = 18
STEPS = 6
A0 = 0.2 / 0.04  # curvature 0.2 per voxel
B = 0.04


def _setup(oracle, gpu):
    g, v = pack_case(oracle, N, seed=3, radius=4.0, porosity=0.35)
    o = Q.default_options(gpu)
    o.a, o.b, o.overlap, o.theta = A0, B, 0.0, 0.0
    dx = g.dx[0]
    dt = 0.5 / (2 * B * 3 / dx ** 2 + 2.0 / dx + abs(A0) * math.sqrt(3) / dx)
    return g, v, o, dt


def _interp_matrix(g, nc=8):
    """Trilinear weights from the nc^3 control grid to the fill-box voxels."""
    n = g.ihi_fb - g.ilo_fb + 1
    t = np.arange(n) / (n - 1) * (nc - 1)
    i0 = np.minimum(np.floor(t).astype(int), nc - 2)
    f = t - i0
    W = np.zeros((n, n, n, nc, nc, nc))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                wz = np.where(dz, f, 1 - f)[:, None, None]
                wy = np.where(dy, f, 1 - f)[None, :, None]
                wx = np.where(dx, f, 1 - f)[None, None, :]
                w = wz * wy * wx
                kk, jj, ii = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
                W[kk, jj, ii, (i0 + dz)[kk], (i0 + dy)[jj], (i0 + dx)[ii]] += w
    return W.reshape(n ** 3, nc ** 3)


def _to_ghost(g, fill):
    ng = g.grid_dims_ghostbox[0]
    out = np.zeros((ng, ng, ng))
    s = slice(g.ilo_fb - g.ilo_gb, g.ihi_fb - g.ilo_gb + 1)
    out[s, s, s] = fill.reshape(out[s, s, s].shape)
    return out


def _fill(g, a):
    s = slice(g.ilo_fb - g.ilo_gb, g.ihi_fb - g.ilo_gb + 1)
    return a[s, s, s]


def _run(gpu, o, v, g, theta, target, dt, ckpt=3, grad=True):
    th = np.ascontiguousarray(theta)
    tg = np.ascontiguousarray(target)
    loss = C.c_double(0)
    if grad:
        gr = np.zeros_like(th)
        rc = gpu.qssgpu_adjoint_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(th), Q.dptr(tg), STEPS, dt, ckpt,
                                      C.byref(loss), Q.dptr(gr))
    else:
        gr = None
        rc = gpu.qssgpu_forward_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(th), Q.dptr(tg), STEPS, dt,
                                      C.byref(loss), None)
    assert rc == 0, gpu.qssgpu_error_string()
    return loss.value, gr


@pytest.fixture(scope="module")
def problem(oracle, gpu):
    g, v, o, dt = _setup(oracle, gpu)
    W = _interp_matrix(g)
    rng = np.random.default_rng(3)
    ctrl = rng.uniform(0, math.radians(60), 512)
    hidden = np.random.default_rng(4).uniform(0, math.radians(60), 512)
    # target: H(phi_T) of the hidden angles (one forward with a zero target gives
    # sum H^2; the target field itself comes from the replica below)
    return g, v, o, dt, W, ctrl, hidden


# ---------------------------------------------------------------------------
# FP64 PyTorch replica of the forward model

def _heaviside(x, eps):
    return torch.where(x < -eps, torch.zeros_like(x),
                       torch.where(x > eps, torch.ones_like(x),
                                   0.5 + x / (2 * eps) + (0.5 / math.pi) * torch.sin(math.pi * x / eps)))


def _side(v1, v2, v3, v4, v5):
    m = torch.maximum(torch.maximum(torch.maximum(torch.maximum(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5)
    eps = 1e-6 * m + 1e-35
    p1 = v1 / 3 - 7 / 6 * v2 + 11 / 6 * v3
    p2 = -(v2 / 6) + 5 / 6 * v3 + v4 / 3
    p3 = v3 / 3 + 5 / 6 * v4 - v5 / 6
    S1 = 13 / 12 * (v1 - 2 * v2 + v3) ** 2 + 0.25 * (v1 - 4 * v2 + 3 * v3) ** 2
    S2 = 13 / 12 * (v2 - 2 * v3 + v4) ** 2 + 0.25 * (v2 - v4) ** 2
    S3 = 13 / 12 * (v3 - 2 * v4 + v5) ** 2 + 0.25 * (3 * v3 - 4 * v4 + v5) ** 2
    a1, a2, a3 = 0.1 / (S1 + eps) ** 2, 0.6 / (S2 + eps) ** 2, 0.3 / (S3 + eps) ** 2
    s = a1 + a2 + a3
    return (a1 * p1 + a2 * p2 + a3 * p3) / s


def _shift(phi, d, k, lo, hi):
    """phi at offset k along axis d (torch dims z, y, x = 0, 1, 2) over the fill box."""
    sl = [slice(lo, hi + 1)] * 3
    sl[d] = slice(lo + k, hi + 1 + k)
    return phi[tuple(sl)]


def _rhs(phi, vel, bco, V, lo, hi, dx):
    inv = 1.0 / dx
    pp, pm = [], []
    for d in (2, 1, 0):  # x, y, z
        P = {k: _shift(phi, d, k, lo, hi) for k in range(-3, 4)}
        F = {m: (P[m] - P[m - 1]) * inv for m in range(-2, 4)}
        pp.append(_side(F[3], F[2], F[1], F[0], F[-1]))
        pm.append(_side(F[-2], F[-1], F[0], F[1], F[2]))
    pos = vel > 0
    ng = 0
    for d in range(3):
        a = torch.where(pos, torch.clamp(pm[d], min=0), torch.clamp(pm[d], max=0))
        c = torch.where(pos, torch.clamp(pp[d], max=0), torch.clamp(pp[d], min=0))
        ng = ng + torch.where(a * a > c * c, a * a, c * c)
    norm = torch.where(ng > 0, torch.sqrt(torch.where(ng > 0, ng, torch.ones_like(ng))), torch.zeros_like(ng))
    tn = vel * norm
    tv = 0
    for d in range(3):
        tv = tv - V[d] * torch.where(V[d] >= 0, pm[d], pp[d])
    f = 0.5 / dx
    c0 = _shift(phi, 0, 0, lo, hi)
    gx = (_shift(phi, 2, 1, lo, hi) - _shift(phi, 2, -1, lo, hi)) * f
    gy = (_shift(phi, 1, 1, lo, hi) - _shift(phi, 1, -1, lo, hi)) * f
    gz = (_shift(phi, 0, 1, lo, hi) - _shift(phi, 0, -1, lo, hi)) * f
    xx = (_shift(phi, 2, 2, lo, hi) + _shift(phi, 2, -2, lo, hi) - 2 * c0) * f * f
    yy = (_shift(phi, 1, 2, lo, hi) + _shift(phi, 1, -2, lo, hi) - 2 * c0) * f * f
    zz = (_shift(phi, 0, 2, lo, hi) + _shift(phi, 0, -2, lo, hi) - 2 * c0) * f * f

    def mixed(d1, d2):
        sl = lambda a, b: phi[tuple(slice(lo + (a if dd == d1 else b if dd == d2 else 0),
                                          hi + 1 + (a if dd == d1 else b if dd == d2 else 0)) for dd in range(3))]
        return (sl(1, 1) + sl(-1, -1) - sl(-1, 1) - sl(1, -1)) * f * f

    xy, xz, yz = mixed(2, 1), mixed(2, 0), mixed(1, 0)
    grad = gx * gx + gy * gy + gz * gz
    curv = (xx * gy * gy + yy * gx * gx - 2 * xy * gx * gy + xx * gz * gz + zz * gx * gx - 2 * xz * gx * gz +
            yy * gz * gz + zz * gy * gy - 2 * yz * gy * gz)
    kappa = torch.where(grad >= 1e-5, curv / torch.where(grad >= 1e-5, grad, torch.ones_like(grad)),
                        torch.zeros_like(grad))
    return tn + bco * kappa + tv


def _extrap(f, g, dist):
    return f + torch.copysign(torch.ones_like(f), f) * torch.abs(f - g) * dist


def _bc(a, lo, hi):
    """Signed linear extrapolation, faces x, then y, then z (ghost box (z, y, x))."""
    n = a.shape[0]
    # x faces for j, k in the fill box
    mid = a[lo:hi + 1, lo:hi + 1, :]
    left = [_extrap(mid[:, :, lo], mid[:, :, lo + 1], lo - i) for i in range(lo)]
    right = [_extrap(mid[:, :, hi], mid[:, :, hi - 1], i - hi) for i in range(hi + 1, n)]
    mid = torch.stack(left + [mid[:, :, i] for i in range(lo, hi + 1)] + right, dim=2)
    a = torch.cat([a[lo:hi + 1, :lo, :], mid, a[lo:hi + 1, hi + 1:, :]], dim=1)
    a = torch.cat([torch.zeros(lo, n, n, dtype=a.dtype), a, torch.zeros(n - hi - 1, n, n, dtype=a.dtype)], dim=0)
    # y faces for k in the fill box, all i
    mid = a[lo:hi + 1]
    low = [_extrap(mid[:, lo, :], mid[:, lo + 1, :], lo - j) for j in range(lo)]
    high = [_extrap(mid[:, hi, :], mid[:, hi - 1, :], j - hi) for j in range(hi + 1, n)]
    mid = torch.stack(low + [mid[:, j, :] for j in range(lo, hi + 1)] + high, dim=1)
    a = torch.cat([a[:lo], mid, a[hi + 1:]], dim=0)
    # z faces, all i, j
    low = [_extrap(a[lo], a[lo + 1], lo - k) for k in range(lo)]
    high = [_extrap(a[hi], a[hi - 1], k - hi) for k in range(hi + 1, n)]
    return torch.stack(low + [a[k] for k in range(lo, hi + 1)] + high, dim=0)


def _embed(fill, lo, hi, n):
    """A ghost-box tensor holding fill on the fill box (the ghost values are
    rebuilt by _bc from the fill box alone)."""
    return torch.nn.functional.pad(fill, (lo, n - hi - 1, lo, n - hi - 1, lo, n - hi - 1))


def replica_loss(g, v, mx, my, mz, bco, V, theta_fill, target_fill, dt):
    dx = g.dx[0]
    lo, hi = g.ilo_fb - g.ilo_gb, g.ihi_fb - g.ilo_gb
    mask = torch.tensor(v["mask"])
    phi = torch.tensor(v["phi"])
    eps_var = 1.5 * dx
    m = mask[lo:hi + 1, lo:hi + 1, lo:hi + 1]
    h1, h2 = _heaviside(-m, eps_var), _heaviside(m, eps_var)
    ag = torch.sqrt(mx * mx + my * my + mz * mz)
    s = m / torch.sqrt(m * m + ag * dx * ag * dx)
    vel = h1 * A0 - s * h2 * torch.cos(theta_fill) * ag
    assert float(torch.abs(vel).min()) >= 1e-5  # no carried normal terms in this set-up
    t = mask - 0.0
    n = mask.shape[0]
    for _ in range(STEPS):
        fill0 = phi[lo:hi + 1, lo:hi + 1, lo:hi + 1]
        s1 = _bc(_embed(fill0 + dt * _rhs(phi, vel, bco, V, lo, hi, dx), lo, hi, n), lo, hi)
        f1 = s1[lo:hi + 1, lo:hi + 1, lo:hi + 1]
        s2 = _bc(_embed(0.75 * fill0 + 0.25 * (f1 + dt * _rhs(s1, vel, bco, V, lo, hi, dx)), lo, hi, n), lo, hi)
        f2 = s2[lo:hi + 1, lo:hi + 1, lo:hi + 1]
        s3 = _bc(_embed(fill0 / 3 + 2 / 3 * (f2 + dt * _rhs(s2, vel, bco, V, lo, hi, dx)), lo, hi, n), lo, hi)
        phi = torch.where(t > s3, t, s3)
    H = _heaviside(phi[lo:hi + 1, lo:hi + 1, lo:hi + 1], 1.5 * dx)
    return ((H - target_fill) ** 2).sum(), H


def _coefficients(oracle, g, v):
    """Mask gradient, curvature coefficient and advection field (theta-independent)."""
    arrs = {k: np.zeros(v["mask"].shape) for k in ("mx", "my", "mz", "b", "vx", "vy", "vz")}
    oracle.getcentralgrad3dorder2_(Q.dptr(arrs["mx"]), Q.dptr(arrs["my"]), Q.dptr(arrs["mz"]), *Q.gb_args(g),
                                   Q.dptr(v["mask"]), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]),
                                   Q.dref(g.dx[1]), Q.dref(g.dx[2]))
    bm, um = C.c_double(0), C.c_double(0)
    oracle.setvarcurvadv3d_(Q.dptr(v["mask"]), Q.dptr(arrs["mx"]), Q.dptr(arrs["my"]), Q.dptr(arrs["mz"]),
                            Q.dptr(arrs["b"]), Q.dptr(arrs["vx"]), Q.dptr(arrs["vy"]), Q.dptr(arrs["vz"]),
                            C.byref(bm), C.byref(um), Q.dref(B), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
    return {k: torch.tensor(_fill(g, a)) for k, a in arrs.items()}


class ThetaLoss(torch.autograd.Function):
    """The library's loss of a per-voxel angle field, with its adjoint gradient."""

    @staticmethod
    def forward(ctx, theta_fill, gpu, o, v, g, target, dt, ckpt):
        th = _to_ghost(g, theta_fill.detach().numpy())
        loss, gr = _run(gpu, o, v, g, th, target, dt, ckpt)
        ctx.save_for_backward(torch.tensor(_fill(g, gr)))
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (gr,) = ctx.saved_tensors
        return gout * gr, None, None, None, None, None, None, None


def test_adjoint_against_replica_and_fd(oracle, gpu, problem):
    g, v, o, dt, W, ctrl, hidden = problem
    coef = _coefficients(oracle, g, v)
    Wt = torch.tensor(W)
    n = g.ihi_fb - g.ilo_fb + 1
    shape = (n, n, n)
    # target: H(phi_T) of the hidden control grid, from the replica
    with torch.no_grad():
        _, Ht = replica_loss(g, v, coef["mx"], coef["my"], coef["mz"], coef["b"],
                             (coef["vx"], coef["vy"], coef["vz"]), (Wt @ torch.tensor(hidden)).reshape(shape),
                             torch.zeros(shape, dtype=torch.float64), dt)
    target = _to_ghost(g, Ht.numpy())
    # library adjoint through the autograd wrapper, composed with the interpolation
    c1 = torch.tensor(ctrl, requires_grad=True)
    th_vox = (Wt @ c1).reshape(shape)
    loss_lib = ThetaLoss.apply(th_vox, gpu, o, v, g, target, dt, 3)
    loss_lib.backward()
    g_lib = c1.grad.numpy().copy()
    # replica
    c2 = torch.tensor(ctrl, requires_grad=True)
    loss_rep, _ = replica_loss(g, v, coef["mx"], coef["my"], coef["mz"], coef["b"],
                               (coef["vx"], coef["vy"], coef["vz"]), (Wt @ c2).reshape(shape),
                               torch.tensor(_fill(g, target)), dt)
    loss_rep.backward()
    g_rep = c2.grad.numpy()
    assert abs(loss_lib.item() - loss_rep.item()) <= 1e-9 * max(1.0, abs(loss_rep.item()))
    scale = np.abs(g_rep).max()
    assert scale > 0
    assert np.abs(g_lib - g_rep).max() <= 1e-7 * scale, (np.abs(g_lib - g_rep).max(), scale)
    # central finite differences of the library's forward on the largest components
    h = 1e-6
    for c in np.argsort(-np.abs(g_lib))[:4]:
        lp = _run(gpu, o, v, g, _to_ghost(g, W @ np.where(np.arange(512) == c, ctrl + h, ctrl)), target, dt,
                  grad=False)[0]
        lm = _run(gpu, o, v, g, _to_ghost(g, W @ np.where(np.arange(512) == c, ctrl - h, ctrl)), target, dt,
                  grad=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g_lib[c]) <= 1e-5 * abs(g_lib[c]), (c, fd, g_lib[c])


def test_adjoint_checkpoint_independent(oracle, gpu, problem):
    g, v, o, dt, W, ctrl, hidden = problem
    theta = _to_ghost(g, W @ ctrl)
    target = _to_ghost(g, np.full(W.shape[0], 0.5))
    l1, g1 = _run(gpu, o, v, g, theta, target, dt, ckpt=1)
    l3, g3 = _run(gpu, o, v, g, theta, target, dt, ckpt=4)
    l6, g6 = _run(gpu, o, v, g, theta, target, dt, ckpt=STEPS)
    lf, _ = _run(gpu, o, v, g, theta, target, dt, grad=False)
    assert l1 == l3 == l6 == lf
    assert np.array_equal(g1, g3) and np.array_equal(g1, g6)
    assert np.abs(g1).max() > 0
