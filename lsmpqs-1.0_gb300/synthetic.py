"""Seeded synthetic grain packs and initial level sets for the lsmpqs path.

No rock images travel with this project, so every workload is a seeded sphere
pack on the reference's own grid layout (3 ghost layers, dx = 0.04, fill box
starting at x = 3*dx, as written by the reference's createMaskUBC tool):

* ``mask`` is the solid level set, positive inside grains and negative in the
  pore space: the maximum over grains of ``r - |x - c|`` (the reference's
  createIntersectionOfSpheres with inside_flag >= 0), evaluated within a
  cut-off distance of each grain and clamped below at ``-cutoff`` elsewhere;
* ``phi0`` follows the reference's createInitFromMask tool: a sphere of
  radius 0.7*L centred 0.7*R before the inlet face (non-wetting fluid
  entering from x = 0), then ``max(mask, phi)``.

Pack generators (porosity = fraction of fill-box voxels with mask < 0):
  overlapping(n, radius, porosity, seed)         centres uniform, fixed radius
  lognormal(n, mu, sigma, porosity, seed)        overlapping, radii lognormal (voxels)
  rsa(n, rmin, rmax, porosity, seed, attempts)   non-overlapping random sequential
                                                 addition with a fixed attempt budget,
                                                 then uniform dilation to the porosity
"""
from __future__ import annotations

import math

import numpy as np

DX = 0.04
NG = 3


def grid_coords(n):
    """Physical coordinates of the ghost-box points along each axis."""
    if np.isscalar(n):
        n = (int(n),) * 3
    return [np.arange(n[d] + 2 * NG, dtype=np.float64) * DX for d in range(3)]


class Pack:
    def __init__(self, n, centers_vox, radii_vox):
        if np.isscalar(n):
            n = (int(n),) * 3
        self.n = tuple(n)
        self.c = np.asarray(centers_vox, dtype=np.float64).reshape(-1, 3)
        self.r = np.asarray(radii_vox, dtype=np.float64).reshape(-1)

    def mask(self, cutoff_vox: float = 6.0) -> np.ndarray:
        """Ghost-box array (nz, ny, nx) of max over grains of (r - |x - c|)*dx."""
        nx, ny, nz = (s + 2 * NG for s in self.n)
        m = np.full((nz, ny, nx), -cutoff_vox * DX, dtype=np.float64)
        xs = np.arange(nx, dtype=np.float64)
        ys = np.arange(ny, dtype=np.float64)
        zs = np.arange(nz, dtype=np.float64)
        for (cx, cy, cz), r in zip(self.c, self.r):
            R = r + cutoff_vox
            i0, i1 = max(0, int(math.floor(cx - R))), min(nx, int(math.ceil(cx + R)) + 1)
            j0, j1 = max(0, int(math.floor(cy - R))), min(ny, int(math.ceil(cy + R)) + 1)
            k0, k1 = max(0, int(math.floor(cz - R))), min(nz, int(math.ceil(cz + R)) + 1)
            if i0 >= i1 or j0 >= j1 or k0 >= k1:
                continue
            dz = (zs[k0:k1] - cz)[:, None, None]
            dy = (ys[j0:j1] - cy)[None, :, None]
            dxv = (xs[i0:i1] - cx)[None, None, :]
            d = (r - np.sqrt(dz * dz + dy * dy + dxv * dxv)) * DX
            sub = m[k0:k1, j0:j1, i0:i1]
            np.maximum(sub, d, out=sub)
        return m


def _fb_solid_fraction(n, c, r):
    p = Pack(n, c, r)
    m = p.mask(cutoff_vox=1.0)
    fb = m[NG:-NG, NG:-NG, NG:-NG]
    return float(np.mean(fb >= 0))


def _add_until(n, rng, porosity, radius_fn, batch=16):
    """Adds overlapping grains (centres uniform in the fill box) until the pore
    fraction of the fill box drops to `porosity`; the solid set is tracked
    incrementally on a boolean grid."""
    if np.isscalar(n):
        n = (int(n),) * 3
    nx, ny, nz = n
    solid = np.zeros((nz, ny, nx), dtype=bool)
    total = solid.size
    count = 0
    centers, radii = [], []
    target = (1.0 - porosity) * total
    xs, ys, zs = np.arange(nx) + NG, np.arange(ny) + NG, np.arange(nz) + NG
    while count < target:
        c = np.array([rng.uniform(NG, NG + nx - 1), rng.uniform(NG, NG + ny - 1), rng.uniform(NG, NG + nz - 1)])
        r = float(radius_fn(rng))
        i0, i1 = max(0, int(c[0] - r) - NG), min(nx, int(c[0] + r) + 2 - NG)
        j0, j1 = max(0, int(c[1] - r) - NG), min(ny, int(c[1] + r) + 2 - NG)
        k0, k1 = max(0, int(c[2] - r) - NG), min(nz, int(c[2] + r) + 2 - NG)
        dz = (zs[k0:k1] - c[2])[:, None, None]
        dy = (ys[j0:j1] - c[1])[None, :, None]
        dxv = (xs[i0:i1] - c[0])[None, None, :]
        inside = (r - np.sqrt(dz * dz + dy * dy + dxv * dxv)) >= 0
        sub = solid[k0:k1, j0:j1, i0:i1]
        new = inside & ~sub
        count += int(new.sum())
        sub |= inside
        centers.append(c)
        radii.append(r)
    return Pack(n, centers, radii)


def overlapping(n, radius_vox=5.0, porosity=0.35, seed=0) -> Pack:
    rng = np.random.default_rng(seed)
    return _add_until(n, rng, porosity, lambda g: radius_vox)


def lognormal(n, mu=math.log(8.0), sigma=0.3, porosity=0.30, seed=512) -> Pack:
    rng = np.random.default_rng(seed)
    return _add_until(n, rng, porosity, lambda g: g.lognormal(mu, sigma))


def rsa(n, rmin=4.0, rmax=12.0, porosity=0.38, seed=1, attempts=20000) -> Pack:
    """Random sequential addition of non-overlapping grains, radii U[rmin,rmax],
    with a fixed attempt budget; the radii are then scaled by one common
    factor (bisection) so that the pore fraction reaches `porosity` (grains
    may then overlap slightly)."""
    if np.isscalar(n):
        n = (int(n),) * 3
    rng = np.random.default_rng(seed)
    lo = np.array([NG, NG, NG], dtype=np.float64)
    hi = lo + np.array(n, dtype=np.float64) - 1
    C, R = [], []
    for _ in range(attempts):
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(lo, hi)
        if C:
            d = np.linalg.norm(np.asarray(C) - c, axis=1)
            if np.any(d < np.asarray(R) + r):
                continue
        C.append(c)
        R.append(r)
    C, R = np.asarray(C), np.asarray(R)
    a, b = 0.5, 3.0
    for _ in range(30):
        s = 0.5 * (a + b)
        if 1.0 - _fb_solid_fraction(n, C, R * s) > porosity:
            a = s
        else:
            b = s
    return Pack(n, C, R * b)


def initial_phi(mask: np.ndarray, n) -> np.ndarray:
    """createInitFromMask: non-wetting sphere at the inlet, then max(mask, phi)."""
    if np.isscalar(n):
        n = (int(n),) * 3
    x_lo = [NG * DX] * 3
    x_hi = [x_lo[d] + n[d] * DX for d in range(3)]
    radius = 0.7 * (x_hi[0] - x_lo[0])
    cy = 0.5 * (x_lo[1] + x_hi[1])
    cx = x_lo[0] - radius * 0.7
    cz = 0.5 * (x_lo[2] + x_hi[2])
    xs, ys, zs = grid_coords(n)
    d = np.sqrt((zs[:, None, None] - cz) ** 2 + (ys[None, :, None] - cy) ** 2 + (xs[None, None, :] - cx) ** 2)
    phi = d - radius
    return np.maximum(mask, phi)


def porosity_of(mask: np.ndarray) -> float:
    fb = mask[NG:-NG, NG:-NG, NG:-NG]
    return float(np.mean(fb < 0))
