"""Known-answer tests of the restated kernels (the oracle), from the
mathematics rather than from another implementation."""
import ctypes as C
import math

import numpy as np
import pytest

import qssgpu as Q


def _grid(lib, n):
    return Q.make_grid(lib, n)


def _coords(g):
    nx, ny, nz = (g.grid_dims_ghostbox[d] for d in range(3))
    z, y, x = np.meshgrid(*(np.arange(s) * g.dx[0] for s in (nz, ny, nx)), indexing="ij")
    return x, y, z


def _rhs_const(lib, name, g, phi, a, b):
    rhs = np.zeros_like(phi)
    h = C.c_double()
    getattr(lib, name)(Q.dptr(phi), Q.dref(a), Q.dref(b), C.byref(h), Q.dptr(rhs), *Q.gb_args(g),
                       *Q.fb_args(g), Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]))
    return rhs, h.value


def _fb(g, a):
    return a[g.klo_fb:g.khi_fb + 1, g.jlo_fb:g.jhi_fb + 1, g.ilo_fb:g.ihi_fb + 1]


@pytest.mark.parametrize("name", ["getrhs3d2ndconst_", "getrhs3d3rdconst_"])
def test_plane_moves_at_speed_a_with_no_curvature(oracle, name):
    g = _grid(oracle, 16)
    x, y, z = _coords(g)
    phi = (x - 0.31) * 0.6 + (y - 0.2) * 0.8  # unit normal, linear
    rhs, h = _rhs_const(oracle, name, g, phi, a=1.5, b=0.04)
    np.testing.assert_allclose(_fb(g, rhs), -1.5, atol=1e-12)  # -a|grad phi|, curvature 0
    assert h > 0


def test_sphere_curvature_term(oracle):
    """b*kappa|grad phi| of a sphere distance function is 2b/r (sum of the two
    principal curvatures); the const RHS with a below the tolerance leaves
    only this term."""
    g = _grid(oracle, 40)
    x, y, z = _coords(g)
    c = 0.12 + 20 * g.dx[0]
    r = np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2)
    phi = r - 0.4
    rhs, _ = _rhs_const(oracle, "getrhs3d2ndconst_", g, phi, a=0.0, b=1.0)
    band = np.abs(_fb(g, phi)) < 0.5 * g.dx[0]
    kappa = 2.0 / _fb(g, r)[band]
    np.testing.assert_allclose(_fb(g, rhs)[band], kappa, rtol=0.02)


def test_linear_extrapolation_is_exact_for_outward_growing_data(oracle):
    """The extrapolation continues |phi| outward with the boundary slope, so a
    positive function growing linearly away from the box centre (an L1
    distance) is reproduced in every ghost point, edges and corners included."""
    g = _grid(oracle, 12)
    x, y, z = _coords(g)
    c = (g.ilo_fb + g.ihi_fb) / 2 * g.dx[0] + 0.013
    phi = 2.0 + np.abs(x - c) + np.abs(y - c) + np.abs(z - c)
    a = phi.copy()
    a[...] = -7.0
    _fb(g, a)[...] = _fb(g, phi)
    oracle.signedLinearExtrapolationBCqss(Q.dptr(a), C.byref(g), 9)
    np.testing.assert_allclose(a, phi, atol=1e-12)


def test_reinit_keeps_a_distance_function(oracle):
    g = _grid(oracle, 24)
    x, y, z = _coords(g)
    c = 0.12 + 12 * g.dx[0]
    phi = np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) - 0.25
    a = phi.copy()
    o = Q.default_options(oracle)
    oracle.reinitializeSubcellFix3d(Q.dptr(a), C.byref(g), C.byref(o))
    band = np.abs(_fb(g, phi)) < 3 * g.dx[0]
    assert np.max(np.abs(_fb(g, a)[band] - _fb(g, phi)[band])) < 0.5 * g.dx[0]


def test_union_find_labels_are_component_maxima(oracle):
    g = _grid(oracle, 6)
    v = Q.Volume(g)
    b = v["phi_bin"]
    b[...] = 0
    b[3, 3, 3] = b[4, 4, 4] = 1      # corner contact: one component
    b[5, 5, 9] = 1                   # isolated
    b[0, 0, 0] = 1                   # the index-0 voxel is labelled 0 like background
    oracle.findConnectivity3d(C.byref(v.p), C.byref(g))
    lab = v["connectivity"]
    flat = lambda k, j, i: i + b.shape[2] * (j + b.shape[1] * k)
    assert lab[3, 3, 3] == lab[4, 4, 4] == flat(4, 4, 4)
    assert lab[5, 5, 9] == flat(5, 5, 9)
    assert lab[0, 0, 0] == 0
    assert int(lab.sum()) == 2 * flat(4, 4, 4) + flat(5, 5, 9)


@pytest.mark.parametrize("density", [0.2, 0.35, 0.6])
def test_union_find_matches_scipy_components(oracle, density):
    """Labels are independent of the order of the unions: on random binaries
    every 26-connected component (scipy's labelling, computed without any
    union-find) carries its largest linear index, background 0."""
    ndimage = pytest.importorskip("scipy.ndimage")
    g = _grid(oracle, (13, 9, 11))
    v = Q.Volume(g)
    rng = np.random.default_rng(int(100 * density))
    b = (rng.random(v.shape) < density).astype(np.uint8)
    v["phi_bin"][...] = b
    oracle.findConnectivity3d(C.byref(v.p), C.byref(g))
    comp, n = ndimage.label(b, structure=np.ones((3, 3, 3), int))
    flat = np.arange(b.size).reshape(b.shape)
    top = np.zeros(n + 1, np.int64)
    np.maximum.at(top, comp.ravel(), flat.ravel())
    want = np.where(comp > 0, top[comp], 0)
    assert np.array_equal(v["connectivity"], want)


def test_portable_sine_is_accurate(oracle):
    xs = np.linspace(-3.3, 3.3, 20001)
    s = np.array([oracle.oracle_portable_sin(float(x)) for x in xs])
    c = np.array([oracle.oracle_portable_cos(float(x)) for x in xs])
    ulp_s = np.spacing(np.abs(np.sin(xs))) + 1e-300
    assert np.max(np.abs(s - np.sin(xs)) / ulp_s) <= 2.0
    assert np.max(np.abs(c - np.cos(xs)) / (np.spacing(np.abs(np.cos(xs))) + 1e-300)) <= 2.0
