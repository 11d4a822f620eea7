"""Batched mode (qssgpu_ladder_batch): several volumes of different sizes,
contact angles, schemes and curvature ladders advanced at once end exactly
as single drain_model3d / imbibe_model3d calls on the plain GPU path leave
them -- every array and every per-step file bit for bit."""
import ctypes as C
import gzip
import os

import pytest

import qssgpu as Q
from qss_cases import clone, diff_arrays, in_tmpdir, options, pack_case

pytestmark = pytest.mark.gpu

# (fill-box side, seed, contact angle in degrees, space order, time order, first a, ladder steps)
VOLUMES = [(20, 11, 0.0, 2, 2, 1.20, 2), (24, 12, 10.0, 5, 3, 1.25, 3), (28, 13, 25.0, 5, 3, 1.10, 2),
           (22, 14, 40.0, 3, 3, 1.30, 2), (26, 15, 55.0, 5, 3, 1.15, 3), (21, 16, 33.0, 2, 2, 1.22, 1)]


def _volume(oracle, lib, side, seed, theta, space, time, a, steps):
    g, v = pack_case(oracle, side, seed=seed, porosity=0.35 + 0.01 * (seed % 5))
    o = options(lib, theta_deg=theta, space=space, time=time, tmax=0.05, tplot=0.02, a=a, amin=a - 0.05)
    o.amax = a + (steps - 0.5) * o.b * o.dc
    return g, v, o


def _step_files(d, prefix):
    out = {}
    for f in sorted(os.listdir(d)):
        if f.startswith(prefix + "data_step"):
            with gzip.open(os.path.join(d, f), "rb") as fh:
                out[f[len(prefix):]] = fh.read()
    return out


@pytest.mark.parametrize("drain,workers", [(1, 0), (1, 2), (0, 3)])
def test_batch_equals_single_volume_path(gpu, oracle, drain, workers):
    vols = [_volume(oracle, gpu, *spec) for spec in VOLUMES]
    plain = []
    for g, v, o in vols:
        w = clone(v)
        oo = options(gpu)
        C.memmove(C.byref(oo), C.byref(o), C.sizeof(Q.Options))

        def go(d, w=w, oo=oo, g=g):
            fp = Q.libc_fopen("out")
            try:
                if drain:
                    gpu.drain_model3d(C.byref(oo), C.byref(w.p), C.byref(g), fp)
                else:
                    gpu.imbibe_model3d(C.byref(oo), C.byref(w.p), C.byref(g), fp)
            finally:
                Q.libc_fclose(fp)
            return _step_files(d, "")

        files = in_tmpdir(go)
        Q.check(gpu)
        plain.append((w, oo, files))
        gpu.qssgpu_release(C.byref(w.p))

    n = len(vols)
    batch = [clone(v) for _, v, _ in vols]
    opts = (C.POINTER(Q.Options) * n)(*[C.pointer(o) for _, _, o in vols])
    arrs = (C.POINTER(Q.QSSDataArrays) * n)(*[C.pointer(b.p) for b in batch])
    grids = (C.POINTER(Q.Grid) * n)(*[C.pointer(g) for g, _, _ in vols])
    prefixes = (C.c_char_p * n)(*[f"v{i}_".encode() for i in range(n)])

    def run(d):
        fps = (C.c_void_p * n)(*[Q.libc_fopen(f"out{i}") for i in range(n)])
        try:
            rc = gpu.qssgpu_ladder_batch(drain, n, opts, arrs, grids, fps, prefixes, workers)
        finally:
            for f in fps:
                Q.libc_fclose(f)
        return rc, [_step_files(d, f"v{i}_") for i in range(n)]

    rc, bfiles = in_tmpdir(run)
    assert rc == 0, gpu.qssgpu_error_string()
    Q.check(gpu)
    for i, (w, oo, files) in enumerate(plain):
        assert diff_arrays(batch[i], w) == {}, i
        assert bfiles[i] == files, i
        # the options the ladder updates (coefficient bounds, inlet indices) agree too
        _, _, o = vols[i]
        for f in ("b_max_over_dx", "max_U_over_dx", "overlap", "phi_nw_ind", "phi_w_ind", "conserve_imbibe"):
            assert getattr(o, f) == getattr(oo, f), (i, f)
    for b in batch:
        gpu.qssgpu_release(C.byref(b.p))


def test_batch_rejects_shared_arrays(gpu, oracle):
    g, v, o = _volume(oracle, gpu, *VOLUMES[0])
    o2 = options(gpu)
    opts = (C.POINTER(Q.Options) * 2)(C.pointer(o), C.pointer(o2))
    arrs = (C.POINTER(Q.QSSDataArrays) * 2)(C.pointer(v.p), C.pointer(v.p))
    grids = (C.POINTER(Q.Grid) * 2)(C.pointer(g), C.pointer(g))
    rc = gpu.qssgpu_ladder_batch(1, 2, opts, arrs, grids, None, None, 0)
    assert rc == 2 and gpu.qssgpu_last_error() == 3
    gpu.qssgpu_clear_error()
