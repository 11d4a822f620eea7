"""The allocation-free volume entry point, for callers that cannot allocate
device memory while they run (a framework that reserved all of HBM for its
own pool allocator, or one that cannot take the device-wide synchronisation
of cudaFree).  It must return, through device pointers, exactly what the
allocating entry point and the oracle return for the same phi, call after
call (the fixed scratch array keeps the previous call's data)."""
import ctypes as C

import numpy as np
import pytest

import qssgpu as Q
from qss_cases import pack_case

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.qssgpu_volume_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_double, C.c_double, C.c_double,
                  C.c_double, C.c_void_p, C.c_void_p]
    return f


def test_volume_noalloc_matches_allocating_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    noalloc = _bind(gpu)
    for n, seed in ((24, 3), (40, 5)):  # two calls in a row, different boxes
        g, v = pack_case(oracle, n, seed=seed)
        phi = v["phi"]
        eps = 1.5 * g.dx[0]
        want = C.c_double(-1.0)
        gpu.qss3dvolumeregionphilessthanzero_(C.byref(want), Q.dptr(phi), *Q.gb_args(g), *Q.fb_args(g),
                                              Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]), Q.dref(eps))
        Q.check(gpu)
        # the oracle's restatement of qss3dVolumeRegionPhiLessThanZero (qss_util3d.f:288-358)
        ref = C.c_double(-2.0)
        oracle.qss3dvolumeregionphilessthanzero_(C.byref(ref), Q.dptr(phi), *Q.gb_args(g), *Q.fb_args(g),
                                                 Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]), Q.dref(eps))
        assert want.value == ref.value, (want.value, ref.value)
        d_phi = torch.from_numpy(phi).to("cuda")
        d_vol = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        gb = (C.c_int * 6)(g.ilo_gb, g.ihi_gb, g.jlo_gb, g.jhi_gb, g.klo_gb, g.khi_gb)
        ib = (C.c_int * 6)(g.ilo_fb, g.ihi_fb, g.jlo_fb, g.jhi_fb, g.klo_fb, g.khi_fb)
        rc = noalloc(d_phi.data_ptr(), gb, ib, g.dx[0], g.dx[1], g.dx[2], eps, d_vol.data_ptr(), None)
        torch.cuda.synchronize()
        Q.check(gpu)
        assert rc == 0
        got = d_vol.item()
        assert want.value > 0
        assert got == want.value, (got, want.value)  # bit for bit, the tolerance of every parity test


def test_volume_noalloc_rejects_boxes_beyond_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    noalloc = _bind(gpu)
    d = torch.zeros(1, dtype=torch.float64, device="cuda")
    gb = (C.c_int * 6)(0, 135, 0, 135, 0, 135)
    ib = (C.c_int * 6)(3, 132, 3, 132, 3, 132)  # 130^3 voxels > 2^21
    rc = noalloc(d.data_ptr(), gb, ib, 0.04, 0.04, 0.04, 0.06, d.data_ptr(), None)
    assert rc != 0
    msg = gpu.qssgpu_error_string().decode()
    gpu.qssgpu_clear_error()
    assert "scratch" in msg


def test_volume_noalloc_on_a_caller_stream_takes_no_device_memory(gpu, oracle):
    """On a stream of the caller's, after a first call that did the set-up,
    further calls leave the device's free memory unchanged and still return
    the allocating entry point's volume."""
    torch = pytest.importorskip("torch")
    noalloc = _bind(gpu)
    g, v = pack_case(oracle, 32, seed=9)
    phi = v["phi"]
    eps = 1.5 * g.dx[0]
    want = C.c_double(-1.0)
    gpu.qss3dvolumeregionphilessthanzero_(C.byref(want), Q.dptr(phi), *Q.gb_args(g), *Q.fb_args(g),
                                          Q.dref(g.dx[0]), Q.dref(g.dx[1]), Q.dref(g.dx[2]), Q.dref(eps))
    Q.check(gpu)
    gb = (C.c_int * 6)(g.ilo_gb, g.ihi_gb, g.jlo_gb, g.jhi_gb, g.klo_gb, g.khi_gb)
    ib = (C.c_int * 6)(g.ilo_fb, g.ihi_fb, g.jlo_fb, g.jhi_fb, g.klo_fb, g.khi_fb)
    d_phi = torch.from_numpy(phi).to("cuda")
    d_vol = torch.zeros(2, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert noalloc(d_phi.data_ptr(), gb, ib, g.dx[0], g.dx[1], g.dx[2], eps, d_vol.data_ptr(),
                   C.c_void_p(side.cuda_stream)) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert noalloc(d_phi.data_ptr(), gb, ib, g.dx[0], g.dx[1], g.dx[2], eps, d_vol[1:].data_ptr(),
                       C.c_void_p(side.cuda_stream)) == 0
    side.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    Q.check(gpu)
    assert free_after == free_before
    assert d_vol[0].item() == want.value and d_vol[1].item() == want.value
