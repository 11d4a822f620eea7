"""Parity over the workloads' own lengths, against the oracle, bit for bit.

* 512^3 grain pack (lognormal radii mu = ln 8, sigma = 0.3 voxels, seed 512,
  porosity 0.30, contact angle 40 degrees; WENO5 + TVD-RK3, variable
  coefficients): one whole constCurvModel3d call, as the benchmark's
  end-to-end call makes it -- about 13 inner steps, the trapping pass, the
  three reinitialisations (mask_w, mask_nw, phi), the max-norm and the
  volumes -- every array of the volume and the returned time compared.  The
  oracle runs the reference's 16-thread z-slab split on 16 host threads and
  the GB300 path the same 16 slabs (the CFL step depends on the split,
  constCurvModel3d.c:105-149).
* 256^3 drainage then imbibition (non-overlapping polydisperse pack, seed 1,
  radii 4-12 voxels, porosity 0.38; WENO5 + TVD-RK3, contact angle 10
  degrees; 40 curvature steps each way between 0.02 and 0.5 per voxel): the
  GB300 library drives the whole ladder step by step through the exported
  C API (the loop body of drain_model3d.c:102-163 and imbibe_model3d.c:99-159);
  at steps 1, 10, 20, 30 and 40 of drainage and 1, 20 and 40 of imbibition
  the oracle starts from the GB300 state before the step, runs the same step,
  and every array after it is compared.  The per-step level sets of the
  step-by-step run equal the data_step files of one drain_model3d /
  imbibe_model3d call on the device."""
import ctypes as C
import gzip
import os

import numpy as np
import pytest

import qssgpu as Q
import synthetic as S
from qss_cases import clone, diff_arrays, in_tmpdir, options, prepare_model

pytestmark = pytest.mark.gpu

THREADS = 16


def _oracle_options(oracle, g, o):
    """A copy of o for the oracle: same fields, the oracle's own function
    pointers (setSpaceDerivFunc, and the defaults of the other two)."""
    oo = Q.default_options(oracle)
    fns = (oo.reinit_func, oo.extrapol_func)
    C.pointer(oo)[0] = o
    oo.reinit_func, oo.extrapol_func = fns
    oracle.setSpaceDerivFunc(C.byref(g), C.byref(oo))
    return oo


def _with_slabs(gpu, oracle, fn):
    gpu.qssgpu_set_slabs(THREADS)
    oracle.oracle_set_threads(THREADS)
    try:
        return fn()
    finally:
        gpu.qssgpu_set_slabs(1)
        oracle.oracle_set_threads(1)


def test_model_call_512_every_array(gpu, oracle):
    n = 512
    g = Q.make_grid(oracle, n)
    mask = S.lognormal(n, mu=np.log(8.0), sigma=0.3, porosity=0.30, seed=512).mask()
    phi0 = S.initial_phi(mask, n)
    vg = Q.Volume(g)
    vg["mask"][...] = mask
    vg["phi"][...] = phi0
    del phi0
    og = options(gpu, theta_deg=40.0, space=5, time=3, a=1.25, b=0.04)
    prepare_model(gpu, og, vg, og.a)
    Q.check(gpu)
    dt_est = 0.5 / (og.b_max_over_dx + og.max_U_over_dx)
    og.tplot = 13 * dt_est * 0.999
    og.tmax = og.tplot * 0.5
    og.use_satn_stop = 0
    vo = clone(vg)
    oo = _oracle_options(oracle, g, og)

    def run():
        def go(d):
            fp = Q.libc_fopen("out")
            try:
                tg = gpu.constCurvModel3d(C.byref(og), C.byref(vg.p), C.byref(g), fp)
                Q.check(gpu)
                steps, outer = C.c_longlong(0), C.c_longlong(0)
                gpu.qssgpu_call_stats(C.byref(vg.p), C.byref(g), C.byref(steps), C.byref(outer))
                gpu.qssgpu_release(C.byref(vg.p))
                to = oracle.constCurvModel3d(C.byref(oo), C.byref(vo.p), C.byref(g), fp)
            finally:
                Q.libc_fclose(fp)
            return tg, to, steps.value

        return in_tmpdir(go)

    tg, to, steps = _with_slabs(gpu, oracle, run)
    assert steps >= 10
    assert tg == to and tg > 0
    assert diff_arrays(vg, vo) == {}
    assert not np.array_equal(vg["phi"], vg["phi_prev"])


def _ladder_step(lib, o, v, g, a0, drain, fp):
    """The body of the curvature ladder (drain_model3d.c:104-162,
    imbibe_model3d.c:101-158) for a contact angle > 0, without the file.
    Returns the next a0, or None when constCurvModel3d returned -1."""
    gp = C.byref(g)
    bm, um = C.c_double(0), C.c_double(0)
    lib.setvarcurvadv3d_(Q.dptr(v["mask"]), Q.dptr(v["mask_x"]), Q.dptr(v["mask_y"]), Q.dptr(v["mask_z"]),
                         Q.dptr(v["curvature_coeff"]), Q.dptr(v["external_velocity_x"]),
                         Q.dptr(v["external_velocity_y"]), Q.dptr(v["external_velocity_z"]), C.byref(bm),
                         C.byref(um), Q.dref(o.b), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
    o.b_max_over_dx, o.max_U_over_dx = bm.value, um.value
    if not drain:
        o.conserve_imbibe = 1
    lib.setvarnorm3d_(Q.dptr(v["mask"]), Q.dptr(v["mask_x"]), Q.dptr(v["mask_y"]), Q.dptr(v["mask_z"]),
                      Q.dptr(v["normal_velocity"]), Q.dref(a0), Q.dref(o.theta), *Q.gb_args(g), *Q.fb_args(g),
                      Q.dref(g.dx[0]))
    if o.check_connectivity:
        lib.trapComponents_mask(C.byref(v.p), gp, C.byref(o))
    t = lib.constCurvModel3d(C.byref(o), C.byref(v.p), gp, fp)
    if t == -1:
        return None
    da = o.b * o.dc
    a0 = a0 + da if drain else a0 - da
    phi = v["phi"]
    if o.reservoir_inlet:  # IMPOSE_MIN (qss_macros.h:239-246)
        ext = v["phi_extra"]
        phi[...] = np.where(phi < ext, phi, ext)
    mask = v["mask"]  # IMPOSE_MASK (qss_macros.h:79-86)
    phi[...] = np.where(mask > phi, mask, phi)
    return a0


def _device_ladder_files(gpu, g, v0, o, imbibe_a, imbibe_min):
    """One drain_model3d call then one imbibe_model3d call on the device:
    the data_step files, decompressed."""
    v = clone(v0)

    def go(d):
        fp = Q.libc_fopen("out")
        try:
            gpu.drain_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
            for f in os.listdir(d):
                if f.startswith("data_step"):
                    os.rename(os.path.join(d, f), os.path.join(d, "drain_" + f))
            o.a, o.amin = imbibe_a, imbibe_min
            gpu.imbibe_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
        finally:
            Q.libc_fclose(fp)
        files = {}
        for f in os.listdir(d):
            if "data_step" in f:
                with gzip.open(os.path.join(d, f), "rb") as fh:
                    files[f[:-3] if f.endswith(".gz") else f] = fh.read()
        return files

    files = in_tmpdir(go)
    gpu.qssgpu_release(C.byref(v.p))
    return files


def test_drain_imbibe_256_sampled_steps(gpu, oracle):
    n, steps = 256, 40
    g = Q.make_grid(oracle, n)
    mask = S.rsa(n, rmin=4.0, rmax=12.0, porosity=0.38, seed=1).mask()
    da = (12.5 - 0.5) / 39  # 0.02 -> 0.5 per voxel in 40 steps at dx = 0.04
    kw = dict(theta_deg=10.0, space=5, time=3, tmax=0.01, tplot=0.005, a=0.5, b=0.04, dc=da / 0.04)
    v = Q.Volume(g)
    v["mask"][...] = mask
    v["phi"][...] = S.initial_phi(mask, n)
    o = options(gpu, **kw)
    step_a = o.b * o.dc
    # the ladders' curvatures by the same repeated additions as the drivers'
    a_drain = [o.a]
    for _ in range(steps - 1):
        a_drain.append(a_drain[-1] + step_a)
    a_imbibe = [a_drain[-1]]
    for _ in range(steps - 1):
        a_imbibe.append(a_imbibe[-1] - step_a)
    o.amax = a_drain[-1] + step_a
    o_dev = _copy(o)
    dev_files = _with_slabs(gpu, oracle, lambda: _device_ladder_files(gpu, g, v, o_dev, a_imbibe[0],
                                                                      a_imbibe[-1] - step_a))
    Q.check(gpu)
    sample = {"drain": {1, 10, 20, 30, 40}, "imbibe": {1, 20, 40}}
    checked, ran = [], {"drain": 0, "imbibe": 0}

    def run():
        def go(d):
            fp = Q.libc_fopen("out")
            try:
                for phase, drain, a_list in (("drain", True, a_drain), ("imbibe", False, a_imbibe)):
                    oo = _copy(o)
                    # the driver's set-up only: a ladder whose loop does not run
                    if drain:
                        oo.amax = oo.a
                        gpu.drain_model3d(C.byref(oo), C.byref(v.p), C.byref(g), fp)
                    else:
                        oo.a = oo.amin = a_list[0]
                        gpu.imbibe_model3d(C.byref(oo), C.byref(v.p), C.byref(g), fp)
                    Q.check(gpu)
                    for step in range(1, steps + 1):
                        a0 = a_list[step - 1]
                        snap = (clone(v), _copy(oo)) if step in sample[phase] else None
                        a_next = _ladder_step(gpu, oo, v, g, a0, drain, fp)
                        Q.check(gpu)
                        name = ("drain_" if drain else "") + f"data_step_{step}"
                        if a_next is None:  # constCurvModel3d returned -1: the ladder stops here
                            assert name not in dev_files
                            break
                        ran[phase] += 1
                        assert a_next == (a_list[step] if step < steps else a_list[-1] + (step_a if drain else -step_a))
                        assert v["phi"].tobytes() == dev_files[name][12:], (phase, step)
                        if snap is not None:
                            vo, o_snap = snap
                            oo_o = _oracle_options(oracle, g, o_snap)
                            a_o = _ladder_step(oracle, oo_o, vo, g, a0, drain, fp)
                            assert a_o == a_next
                            assert diff_arrays(v, vo) == {}, (phase, step)
                            checked.append((phase, step))
                            del vo
            finally:
                Q.libc_fclose(fp)

        in_tmpdir(go)

    _with_slabs(gpu, oracle, run)
    # every step the device ladders wrote was reproduced step by step
    assert ran["drain"] + ran["imbibe"] == len(dev_files)
    assert ("drain", 1) in checked and ("imbibe", 1) in checked
    assert ran["drain"] >= 10


def _copy(o):
    c = Q.Options()
    C.pointer(c)[0] = o
    return c
