"""Golden cases of the level-set path: seeded inputs, one call of a C entry
point, SHA-256 of every output array.  Shared by tests/golden/make_golden.py
(reference C drivers) and the tests (oracle and GB300 library)."""
import ctypes as C
import gzip
import hashlib
import os

import numpy as np

import qssgpu as Q
from qss_cases import in_tmpdir, options, pack_case, prepare_model

CASES = {
    "drain_eno2_rk2_theta0_n20": dict(kind="drain", n=20, seed=11, theta=0, space=2, time=2, a=1.2,
                                      steps=3, tplot=0.02, tmax=0.05),
    "drain_weno5_rk3_theta40_n18": dict(kind="drain", n=18, seed=12, theta=40, space=5, time=3, a=1.2,
                                        steps=2, tplot=0.02, tmax=0.04),
    "drain_imbibe_eno3_theta10_n18_t3": dict(kind="drain_imbibe", n=18, seed=13, theta=10, space=3, time=3,
                                             a=1.2, steps=2, tplot=0.02, tmax=0.04, threads=3),
    "model_weno5_rk3_theta30_n16": dict(kind="model", n=16, seed=14, theta=30, space=5, time=3, a=1.25,
                                        tplot=0.015, tmax=0.03),
    "model_eno2_rk1_theta0_n16_t2": dict(kind="model", n=16, seed=15, theta=0, space=2, time=1, a=1.25,
                                         tplot=0.015, tmax=0.03, threads=2),
    "trap_center_n20": dict(kind="trap", n=20, seed=16, center=1),
    "reinit_mask_n20": dict(kind="reinit", n=20, seed=17),
}

SKIP = ("theta", "overlap")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def inputs(lib, case):
    g, v = pack_case(lib, case["n"], seed=case["seed"])
    return g, v


def run_case(lib, case):
    g, v = inputs(lib, case)
    rec = {"inputs": {k: sha(v[k]) for k in ("mask", "phi")}, "scalars": {}, "files": {}}
    kind = case["kind"]
    o = options(lib, case.get("theta", 0), case.get("space", 2), case.get("time", 2),
                tmax=case.get("tmax", 0.05), tplot=case.get("tplot", 0.02), a=case.get("a", 1.2))
    if kind in ("drain", "drain_imbibe"):
        o.amax = case["a"] + (case["steps"] - 0.5) * o.b * o.dc
        o.amin = case["a"] - 0.5 * o.b * o.dc

        def go(d):
            fp = Q.libc_fopen("out")
            lib.drain_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
            if kind == "drain_imbibe":
                o.a = case["a"] + case["steps"] * o.b * o.dc
                lib.imbibe_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
            Q.libc_fclose(fp)
            files = {}
            for f in sorted(os.listdir(d)):
                if f.startswith("data_step"):
                    with gzip.open(os.path.join(d, f), "rb") as fh:
                        files[f] = hashlib.sha256(fh.read()).hexdigest()
            return files

        rec["files"] = in_tmpdir(go)
    elif kind == "model":
        prepare_model(lib, o, v, case["a"])
        var = case["theta"] > 0

        def go(d):
            fp = Q.libc_fopen("out")  # the reference writes to fp_out unconditionally
            try:
                if var:
                    return lib.constCurvModel3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
                return lib.constCurvModel3dNoVar(C.byref(o), C.byref(v.p), C.byref(g), fp, case["a"])
            finally:
                Q.libc_fclose(fp)

        rec["scalars"]["t"] = float(in_tmpdir(go)).hex()
    elif kind == "trap":
        o.center_inlet = case["center"]
        lib.getMainInd_new(C.byref(o), C.byref(v.p), C.byref(g))
        lib.initializeDisconnectedMasks(v["mask_nw"].ctypes.data_as(Q.c_double_p), C.byref(g))
        v["phi"][...] = np.maximum(0.04 * np.sin(np.arange(v["phi"].size).reshape(v.shape) * 0.37), v["mask"])
        rec["inputs"]["phi"] = sha(v["phi"])
        lib.trapComponents_mask(C.byref(v.p), C.byref(g), C.byref(o))
    elif kind == "reinit":
        lib.reinitializeSubcellFix3d(Q.dptr(v["mask"]), C.byref(g), C.byref(o))
    rec["scalars"]["b_max_over_dx"] = float(o.b_max_over_dx).hex()
    rec["scalars"]["max_U_over_dx"] = float(o.max_U_over_dx).hex()
    rec["arrays"] = {k: sha(a) for k, a in v.arrays.items() if k not in SKIP}
    return rec
