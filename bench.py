"""Benchmark of the quasi-static level-set inner loop on GB300.

Workload (the 512^3 throughput configuration): a seeded grain pack on a
512^3 fill box (3 ghost layers, dx = 0.04), grain radii lognormal
(mu = ln 8, sigma = 0.3) voxels, porosity 0.30, contact angle 40 degrees,
so the variable-coefficient model runs with HJ-WENO5 in space and TVD-RK3 in
time.  One benchmark step is one full inner pseudo-time step of
constCurvModel3d: CFL estimate, three fused RHS + RK stage kernels, the
ghost-layer boundary condition after each stage and the three mask
impositions, over every fill-box voxel.  Metric: voxel-step updates per
second (fill-box voxels x inner steps / time).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--n 512]

--impl gb300 (default) times the GB300 library: `value` with the arrays
resident in HBM (CUDA events on the library's stream), `e2e` through the
reference's C entry point constCurvModel3d with host arrays (host<->device
copies, trapping, reinitialisation and the volume integrals included).
--impl reference times the reference algorithm on the host cores (the CPU
oracle: the reference's drivers and restated kernels, OpenMP over all
cores) on a bounded z-slab of the same workload.
For N > 1 (torchrun) every rank advances its own independent volume:
the path has no exchange between volumes ("replicas only").
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lsmpqs-1.0_gb300")
sys.path.insert(0, PKG)

import qssgpu as Q  # noqa: E402
import synthetic as S  # noqa: E402

METRIC = "voxel-step updates/s (512^3 FP64, WENO5 + TVD-RK3)"
UNIT = "voxel-steps/s"
THETA_DEG = 40.0
SEED = 512


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks for independent replicas (gloo on the host)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def make_workload(n: int, nz: int | None = None):
    """Mask and initial level set of the grain pack (numpy, ghost box)."""
    nz = nz or n
    pack = S.lognormal((n, n, nz), mu=math.log(8.0), sigma=0.3, porosity=0.30, seed=SEED)
    mask = pack.mask()
    phi = S.initial_phi(mask, (n, n, nz))
    return mask, phi


def set_options(lib, o):
    o.theta = THETA_DEG * 3.14159 / 180
    o.order_space_accur = 5
    o.order_time_accur = 3
    o.a = 0.05 / 0.04
    o.b = 0.04
    o.check_connectivity = 1


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"qss_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class ResultLine:
    """Keeps fd 1 for the one JSON result line.

    The library mirrors the reference's printf progress lines
    (constCurvModel3d.c:316-323, drain_model3d.c:104); libc buffers them
    separately from Python's sys.stdout and flushes them at exit, after any
    line printed from Python.  While the arms run, fd 1 points at fd 2, so
    every C and Python write goes to stderr; emit() flushes both buffers,
    restores fd 1 and prints the line as the last write to stdout."""

    def __init__(self):
        self._libc = C.CDLL(None)
        sys.stdout.flush()
        self._saved = os.dup(1)
        os.dup2(2, 1)

    def _flush(self):
        self._libc.fflush(None)
        sys.stdout.flush()
        sys.stderr.flush()

    def emit(self, line: dict | None):
        self._flush()
        os.dup2(self._saved, 1)
        os.close(self._saved)
        self._saved = None
        if line is not None:
            print(json.dumps(line), flush=True)

    def close(self):
        if self._saved is not None:
            self.emit(None)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# Algorithmic FP64 operations per voxel (+, -, *, /, sqrt each count one;
# max/min of squares are integer compares) of each stage kernel:
#   fused stage kernel: 3 x (16 differences/scalings + 2 x 75 WENO5 side)
#     + 10 Godunov + 5 advection + 72 curvature + 2 sums + 5 RK combination;
#   one WENO5 axis pass with shared sub-expressions: 9 per face (difference,
#     scaling, square, 6 scaled copies) + 35 per centre (smoothness terms)
#     + 2 eps + 2 x 26 per side (3 candidates, weights, combination);
#   combine: 10 Godunov + 5 advection + 72 curvature + 2 sums + 5 RK.
FLOP_PER_VOXEL = {0: 3 * (16 + 2 * 75) + 10 + 5 + 72 + 2 + 5,
                  1: 9 + 35 + 2 + 2 * 26, 2: 9 + 35 + 2 + 2 * 26, 3: 9 + 35 + 2 + 2 * 26,
                  4: 10 + 5 + 72 + 2 + 5}
KERNEL_NAME = {0: "k_stage<WENO5,var> (fused RHS + TVD-RK stage)",
               1: "k_weno_tile<0> (WENO5 x-pass, {} tiles, shared sub-expressions)",
               2: "k_weno_tile<1> (WENO5 y-pass, {} tiles, shared sub-expressions)",
               3: "k_weno_tile<2> (WENO5 z-pass, {} tiles, shared sub-expressions)",
               4: "k_weno_combine (Godunov + advection + curvature + TVD-RK)"}
# the window forms (--axis-variant 0/1/2) run k_weno_axis<axis> instead
WINDOW_NAME = {1: "k_weno_axis<0> (WENO5 x-pass, sliding window)",
               2: "k_weno_axis<1> (WENO5 y-pass, sliding window)",
               3: "k_weno_axis<2> (WENO5 z-pass, sliding window)"}
# FP64-pipe instructions (DADD + DMUL) per fill-box voxel of one tile-form axis
# pass by tile geometry, from ncu (smsp__sass_thread_inst_executed_op_{dadd,dmul}_pred_on.sum
# of one launch over its voxels; 16 x 16 at 192^3: 50.94 + 5.07, 8 x 27 at
# 216^3: 49.33 + 4.66); the rest of the 98 algorithmic operations (divisions,
# squares, scalings, maxima, scaled copies, the weights' products) run on the
# integer pipes.  FP64_PIPE_BUSY_TILE: sm__inst_executed_pipe_fp64 (pct of
# peak, active) of the same launches (a build before the out-of-line division
# and product, which leave the FP64 instruction counts unchanged).
FP64_INSTR_PER_VOXEL_TILE = {"16 x 16": 56.0, "8 x 27": 54.0}
FP64_PIPE_BUSY_TILE = {"16 x 16": ("192^3", 72.8), "8 x 27": ("216^3", 76.0)}


def tile_geometry(line: int) -> str:
    """The library's default tile for a line of `line` voxels: 8 x 27 where the
    last 27-voxel tile is at most 2 % idle, else 16 x 16."""
    tiles = -(-line // 27)
    return "8 x 27" if tiles * 27 * 50 <= line * 51 else "16 x 16"
N_KINDS = 5
# DRAM bytes per fill-box voxel of one launch of each stage kernel, measured at
# 512^3 with ncu (dram__bytes_read.sum + dram__bytes_write.sum, one pass):
# x pass 7.74 GB, y pass 3.40 GB, z pass 3.37 GB, combine 14.22 GB for 134.2 M
# voxels; the fused kernel was not captured
TRAFFIC_BYTES_PER_VOXEL = {1: 57.7, 2: 25.3, 3: 25.1, 4: 105.9}
# the same for the 16 x 16 tile form of the axis passes and the combine kernel,
# measured at 256^3 with ncu (one kernel and at most three launches per
# capture): x pass 474.2 MB, y 363.9 MB, z 362.2 MB, combine 2470.3 MB for
# 16.78 M voxels
TRAFFIC_BYTES_PER_VOXEL_TILE = {1: 28.3, 2: 21.7, 3: 21.6, 4: 147.2}
# algorithmic HBM bytes per voxel-step (each array touched once per stage):
# stage 1 phi + 5 coefficients -> phi1, stage 2 phi1 + phi + 5 coeff -> phi2,
# stage 3 phi2 + phi + 5 coeff + 3 masks -> phi1, phi
BYTES_PER_VOXEL_STEP = 8 * ((1 + 5 + 1) + (2 + 5 + 1) + (2 + 5 + 3 + 2))


def gpu_arm(args, dist: Dist):
    lib = Q.load(Q.GPU_LIB)
    if not lib.qssgpu_device_available():
        raise RuntimeError("GB300 library: no CUDA device")
    if args.axis_variant is not None:
        lib.qssgpu_set_axis_variant(args.axis_variant)
    n = args.n
    mask, phi = make_workload(n)
    g = Q.make_grid(lib, n)
    v = Q.Volume(g)
    v["mask"][...] = mask
    v["phi"][...] = phi
    o = Q.default_options(lib)
    set_options(lib, o)
    a0 = o.a
    if lib.qssgpu_prepare_step(C.byref(o), C.byref(v.p), C.byref(g), a0):
        Q.check(lib)
    nvox = n ** 3
    out = (C.c_double * (5 + 2 * N_KINDS))()
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        lib.qssgpu_time_steps(C.byref(o), C.byref(v.p), C.byref(g), a0, args.warmup, args.steps, out)
        Q.check(lib)
    dist.barrier()
    ms = dist.max(out[0])
    value = dist.ws * nvox * args.steps / (ms / 1e3)
    top = int(out[4])
    top_ms = out[1]
    window = args.axis_variant in (0, 1, 2)
    geom = {None: tile_geometry(n), 3: "16 x 16", 4: "8 x 27"}.get(args.axis_variant)

    def kname(k):
        return (WINDOW_NAME if window and k in WINDOW_NAME else KERNEL_NAME)[k].format(geom)

    kinds = {kname(k).split(" ")[0]: {"ms_total": round(out[5 + k], 3),
                                            "launches": int(out[5 + N_KINDS + k]),
                                            "share_of_step": round(out[5 + k] / ms, 4) if ms else None}
             for k in range(N_KINDS) if out[5 + N_KINDS + k] > 0}
    launches = int(out[2]) * args.steps

    # e2e through the C entry point with host arrays: one outer iteration of
    # constCurvModel3d whose pseudo-time window holds about `steps` steps.
    # An untimed call on a small pack first loads the kernels the call uses
    # (trapping, reinitialisation, reductions) that the device-resident steps
    # above did not.
    e2e = None
    if args.e2e:
        wm, wp = make_workload(48)
        _e2e_call(lib, Q.make_grid(lib, 48), wm, wp, args.steps, dist)
        # the call is repeated on fresh host arrays and the median call
        # reported: host page faults make single calls vary by ~10 %
        runs = sorted((_e2e_call(lib, g, v["mask"], v["phi"], args.steps, dist, pinned=True)
                       for _ in range(args.e2e_calls)), key=lambda x: x["wall"])
        r = runs[len(runs) // 2]
        pg = _e2e_call(lib, g, v["mask"], v["phi"], args.steps, dist, pinned=False)
        npts = g.num_gridpts
        h2d = 8 * npts * len(E2E_FROM_HOST)
        d2h = 8 * npts * 5 + 4 * npts + npts  # phi, phi_next, phi_prev, mask_w, mask_nw, labels, phi_bin
        # the call copies its arrays once in each direction for all its
        # inner steps: per step is the call's bytes over its inner steps
        e2e = {"value": dist.ws * nvox * r["steps"] / r["wall"], "unit": UNIT,
               "h2d_bytes_per_step": round(h2d / max(r["steps"], 1)),
               "d2h_bytes_per_step": round(d2h / max(r["steps"], 1)),
               "h2d_bytes_per_call": h2d, "d2h_bytes_per_call": d2h,
               "inner_steps": r["steps"], "outer_iterations": r["outer"],
               "wall_s": r["wall"], "calls": len(runs), "wall_s_all": [round(x["wall"], 3) for x in runs],
               "phases_s": r["phases"], "device_phases_s": r["device_phases"],
               "host_arrays": "page-locked (qssgpu_host_alloc)",
               "pageable": {"value": dist.ws * nvox * pg["steps"] / pg["wall"], "wall_s": pg["wall"],
                            "phases_s": pg["phases"]},
               "note": "one constCurvModel3d call with page-locked host arrays (the median of `calls` calls, "
                       "each on fresh arrays): uploads, inner steps, trapping, three reinitialisations, volume "
                       "integrals, downloads; `pageable` is one call on ordinary (pageable) arrays; "
                       "device_phases_s is each phase's device time (CUDA events on the library's stream "
                       "where the phase begins and ends; 'total' is their sum); phases_s is the host-side "
                       "split, where device work is charged to the phase whose host code waits for it"}

    peaks, kind = measured_peaks()
    probe = (C.c_double * 2)()
    # The kernels are built without FMA contraction (bit parity), so every
    # FP64-pipe instruction retires one operation: the ceiling of the FP64
    # pipe for them is its non-FMA issue rate, measured by the DADD probe.
    dfma_tflops, fp64_peak = args.fp64_peak, args.fp64_peak / 2
    peak_src = "nominal GB300 FP64 without FMA (half of 1.25 TFLOP/s)"
    if not lib.qssgpu_fp64_peak(probe):
        dfma_tflops, fp64_peak = round(probe[0], 4), round(probe[1], 4)
        peak_src = ("measured non-FMA FP64 issue rate (the repo's DADD probe, 8 chains/thread): the FP64 pipe's "
                    "ceiling for kernels built without FMA contraction; no FP64 figure in MEASURED_PEAKS.json")
    flop_launch = FLOP_PER_VOXEL[top] * nvox
    achieved_tf = flop_launch / (top_ms / 1e3) / 1e12 if top_ms > 0 else 0.0
    tile = top in (1, 2, 3) and not window
    if tile or (top == 4 and not window):
        traffic_table = dict(TRAFFIC_BYTES_PER_VOXEL_TILE)
        traffic_unit = "bytes per launch (ncu at 256^3 with 16 x 16 tiles, scaled per voxel to this size)"
    else:
        traffic_table = TRAFFIC_BYTES_PER_VOXEL
        traffic_unit = "bytes per launch (ncu at 512^3, scaled per voxel to this size)"
    fp64_pipe = None
    if tile and top_ms > 0:
        per_voxel = FP64_INSTR_PER_VOXEL_TILE[geom]
        instr = per_voxel * nvox / (top_ms / 1e3) / 1e12
        fp64_pipe = {"instructions_per_voxel": per_voxel, "tile": geom, "achieved": round(instr, 4),
                     "peak": fp64_peak, "unit": "T instructions/s", "frac": round(instr / fp64_peak, 4),
                     "ncu_busy_pct": FP64_PIPE_BUSY_TILE[geom][1], "ncu_case": FP64_PIPE_BUSY_TILE[geom][0],
                     "note": "FP64-pipe instructions (DADD + DMUL, ncu count per voxel) over the launch time, "
                             "against the non-FMA issue rate; ncu_busy_pct is sm__inst_executed_pipe_fp64 "
                             "(pct of peak) of the same kernel in the ncu_case capture"}
    # HBM: the step's algorithmic bytes over the time of all its stage kernels
    stage_total_ms = out[3] / args.steps
    achieved_gbs = BYTES_PER_VOXEL_STEP * nvox / (stage_total_ms / 1e3) / 1e9 if stage_total_ms > 0 else 0.0
    roofline = {"bound": "fp64", "achieved": round(achieved_tf, 4), "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": round(achieved_tf / fp64_peak, 4) if fp64_peak else None,
                "traffic": args.traffic if args.traffic is not None else (
                    round(traffic_table[top] * nvox) if top in traffic_table else None),
                "traffic_unit": traffic_unit,
                "kernel": kname(top), "flop_per_voxel": FLOP_PER_VOXEL[top],
                "launch_ms": round(top_ms, 4), "kernels": kinds,
                "peak_source": peak_src, "dfma_peak_tflops": dfma_tflops,
                "note": "achieved = the kernel's algorithmic FP64 operations per launch over its mean launch time "
                        "(CUDA events); about a third of them (divisions, squares, power-of-two scalings, maxima, "
                        "scaled copies) run bit-exactly on the integer pipes, so frac against the FP64 pipe's "
                        "non-FMA ceiling can exceed 1; fp64_pipe is the pipe's own utilisation",
                "fp64_pipe": fp64_pipe,
                "hbm": {"achieved": round(achieved_gbs, 1), "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                        "frac": round(achieved_gbs / peaks["hbm_gbs"], 4), "peak_kind": kind}}
    tuned = []
    nt = lib.qssgpu_axis_tuning(None, 0)
    if nt:
        rows = (C.c_int * (7 * nt))()
        nt = min(nt, lib.qssgpu_axis_tuning(rows, nt))
        tuned = [dict(zip(("level", "axis", "lanes", "lines_per_lane", "line", "form", "seg_len"),
                          rows[7 * i:7 * i + 7])) for i in range(nt)]
    return {"value": value, "ms": ms, "e2e": e2e, "roofline": roofline, "clocks": clk.summary(),
            "gpu_launches": launches, "stage_ms": top_ms, "axis_tuning": tuned}


# host arrays the e2e call uploads (drain_model3d's coefficients and masks)
E2E_FROM_HOST = ["phi", "mask", "mask_w", "mask_nw", "normal_velocity", "curvature_coeff",
                 "external_velocity_x", "external_velocity_y", "external_velocity_z"]
PHASES = ["total", "setup", "upload", "inner", "trap", "reinit", "reduce", "download"]


def _e2e_call(lib, g, mask, phi, steps, dist, pinned=False):
    """One constCurvModel3d call on fresh host arrays holding (mask, phi),
    timed on the host; returns wall time, inner steps and the phase split.
    With pinned, the arrays are page-locked host memory from the library's
    qssgpu_host_alloc (cudaHostAlloc), freed after the call."""
    buffers = []

    def pinned_zeros(shape, dtype):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        ptr = lib.qssgpu_host_alloc(nbytes)
        if not ptr:
            raise RuntimeError("qssgpu_host_alloc failed")
        buffers.append(ptr)
        raw = (C.c_ubyte * nbytes).from_address(ptr)
        return np.frombuffer(raw, dtype=dtype).reshape(shape)

    try:
        w = Q.Volume(g, alloc=pinned_zeros if pinned else None)
        w["mask"][...] = mask
        w["phi"][...] = phi
        o = Q.default_options(lib)
        set_options(lib, o)
        _fill_host_coefficients(lib, o, w, o.a)
        dt_est = 0.5 / (o.b_max_over_dx + o.max_U_over_dx)
        o.tplot = steps * dt_est * 0.999
        o.tmax = o.tplot * 0.5
        o.use_satn_stop = 0
        dist.barrier()
        t0 = time.perf_counter()
        lib.constCurvModel3d(C.byref(o), C.byref(w.p), C.byref(g), None)
        t1 = time.perf_counter()
        Q.check(lib)
        steps_done, outer = C.c_longlong(0), C.c_longlong(0)
        lib.qssgpu_call_stats(C.byref(w.p), C.byref(g), C.byref(steps_done), C.byref(outer))
        ph = (C.c_double * 8)()
        lib.qssgpu_call_times(C.byref(w.p), C.byref(g), ph)
        dph = (C.c_double * 8)()
        lib.qssgpu_call_device_times(C.byref(w.p), C.byref(g), dph)
        lib.qssgpu_release(C.byref(w.p))
        res = {"wall": dist.max(t1 - t0), "steps": steps_done.value, "outer": outer.value,
               "phases": {k: round(ph[i], 3) for i, k in enumerate(PHASES) if k not in ("total", "setup")},
               "device_phases": {k: round(dph[i], 3) for i, k in enumerate(PHASES) if k != "setup"}}
    finally:
        # the page-locked buffers go back even when the call failed
        for ptr in buffers:
            lib.qssgpu_host_free(ptr)
    return res


def _fill_host_coefficients(lib, o, w, a0):
    """Fills the host arrays the way drain_model3d does before calling
    constCurvModel3d (disconnected masks, mask gradient, coefficients)."""
    g = w.g
    gp = C.byref(g)
    lib.initializeDisconnectedMasks(w["mask_w"].ctypes.data_as(Q.c_double_p), gp)
    lib.initializeDisconnectedMasks(w["mask_nw"].ctypes.data_as(Q.c_double_p), gp)
    lib.getcentralgrad3dorder2_(Q.dptr(w["mask_x"]), Q.dptr(w["mask_y"]), Q.dptr(w["mask_z"]), *Q.gb_args(g),
                                Q.dptr(w["mask"]), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]), Q.dref(g.dx[1]),
                                Q.dref(g.dx[2]))
    lib.setSpaceDerivFunc(gp, C.byref(o))
    lib.setThetaOverlap(C.byref(w.p), gp, C.byref(o))
    lib.getMainInd_new(C.byref(o), C.byref(w.p), gp)
    bm, um = C.c_double(0), C.c_double(0)
    lib.setvarcurvadv3d_(Q.dptr(w["mask"]), Q.dptr(w["mask_x"]), Q.dptr(w["mask_y"]), Q.dptr(w["mask_z"]),
                         Q.dptr(w["curvature_coeff"]), Q.dptr(w["external_velocity_x"]),
                         Q.dptr(w["external_velocity_y"]), Q.dptr(w["external_velocity_z"]), C.byref(bm),
                         C.byref(um), Q.dref(o.b), *Q.gb_args(g), *Q.fb_args(g), Q.dref(g.dx[0]))
    o.b_max_over_dx, o.max_U_over_dx = bm.value, um.value
    lib.setvarnorm3d_(Q.dptr(w["mask"]), Q.dptr(w["mask_x"]), Q.dptr(w["mask_y"]), Q.dptr(w["mask_z"]),
                      Q.dptr(w["normal_velocity"]), Q.dref(a0), Q.dref(o.theta), *Q.gb_args(g), *Q.fb_args(g),
                      Q.dref(g.dx[0]))
    Q.check(lib)


def batched_arm(args):
    """Batched mode on uneven volumes: sides uniform in 48..160 voxels (seed 2),
    porosity uniform in 0.30..0.40, contact angle uniform in 0..60 degrees and
    a curvature ladder per volume, WENO5 + TVD-RK3.  The same volumes run once
    through the plain single-volume path (drain_model3d per volume, one after
    the other) and once through qssgpu_ladder_batch; every volume must end
    bit-identical.  Returns voxel-steps/s of both (wall clock, host arrays,
    uploads and downloads included)."""
    lib = Q.load(Q.GPU_LIB)
    rng = np.random.default_rng(2)
    nv = args.batch_volumes
    sides = rng.integers(48, 161, nv)
    poros = rng.uniform(0.30, 0.40, nv)
    thetas = rng.uniform(0.0, 60.0, nv)
    a0s = rng.uniform(1.0, 1.5, nv)
    vols = []
    for i in range(nv):
        n = int(sides[i])
        g = Q.make_grid(lib, n)
        v = Q.Volume(g)
        m = S.lognormal(n, mu=math.log(6.0), sigma=0.3, porosity=float(poros[i]), seed=100 + i).mask()
        v["mask"][...] = m
        v["phi"][...] = S.initial_phi(m, n)
        o = Q.default_options(lib)
        o.theta = float(thetas[i]) * 3.14159 / 180
        o.order_space_accur, o.order_time_accur = 5, 3
        o.a, o.b, o.dc = float(a0s[i]), 0.04, 0.9722
        o.amax = o.a + (args.batch_steps - 0.5) * o.b * o.dc
        o.tmax, o.tplot = 0.05, 0.02
        o.check_connectivity = 1
        vols.append((n, g, v, o))

    def copy_opts(o):
        c = Q.Options()
        C.pointer(c)[0] = o
        return c

    def clone(v):
        w = Q.Volume(v.g)
        w.copy_from(v)
        return w

    # plain path: one volume at a time (the drain_model3d ladder without its
    # per-step files, as in the batched run)
    plain, stats, phases_plain, walls = [], [], [], []
    t0 = time.perf_counter()
    for n, g, v, o in vols:
        w, oo = clone(v), copy_opts(o)
        one_o = (C.POINTER(Q.Options) * 1)(C.pointer(oo))
        one_p = (C.POINTER(Q.QSSDataArrays) * 1)(C.pointer(w.p))
        one_g = (C.POINTER(Q.Grid) * 1)(C.pointer(g))
        tv = time.perf_counter()
        if lib.qssgpu_ladder_batch(1, 1, one_o, one_p, one_g, None, None, 1):
            Q.check(lib)
        walls.append(time.perf_counter() - tv)
        s_in, s_out = C.c_longlong(0), C.c_longlong(0)
        lib.qssgpu_call_stats(C.byref(w.p), C.byref(g), C.byref(s_in), C.byref(s_out))
        stats.append(s_in.value)
        ph = (C.c_double * 8)()
        lib.qssgpu_call_times(C.byref(w.p), C.byref(g), ph)
        phases_plain.append(list(ph))
        lib.qssgpu_release(C.byref(w.p))
        plain.append(w)
    t_plain = time.perf_counter() - t0
    # batched
    batch = [clone(v) for _, _, v, _ in vols]
    opts_b = [copy_opts(o) for *_, o in vols]
    arr_o = (C.POINTER(Q.Options) * nv)(*[C.pointer(o) for o in opts_b])
    arr_p = (C.POINTER(Q.QSSDataArrays) * nv)(*[C.pointer(b.p) for b in batch])
    arr_g = (C.POINTER(Q.Grid) * nv)(*[C.pointer(g) for _, g, _, _ in vols])
    t0 = time.perf_counter()
    rc = lib.qssgpu_ladder_batch(1, nv, arr_o, arr_p, arr_g, None, None, args.batch_workers)
    t_batch = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"batched mode: {rc} volumes failed: {lib.qssgpu_error_string().decode()}")
    exact = all(np.array_equal(batch[i].arrays[k], plain[i].arrays[k]) for i in range(nv)
                for k in batch[i].arrays)
    phases_batch = []
    for b, (_, g, _, _) in zip(batch, vols):
        ph = (C.c_double * 8)()
        lib.qssgpu_call_times(C.byref(b.p), C.byref(g), ph)
        phases_batch.append(list(ph))
        lib.qssgpu_release(C.byref(b.p))
    names = ["total", "setup", "upload", "inner", "trap", "reinit", "reduce", "download"]
    sum_plain = {k: round(sum(p[i] for p in phases_plain), 3) for i, k in enumerate(names)}
    sum_batch = {k: round(sum(p[i] for p in phases_batch), 3) for i, k in enumerate(names)}
    work = sum(float(n) ** 3 * st for (n, *_), st in zip(vols, stats))
    # Roof of any batching of these volumes: the best rate one volume reached
    # alone on the plain path (a large one, whose kernels fill the GPU) is
    # taken as the rate the GPU sustains on this work; overlapping volumes
    # can win back the rest of the plain path's time, no more.
    rates = [float(n) ** 3 * st / t for (n, *_), st, t in zip(vols, stats, walls) if t > 0]
    best = max(rates) if rates else 0.0
    roof = {"best_single_volume_rate": best,
            "best_single_volume_side": int(vols[rates.index(best)][0]) if rates else None,
            "speedup_bound": t_plain / (work / best) if best > 0 else None,
            "batched_over_best_rate": (work / t_batch) / best if best > 0 else None,
            "note": "speedup_bound = plain wall time / (all voxel-steps at the best rate one volume reached "
                    "alone on the plain path); batched_over_best_rate = the batch's rate over that rate"}
    return {"volumes": nv, "sides": [int(x) for x in (sides.min(), sides.max())],
            "fill_voxels": int(sum(int(x) ** 3 for x in sides)), "ladder_steps": args.batch_steps,
            "inner_steps_total": int(sum(stats)), "workers": args.batch_workers or nv,
            "plain": {"value": work / t_plain, "wall_s": t_plain},
            "batched": {"value": work / t_batch, "wall_s": t_batch},
            "speedup": t_plain / t_batch, "per_volume_exact": bool(exact), "unit": UNIT, "roof": roof,
            "phase_seconds_summed_over_volumes": {"plain": sum_plain, "batched": sum_batch},
            "note": "wall clock of drain_model3d ladders with host arrays (WENO5 + TVD-RK3, tplot 0.02, "
                    "tmax 0.05, reinit and trapping included, no per-step files); plain = one volume "
                    "after the other, batched = all volumes in one qssgpu_ladder_batch call"}


def adjoint_arm(args):
    """Adjoint mode: 128^3 sphere pack (seed 3, radius 6 voxels, porosity 0.35),
    contact angle = trilinear interpolation of an 8^3 control grid in 0..60
    degrees (seed 3), target = H_eps(phi_T) of a hidden control grid (seed 4),
    TVD-RK3 WENO5 steps at curvature 0.2 per voxel, checkpoints every 20 steps.
    Reports the wall-clock ratio of forward + gradient to forward alone."""
    lib = Q.load(Q.GPU_LIB)
    n, steps, ckpt = args.adj_n, args.adj_steps, args.adj_ckpt
    g = Q.make_grid(lib, n)
    v = Q.Volume(g)
    m = S.overlapping(n, radius_vox=6.0, porosity=0.35, seed=3).mask()
    v["mask"][...] = m
    v["phi"][...] = S.initial_phi(m, n)
    o = Q.default_options(lib)
    dx = g.dx[0]
    o.a, o.b, o.overlap = 0.2 / dx, 0.04, 0.0
    dt = 0.5 / (2 * o.b * 3 / dx ** 2 + 2.0 / dx + abs(o.a) * math.sqrt(3) / dx)

    def angles(seed):
        c = np.random.default_rng(seed).uniform(0.0, math.radians(60.0), (8, 8, 8))
        t = np.arange(n) / (n - 1) * 7
        i0 = np.minimum(np.floor(t).astype(int), 6)
        f = t - i0
        out = np.zeros((n, n, n))
        for dz in (0, 1):
            for dy in (0, 1):
                for dxx in (0, 1):
                    w = (np.where(dz, f, 1 - f)[:, None, None] * np.where(dy, f, 1 - f)[None, :, None] *
                         np.where(dxx, f, 1 - f)[None, None, :])
                    out += w * c[np.ix_(i0 + dz, i0 + dy, i0 + dxx)]
        full = np.zeros(v["mask"].shape)
        full[3:n + 3, 3:n + 3, 3:n + 3] = out
        return full

    theta, hidden = angles(3), angles(4)
    zeros = np.zeros(v["mask"].shape)
    loss = C.c_double(0)
    phiT = np.zeros(v["mask"].shape)
    if lib.qssgpu_forward_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(hidden), Q.dptr(zeros), steps, dt,
                                C.byref(loss), Q.dptr(phiT)):
        Q.check(lib)
    eps = 1.5 * dx
    target = np.where(phiT < -eps, 0.0, np.where(phiT > eps, 1.0, 0.5 + phiT / (2 * eps) +
                                                  np.sin(math.pi * phiT / eps) / (2 * math.pi)))
    # warm-up, then timed forward and forward + gradient
    lib.qssgpu_forward_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(theta), Q.dptr(target), 2, dt,
                             C.byref(loss), None)
    t0 = time.perf_counter()
    if lib.qssgpu_forward_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(theta), Q.dptr(target), steps, dt,
                                C.byref(loss), None):
        Q.check(lib)
    t_fwd = time.perf_counter() - t0
    grad = np.zeros(v["mask"].shape)
    t0 = time.perf_counter()
    if lib.qssgpu_adjoint_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(theta), Q.dptr(target), steps, dt,
                                ckpt, C.byref(loss), Q.dptr(grad)):
        Q.check(lib)
    t_adj = time.perf_counter() - t0
    # the same gradient with the whole trajectory kept in HBM (one segment:
    # no recomputation; ~85 GB at 128^3 / 200 steps); the gradient does not
    # depend on the checkpoint spacing, bit for bit
    store_all = None
    if args.adj_store_all:
        grad1 = np.zeros(v["mask"].shape)
        loss1 = C.c_double(0)
        t0 = time.perf_counter()
        rc = lib.qssgpu_adjoint_theta(C.byref(o), C.byref(v.p), C.byref(g), Q.dptr(theta), Q.dptr(target), steps,
                                      dt, 0, C.byref(loss1), Q.dptr(grad1))
        t_all = time.perf_counter() - t0
        if rc:
            store_all = {"error": lib.qssgpu_error_string().decode(errors="replace")}
            lib.qssgpu_clear_error()
        else:
            store_all = {"forward_and_gradient_s": t_all, "adjoint_cost_over_forward": t_all / t_fwd,
                         "gradient_equals_checkpointed": bool(np.array_equal(grad1, grad)),
                         "note": "checkpoint_every = steps: every stage state and WENO5 derivative of the "
                                 "forward pass kept in HBM, so the backward pass is the reverse sweep alone"}
    return {"n": n, "steps": steps, "checkpoint_every": ckpt, "loss": loss.value,
            "forward_s": t_fwd, "forward_and_gradient_s": t_adj, "adjoint_cost_over_forward": t_adj / t_fwd,
            "backward_over_forward": (t_adj - t_fwd) / t_fwd,
            "forward_voxel_steps_per_s": n ** 3 * steps / t_fwd,
            "grad_abs_max": float(np.abs(grad).max()),
            "store_all": store_all,
            "note": "wall clock including uploads; adjoint_cost_over_forward = (forward + gradient) / forward, "
                    "backward_over_forward = the backward pass (checkpoint recomputation + reverse sweep) / "
                    "forward; gradient d loss / d theta per voxel (radians)"}


def cpu_arm(args, nz: int, steps: int, warmup: int, threads: int):
    """The reference algorithm on the host cores (CPU oracle, OpenMP) on a
    512 x 512 x nz slab of the workload; returns voxel-steps/s and details."""
    olib = Q.load(os.path.join(ROOT, "oracle", "liboracle.so"))
    olib.oracle_set_threads(threads)
    olib.oracle_time_inner_steps.restype = C.c_double
    olib.oracle_time_inner_steps.argtypes = [C.POINTER(Q.Options), C.POINTER(Q.QSSDataArrays),
                                             C.POINTER(Q.Grid), C.c_int, C.c_double, C.c_int]
    n = args.n
    mask, phi = make_workload(n, nz)
    g = Q.make_grid(olib, (n, n, nz))
    w = Q.Volume(g)
    w["mask"][...] = mask
    w["phi"][...] = phi
    o = Q.default_options(olib)
    set_options(olib, o)
    _fill_host_coefficients(olib, o, w, o.a)
    o.tplot = 1e300
    if warmup:
        olib.oracle_time_inner_steps(C.byref(o), C.byref(w.p), C.byref(g), 1, o.a, warmup)
    sec = olib.oracle_time_inner_steps(C.byref(o), C.byref(w.p), C.byref(g), 1, o.a, steps)
    vox = n * n * nz
    return {"value": vox * steps / sec, "sec": sec, "sample": f"{n}x{n}x{nz} fill box (a z-slab of the {n}^3 "
            f"workload), {steps} inner WENO5/TVD-RK3 steps after {warmup} warm-up", "cores": threads}


def ladder_arm(threads: int):
    """Time to solution of the reference's own CPU-sized workload: the 64^3
    drainage ladder (overlapping pack, seed 0, radius 5, porosity 0.35; ENO2 +
    TVD-RK2, contact angle 0; curvature 0.05 -> 0.4 per voxel in 10 steps),
    one drain_model3d call with host arrays and its per-step files, through
    the GB300 library (z-slabs = the host's threads) and through the CPU
    oracle on the same number of OpenMP threads.  The CFL step depends on the
    slab split, so both runs do the same steps; their files must be equal."""
    import gzip

    lib = Q.load(Q.GPU_LIB)
    olib = Q.load(os.path.join(ROOT, "oracle", "liboracle.so"))
    n = 64
    mask = S.overlapping(n, radius_vox=5.0, porosity=0.35, seed=0).mask()
    phi = S.initial_phi(mask, n)
    da = 0.97222

    def run(l, set_par):
        g = Q.make_grid(l, n)
        v = Q.Volume(g)
        v["mask"][...] = mask
        v["phi"][...] = phi
        o = Q.default_options(l)
        o.theta = 0.0
        o.order_space_accur, o.order_time_accur = 2, 2
        o.a, o.b, o.dc = 1.25, 0.04, da / 0.04
        o.amax, o.amin = 10.0 + 0.5 * da, 0.5
        o.tmax, o.tplot = 0.1, 0.0167
        o.check_connectivity = 1
        set_par(threads)
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                fp = Q.libc_fopen("out")
                t0 = time.perf_counter()
                l.drain_model3d(C.byref(o), C.byref(v.p), C.byref(g), fp)
                t = time.perf_counter() - t0
                Q.libc_fclose(fp)
                files = {}
                for f in sorted(os.listdir(d)):
                    if f.startswith("data_step"):
                        with gzip.open(f, "rb") as fh:
                            files[f] = fh.read()
            finally:
                os.chdir(cwd)
                set_par(1)
        return t, files

    run(lib, lib.qssgpu_set_slabs)  # warm-up: loads the kernels of every phase
    Q.check(lib)
    t_gpu, f_gpu = run(lib, lib.qssgpu_set_slabs)
    Q.check(lib)
    t_cpu, f_cpu = run(olib, olib.oracle_set_threads)
    lib.qssgpu_set_slabs(0)
    return {"workload": "64^3 drainage ladder (overlapping pack seed 0, radius 5, porosity 0.35), ENO2 + TVD-RK2, "
                        "contact angle 0, curvature 0.05 -> 0.4 per voxel in 10 steps, per-step files written",
            "slabs": threads, "gpu_s": t_gpu, "cpu_s": t_cpu, "cpu_cores": threads, "cpu_kind": "port",
            "speedup": t_cpu / t_gpu, "steps_saved": len(f_gpu),
            "files_identical": list(f_gpu) == list(f_cpu) and all(f_gpu[k] == f_cpu[k] for k in f_cpu)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--e2e-calls", type=int, default=3, help="timed e2e calls (the median is reported)")
    ap.add_argument("--no-cpu", dest="cpu", action="store_false")
    ap.add_argument("--cpu-nz", type=int, default=64)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--fp64-peak", type=float, default=1.25)
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the batched-mode measurement (uneven volumes)")
    ap.add_argument("--batch-volumes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--batch-workers", type=int, default=0)
    ap.add_argument("--batch-only", action="store_true", help="measure batched mode only")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false", help="skip the adjoint-mode measurement")
    ap.add_argument("--no-ladder", dest="ladder", action="store_false",
                    help="skip the 64^3 drainage-ladder time to solution (GB300 vs CPU oracle)")
    ap.add_argument("--adjoint-only", action="store_true")
    ap.add_argument("--adj-n", type=int, default=128)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--adj-ckpt", type=int, default=20)
    ap.add_argument("--no-adj-store-all", dest="adj_store_all", action="store_false",
                    help="skip the adjoint run that keeps the whole trajectory in HBM (no recomputation)")
    ap.add_argument("--axis-variant", type=int, default=None,
                    help="WENO5 axis passes: 0 registers, 1 shared memory, 2 launch shapes tuned by timing, "
                         "3 tiles with one voxel per thread (default: tiles)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the roofline kernel (overrides the measured table)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, _, local = dist_info()
    if ws > 1 and args.impl == "gb300":
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)  # one GPU per rank, before CUDA starts
    dist = Dist()
    threads = os.cpu_count() or 1
    out = ResultLine()
    try:
        _run(args, dist, threads, out)
    finally:
        out.close()
        dist.close()


def _run(args, dist: Dist, threads: int, out: ResultLine):
    if args.impl == "reference":
        if dist.rank != 0:
            return
        r = cpu_arm(args, args.cpu_nz, args.steps, args.warmup, threads)
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * r["sec"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": f"{args.n}^3 lognormal grain pack, porosity 0.30, theta 40 deg, "
                                       "WENO5 + TVD-RK3 (sampled on a z-slab)", "n": args.n},
                "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": r["sample"]},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        out.emit(line)
        return

    if args.adjoint_only:
        if dist.rank == 0:
            out.emit({"adjoint_mode": adjoint_arm(args)})
        return
    if args.batch_only:
        if dist.rank == 0:
            out.emit({"batched_mode": batched_arm(args)})
        return
    res = gpu_arm(args, dist)
    cpu = None
    if dist.rank == 0 and args.cpu:
        c = cpu_arm(args, args.cpu_nz, args.cpu_steps, 1, threads)
        cpu = {"value": c["value"], "unit": UNIT, "cores": threads, "kind": "port", "sample": c["sample"]}
    if dist.rank == 0:
        line = {"metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"{args.n}^3 lognormal grain pack (mu=ln 8, sigma=0.3 voxels), porosity 0.30, "
                                       "theta 40 deg, WENO5 + TVD-RK3, variable coefficients",
                           "n": args.n, "ghost": 3, "dx": 0.04, "parallelism": f"replicas x{dist.ws}",
                           "l2": "inputs larger than L2 (each FP64 array 1.1 GB)",
                           "axis_variant": {None: "by size", 0: "registers", 1: "shared memory",
                                            2: "tuned", 3: "tiles"}.get(args.axis_variant, args.axis_variant)},
                "e2e": res["e2e"], "gpu_launches": res["gpu_launches"], "roofline": res["roofline"],
                "cpu_baseline": cpu, "clocks": res["clocks"]}
        if res["axis_tuning"]:
            line["config"]["axis_tuning"] = res["axis_tuning"]
        if args.batched:
            line["batched_mode"] = batched_arm(args)
        if args.adjoint:
            line["adjoint_mode"] = adjoint_arm(args)
        if args.ladder and args.cpu:
            line["ladder_64_eno2"] = ladder_arm(threads)
        out.emit(line)


if __name__ == "__main__":
    main()
