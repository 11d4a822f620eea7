"""ctypes binding of the lsmpqs C API (drain/imbibe/constant-curvature path).

The same binding drives any library that exports the reference's entry points:
the GB300 library built from ``csrc/`` (``libqssgpu.so``) and, in the tests,
the CPU oracle.  Struct layouts mirror ``include/lsmpqs_types.h`` (FP64 build
of ``Grid``, ``QSS_DataArrays``, ``Options``).

``Volume`` owns numpy arrays for every ``QSS_DataArrays`` member and exposes
the struct, so a test or a benchmark can build inputs in numpy, call
``drain_model3d(opts, vol.p, vol.g, fp)`` and read the results back as numpy
views without copies.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GPU_LIB = os.path.join(HERE, "libqssgpu.so")

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)
c_uchar_p = C.POINTER(C.c_ubyte)


class Grid(C.Structure):
    """``Grid`` (reference src/geometry/qss_grid.h:29-81)."""

    _fields_ = [
        ("num_dims", C.c_int),
        ("x_lo", C.c_double * 3),
        ("x_hi", C.c_double * 3),
        ("x_lo_ghostbox", C.c_double * 3),
        ("x_hi_ghostbox", C.c_double * 3),
        ("grid_dims", C.c_int * 3),
        ("grid_dims_ghostbox", C.c_int * 3),
        ("dx", C.c_double * 3),
        ("num_gridpts", C.c_int),
    ] + [(n, C.c_int) for n in (
        "ilo_gb ihi_gb jlo_gb jhi_gb klo_gb khi_gb "
        "ilo_fb ihi_fb jlo_fb jhi_fb klo_fb khi_fb "
        "ilo_D1_fb ihi_D1_fb jlo_D1_fb jhi_D1_fb klo_D1_fb khi_D1_fb "
        "ilo_D2_fb ihi_D2_fb jlo_D2_fb jhi_D2_fb klo_D2_fb khi_D2_fb "
        "ilo_D3_fb ihi_D3_fb jlo_D3_fb jhi_D3_fb klo_D3_fb khi_D3_fb "
        "num_nb_levels").split()] + [
        ("mark_gb", C.c_ubyte), ("mark_D1", C.c_ubyte), ("mark_D2", C.c_ubyte),
        ("mark_D3", C.c_ubyte), ("mark_fb", C.c_ubyte),
        ("beta", C.c_double), ("gamma", C.c_double),
    ]


REAL_ARRAYS = (
    "phi phi_next phi_extra phi_prev mask lse_rhs normal_velocity curvature_coeff "
    "external_velocity_x external_velocity_y external_velocity_z mask_x mask_y mask_z "
    "scratch1 scratch2"
).split()
REAL_ARRAYS_2 = "mask_w mask_nw mask_disconn_init theta overlap".split()


class QSSDataArrays(C.Structure):
    """``QSS_DataArrays`` (reference src/utilities/qss_data_arrays.h:24-73)."""

    _fields_ = ([(n, c_double_p) for n in REAL_ARRAYS]
                + [("connectivity", c_int_p), ("phi_bin", c_uchar_p)]
                + [(n, c_double_p) for n in REAL_ARRAYS_2])


_FN = C.c_void_p


class Options(C.Structure):
    """``Options`` (reference src/utilities/qss_options.h:34-168)."""

    _fields_ = [
        ("outfile", C.c_char * 256), ("path", C.c_char * 256),
        ("dx", C.c_double), ("tmax", C.c_double), ("tmax_r", C.c_double), ("tplot", C.c_double),
        ("accuracy", C.c_char * 20), ("accuracy_id", C.c_int),
        ("a", C.c_double), ("b", C.c_double),
        ("save_data", C.c_int), ("do_reinit", C.c_int), ("do_mask", C.c_int),
        ("eps_stop", C.c_double), ("subcell_fix", C.c_int), ("reinit_func", _FN),
        ("dc", C.c_double), ("cmax", C.c_double), ("amax", C.c_double), ("amin", C.c_double),
        ("vol_frac_max", C.c_double), ("vol_frac_min", C.c_double),
        ("mask_reinit", C.c_int), ("narrow_band", C.c_int), ("init_step", C.c_int),
        ("overlap", C.c_double), ("stop_touch", C.c_int), ("eps_coefficient", C.c_double),
        ("extrapol_id", C.c_int), ("extrapol_func", _FN), ("space_deriv_func", _FN),
        ("order_space_accur", C.c_int), ("order_time_accur", C.c_int),
        ("checkpoint", C.c_int), ("reservoir_inlet", C.c_int),
        ("theta", C.c_double), ("C", C.c_double),
        ("b_max_over_dx", C.c_double), ("max_U_over_dx", C.c_double),
        ("check_connectivity", C.c_int), ("phi_w_ind", C.c_int), ("phi_nw_ind", C.c_int),
        ("err_check_zone", C.c_double), ("use_var_theta", C.c_int),
        ("theta_1", C.c_double), ("theta_2", C.c_double),
        ("print_details", C.c_int), ("use_satn_stop", C.c_int),
        ("conserve_imbibe", C.c_int), ("center_inlet", C.c_int),
    ]


_GB = [c_int_p] * 6
_PTR = C.c_void_p

# Fortran-convention kernels: every argument by pointer.
KERNEL_SIGS = {
    "setvarnorm3d_": 7 + 12 + 1,
    "setvarnorm3dtheta_": 7 + 12 + 1,
    "setvarcurvadv3d_": 11 + 12 + 1,
    "getrhs3d2ndconst_": 5 + 12 + 3,
    "getrhs3d3rdconst_": 5 + 12 + 3,
    "getrhs3d2nd_": 8 + 12 + 3,
    "getrhs3d3rd_": 8 + 12 + 3,
    "getrhs3d5th_": 8 + 12 + 3,
    "getcentralgrad3dorder2_": 3 + 6 + 1 + 12 + 3,
    "signedlinearextrapolation3d_": 1 + 12 + 1,
    "qss3drk1step_": 3 * 7 + 6 + 1,
    "qss3dtvdrk2stage2_": 4 * 7 + 6 + 1,
    "qss3dtvdrk3stage3_": 4 * 7 + 6 + 1,
    "qss3dcomputedistanceforsubcellfix_": 2 + 12 + 3,
    "qss3dcomputereinitializationeqnrhssubcellfixorder1_": 2 + 6 + 2 + 6 + 3,
    "qss3dmaxnormdifflocal_": 2 + 6 + 1 + 6 + 6 + 1,
    "imposemaskparallel_": 4 + 6 + 2,
    "qss3dvolumeregionphilessthanzero_": 2 + 12 + 4,
    "imposetrapvelocity3d_": 7 + 12 + 1,
}


def load(path: str) -> C.CDLL:
    """Open a library exporting the lsmpqs C API and declare the signatures."""
    lib = C.CDLL(path)
    P = C.POINTER
    sig = {
        "drain_model3d": (None, [P(Options), P(QSSDataArrays), P(Grid), _PTR]),
        "imbibe_model3d": (None, [P(Options), P(QSSDataArrays), P(Grid), _PTR]),
        "constCurvModel3d": (C.c_double, [P(Options), P(QSSDataArrays), P(Grid), _PTR]),
        "constCurvModel3dNoVar": (C.c_double, [P(Options), P(QSSDataArrays), P(Grid), _PTR, C.c_double]),
        "trapComponents_mask": (None, [P(QSSDataArrays), P(Grid), P(Options)]),
        "findConnectivity3d": (None, [P(QSSDataArrays), P(Grid)]),
        "getMainInd_new": (None, [P(Options), P(QSSDataArrays), P(Grid)]),
        "reinitializeSubcellFix3d": (None, [c_double_p, P(Grid), P(Options)]),
        "signedLinearExtrapolationBCqss": (None, [c_double_p, P(Grid), C.c_int]),
        "setSpaceDerivFunc": (None, [P(Grid), P(Options)]),
        "setThetaOverlap": (None, [P(QSSDataArrays), P(Grid), P(Options)]),
        "initializeDisconnectedMasks": (None, [c_double_p, P(Grid)]),
        "createReservoirInlet3d": (None, [P(QSSDataArrays), P(Grid)]),
        "createGridSetGridDims": (P(Grid), [C.c_int, c_int_p, c_double_p, c_double_p, C.c_int]),
        "createOptionsDefault": (P(Options), []),
        "destroyOptions": (None, [P(Options)]),
        "destroyGrid": (None, [P(Grid)]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    for name in KERNEL_SIGS:
        if hasattr(lib, name):
            getattr(lib, name).restype = None
    extra = {
        "qssgpu_last_error": (C.c_int, []),
        "qssgpu_error_string": (C.c_char_p, []),
        "qssgpu_clear_error": (None, []),
        "qssgpu_device_available": (C.c_int, []),
        "qssgpu_set_slabs": (None, [C.c_int]),
        "qssgpu_set_weno_split": (C.c_int, [C.c_int]),
        "qssgpu_set_emu_level": (C.c_int, [C.c_int]),
        "qssgpu_set_axis_variant": (C.c_int, [C.c_int]),
        "qssgpu_axis_tuning": (C.c_int, [C.POINTER(C.c_int), C.c_int]),
        "qssgpu_axis_tuning_reset": (None, []),
        "qssgpu_axis_tuning_save": (C.c_int, [C.c_char_p]),
        "qssgpu_axis_tuning_load": (C.c_int, [C.c_char_p]),
        "qssgpu_host_alloc": (C.c_void_p, [C.c_size_t]),
        "qssgpu_host_free": (None, [C.c_void_p]),
        "qssgpu_call_times": (None, [P(QSSDataArrays), P(Grid), P(C.c_double)]),
        "qssgpu_call_device_times": (None, [P(QSSDataArrays), P(Grid), P(C.c_double)]),
        "qssgpu_loop_sum": (C.c_int, [P(C.c_double), C.c_longlong, P(C.c_double)]),
        "qss_reinitialize_mask": (None, [P(QSSDataArrays), P(Grid), P(Options)]),
        "qssgpu_create_mask_ubc": (C.c_int, [P(C.c_ubyte), P(QSSDataArrays), P(Grid), P(Options)]),
        "qssgpu_create_init_from_mask": (C.c_int, [P(QSSDataArrays), P(Grid), P(Options)]),
        "qssgpu_diff_steps": (C.c_int, [P(C.c_double), P(C.c_double), P(Grid), P(C.c_double), P(C.c_double),
                                        P(C.c_int)]),
        "qssgpu_phase_uchar": (C.c_int, [P(C.c_double), P(C.c_double), P(Grid), C.c_char, P(C.c_ubyte),
                                         P(C.c_ubyte)]),
        "oracle_phase_uchar": (C.c_int, [P(C.c_double), P(C.c_double), P(Grid), C.c_char, P(C.c_ubyte),
                                         P(C.c_ubyte)]),
        "oracle_create_mask_ubc": (C.c_int, [P(C.c_ubyte), P(QSSDataArrays), P(Grid), P(Options)]),
        "oracle_create_init_from_mask": (C.c_int, [P(QSSDataArrays), P(Grid), P(Options)]),
        "oracle_diff_steps": (C.c_int, [P(C.c_double), P(C.c_double), P(Grid), P(C.c_double), P(C.c_double),
                                        P(C.c_int)]),
        "qssgpu_adjoint_theta": (C.c_int, [P(Options), P(QSSDataArrays), P(Grid), P(C.c_double), P(C.c_double),
                                           C.c_int, C.c_double, C.c_int, P(C.c_double), P(C.c_double)]),
        "qssgpu_forward_theta": (C.c_int, [P(Options), P(QSSDataArrays), P(Grid), P(C.c_double), P(C.c_double),
                                           C.c_int, C.c_double, P(C.c_double), P(C.c_double)]),
        "qssgpu_ladder_batch": (C.c_int, [C.c_int, C.c_int, P(P(Options)), P(P(QSSDataArrays)), P(P(Grid)),
                                          P(_PTR), P(C.c_char_p), C.c_int]),
        "qssgpu_emu_selftest": (C.c_int, [C.c_longlong, C.c_ulonglong, P(C.c_longlong), P(C.c_double)]),
        "qssgpu_op_rates": (C.c_int, [P(C.c_double)]),
        "qssgpu_get_slabs": (C.c_int, [C.c_void_p]),
        "qssgpu_release": (None, [P(QSSDataArrays)]),
        "qssgpu_call_stats": (None, [P(QSSDataArrays), P(Grid), P(C.c_longlong), P(C.c_longlong)]),
        "qssgpu_prepare_step": (C.c_int, [P(Options), P(QSSDataArrays), P(Grid), C.c_double]),
        "qssgpu_time_steps": (C.c_int, [P(Options), P(QSSDataArrays), P(Grid), C.c_double, C.c_int, C.c_int,
                                        c_double_p]),
        "qssgpu_fp64_peak": (C.c_int, [c_double_p]),
        "oracle_set_threads": (None, [C.c_int]),
        "oracle_portable_sin": (C.c_double, [C.c_double]),
        "oracle_portable_cos": (C.c_double, [C.c_double]),
    }
    for name, (res, args) in extra.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    return lib


def check(lib: C.CDLL) -> None:
    """Raise if the GB300 library recorded an error since the last clear."""
    if hasattr(lib, "qssgpu_last_error") and lib.qssgpu_last_error():
        msg = lib.qssgpu_error_string().decode()
        lib.qssgpu_clear_error()
        raise RuntimeError(f"qssgpu error: {msg}")


def fn_address(lib: C.CDLL, name: str) -> int:
    """Address of an exported function, for ``Options.space_deriv_func``."""
    return C.cast(getattr(lib, name), C.c_void_p).value


def make_grid(lib: C.CDLL, n, dx: float = 0.04, accuracy: int = 1) -> Grid:
    """Grid of fill-box size ``n`` (int or 3-tuple) laid out the way the
    reference's createMaskUBC tool does it: x_lo = 3*dx, x_hi = x_lo + n*dx."""
    if np.isscalar(n):
        n = (int(n),) * 3
    dims = (C.c_int * 3)(*n)
    ng = 3
    lo = [0 + ng * dx for _ in range(3)]
    hi = [lo[d] + n[d] * dx for d in range(3)]
    gp = lib.createGridSetGridDims(3, dims, (C.c_double * 3)(*lo), (C.c_double * 3)(*hi), accuracy)
    g = Grid()
    C.pointer(g)[0] = gp[0]
    lib.destroyGrid(gp)
    return g


def default_options(lib: C.CDLL) -> Options:
    op = lib.createOptionsDefault()
    o = Options()
    C.pointer(o)[0] = op[0]
    lib.destroyOptions(op)
    return o


class Volume:
    """All arrays of one ``QSS_DataArrays`` as numpy buffers (ghost box,
    column-major: numpy shape (nz, ny, nx))."""

    def __init__(self, g: Grid, alloc=None):
        """alloc(shape, dtype) -> zeroed ndarray overrides np.zeros (e.g. page-locked buffers)."""
        self.g = g
        nx, ny, nz = (g.grid_dims_ghostbox[d] for d in range(3))
        self.shape = (nz, ny, nx)
        self.arrays: dict[str, np.ndarray] = {}
        self.p = QSSDataArrays()
        zeros = alloc or (lambda shape, dtype: np.zeros(shape, dtype=dtype))
        for name in REAL_ARRAYS + REAL_ARRAYS_2:
            a = zeros(self.shape, np.float64)
            self.arrays[name] = a
            setattr(self.p, name, a.ctypes.data_as(c_double_p))
        a = zeros(self.shape, np.int32)
        self.arrays["connectivity"] = a
        self.p.connectivity = a.ctypes.data_as(c_int_p)
        a = zeros(self.shape, np.uint8)
        self.arrays["phi_bin"] = a
        self.p.phi_bin = a.ctypes.data_as(c_uchar_p)

    def __getitem__(self, name: str) -> np.ndarray:
        return self.arrays[name]

    def fb(self, name: str) -> np.ndarray:
        g = self.g
        return self.arrays[name][g.klo_fb:g.khi_fb + 1, g.jlo_fb:g.jhi_fb + 1, g.ilo_fb:g.ihi_fb + 1]

    def copy_from(self, other: "Volume", names=None):
        for n in names or self.arrays:
            self.arrays[n][...] = other.arrays[n]


def gb_args(g: Grid):
    """The six ghost-box bounds as C int pointers (Fortran convention)."""
    return [C.byref(C.c_int(v)) for v in (g.ilo_gb, g.ihi_gb, g.jlo_gb, g.jhi_gb, g.klo_gb, g.khi_gb)]


def fb_args(g: Grid, klo=None, khi=None):
    return [C.byref(C.c_int(v)) for v in (g.ilo_fb, g.ihi_fb, g.jlo_fb, g.jhi_fb,
                                          g.klo_fb if klo is None else klo,
                                          g.khi_fb if khi is None else khi)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(c_double_p)


def dref(x: float):
    return C.byref(C.c_double(x))


def libc_fopen(path: str, mode: str = "w") -> int:
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    return libc.fopen(path.encode(), mode.encode())


def libc_fclose(fp: int) -> None:
    libc = C.CDLL(None)
    libc.fclose.argtypes = [C.c_void_p]
    libc.fclose(fp)
