"""ctypes mirror of include/vebi.h and the loader of the CUDA library.

The structures below must match include/vebi.h field for field; tests/test_abi.py checks
their sizes against the compiled library.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

MAX_PATCHES = 16
MAX_CIRCLES = 8
NSTAGES = 16

VEBI_OK = 0
STATUS_NAMES = {
    0: "VEBI_OK",
    1: "VEBI_ERR_ARG",
    2: "VEBI_ERR_CUDA",
    3: "VEBI_ERR_OUT_OF_DOMAIN",
    4: "VEBI_ERR_CELL_CAPACITY",
    5: "VEBI_ERR_NEIGH_CAPACITY",
    6: "VEBI_ERR_ALL_IN_BIN",
    7: "VEBI_ERR_MIRROR_CAPACITY",
    8: "VEBI_ERR_TIMEOUT",
    9: "VEBI_ERR_NO_DEVICE",
    10: "VEBI_ERR_BOUNDARY",
    11: "VEBI_ERR_DIVERGED",
}
STATUS = {v: k for k, v in STATUS_NAMES.items()}
WARN_BICGSTAB_BREAKDOWN = 1
WARN_MAXITER = 2
WARN_ESCAPEES = 4
PREC_FP64 = 0
PRECOND_NONE = 0
PRECOND_MULTIGRID = 1
PREC_MIXED = 1

_D2P = C.c_double * 2 * MAX_PATCHES
_D2C = C.c_double * 2 * MAX_CIRCLES


class VebiParams(C.Structure):
    _fields_ = [
        ("h", C.c_double), ("dx", C.c_double), ("dv", C.c_double),
        ("Ra", C.c_double), ("Pr", C.c_double), ("El", C.c_double), ("beta", C.c_double),
        ("ve_nonlinearity", C.c_double), ("alpha_evss", C.c_double),
        ("body_force", C.c_double * 2),
        ("dt_coef_cfl", C.c_double), ("dt_coef_visc", C.c_double),
        ("tol", C.c_double),
        ("x_mint", C.c_double), ("x_maxt", C.c_double), ("y_mint", C.c_double), ("y_maxt", C.c_double),
        ("b_node", _D2P), ("b_edge", _D2P),
        ("b_vel", C.c_double * MAX_PATCHES), ("b_thermal", C.c_double * MAX_PATCHES),
        ("c_centre", _D2C), ("c_radius", C.c_double * MAX_CIRCLES),
        ("c_omega", C.c_double * MAX_CIRCLES), ("c_vel", _D2C),
        ("c_thermal", C.c_double * MAX_CIRCLES),
        ("b_type", C.c_int32 * MAX_PATCHES), ("b_periodic_parent", C.c_int32 * MAX_PATCHES),
        ("nb_patches", C.c_int32), ("nb_circles", C.c_int32),
        ("i_open_domain", C.c_int32), ("i_shift_coeff", C.c_int32),
        ("npfb", C.c_int32), ("nbS", C.c_int32),
        ("const_mod", C.c_int32), ("itermax", C.c_int32), ("nplink", C.c_int32),
        ("nmirror_cap", C.c_int32), ("precision", C.c_int32), ("correct_velocity", C.c_int32),
        ("ppe_warm_start", C.c_int32), ("ppe_precond", C.c_int32),
        ("reserved", C.c_int32 * 4),
    ]


class VebiDumpInfo(C.Structure):
    """vebi_dump_info of include/vebi.h: the host scalars of the dump files."""
    _fields_ = [(k, C.c_double) for k in ("time", "dt", "xb_min", "xb_max", "yb_min", "yb_max", "dx", "av_conc",
                                          "dv")] + \
               [(k, C.c_int32) for k in ("itime", "n_dump", "np_inflow", "flags")]


class VebiStepStats(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("LS_residual", C.c_double), ("umax", C.c_double),
        ("max_abs_u", C.c_double), ("max_abs_v", C.c_double), ("max_abs_p", C.c_double),
        ("rms_u", C.c_double), ("ppe_rhs_mean", C.c_double),
        ("stage_ms", C.c_double * NSTAGES),
        ("circle_force", C.c_double * 2),
        ("LS_iters", C.c_int32), ("n_inbin", C.c_int32),
        ("np", C.c_int32), ("npfb", C.c_int32), ("nmirror", C.c_int32), ("maxneighbours", C.c_int32),
        ("n_escapees", C.c_int32), ("error", C.c_int32), ("warnings", C.c_int32),
        ("gpu_launches", C.c_int32), ("refine_iters", C.c_int32),
        ("LS_iters_total", C.c_int32), ("nsteps", C.c_int32),
        ("n_near_pole", C.c_int32), ("n_near_pole_total", C.c_int32),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name in ("stage_ms", "circle_force") else v
        return d


STAGE_NAMES = [
    "advect_bin", "mirrors", "cells", "neighbours", "weights", "shifting",
    "gradients", "logconf", "predictor", "ppe_assembly", "ppe_solve", "pressure_grad",
    "final_update", "secondary", "reserved14", "reserved15",
]

PACKAGE_DIR = pathlib.Path(__file__).resolve().parent
BUILD_DIR = PACKAGE_DIR / "_build"
LIB_NAME = "libvebi_gb300.so"

# symbols include/vebi.h declares; the library must export every one of them
EXPORTED_SYMBOLS = [
    "vebi_create", "vebi_upload_state", "vebi_step", "vebi_run_steps", "vebi_download_state",
    "vebi_destroy", "vebi_pin_host", "vebi_unpin_host", "vebi_set_timing", "vebi_debug_size",
    "vebi_debug_get", "vebi_version", "vebi_last_error", "vebi_ppe_solve_noalloc",
    "vebi_batch_create", "vebi_batch_get", "vebi_batch_step", "vebi_batch_destroy", "vebi_set_solver_grid",
    "vebi_dump_async", "vebi_dump_write", "vebi_dump_wait", "vebi_format_list",
    "vebi_set_weissenberg", "vebi_adjoint_create", "vebi_adjoint_record", "vebi_adjoint_replay",
    "vebi_adjoint_restore", "vebi_adjoint_reverse", "vebi_adjoint_destroy", "vebi_test_barrier_timeout",
    "vebi_test_conversions",
    "vebi_set_velocity_limit", "vebi_set_coarse_block_rows",
]
DUMP_BACKGROUND = 1
DUMP_RESTART_READABLE = 2
NOALLOC_MAX_ROWS = 65536

_lib = None


def library_path() -> pathlib.Path:
    return pathlib.Path(os.environ.get("VEBI_LIB", BUILD_DIR / LIB_NAME))


def load_library():
    """Load the CUDA step library.  Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(path))
    P = C.POINTER
    vp = C.c_void_p
    lib.vebi_create.argtypes = [P(VebiParams), P(vp)]
    lib.vebi_upload_state.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                      P(C.c_double), P(C.c_uint8), C.c_int32]
    lib.vebi_step.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int32,
                              P(VebiStepStats)]
    lib.vebi_run_steps.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int32,
                                   P(C.c_double), P(VebiStepStats)]
    lib.vebi_download_state.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                        P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                        P(C.c_int32), P(C.c_uint8), C.c_int32]
    lib.vebi_destroy.argtypes = [vp]
    lib.vebi_pin_host.argtypes = [vp, C.c_int64]
    lib.vebi_unpin_host.argtypes = [vp]
    lib.vebi_set_timing.argtypes = [vp, C.c_int32]
    lib.vebi_debug_size.argtypes = [vp, C.c_char_p, P(C.c_int64), P(C.c_int64)]
    lib.vebi_debug_get.argtypes = [vp, C.c_char_p, vp, C.c_int64]
    lib.vebi_ppe_solve_noalloc.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int32, C.c_int64, C.c_int32,
                                           C.c_double, C.c_int32, vp, P(C.c_int32), P(C.c_double)]
    lib.vebi_ppe_solve_noalloc.restype = C.c_int
    lib.vebi_batch_create.argtypes = [P(VebiParams), C.c_int32, P(vp)]
    lib.vebi_batch_get.argtypes = [vp, C.c_int32, P(vp)]
    lib.vebi_batch_step.argtypes = [vp, C.c_int32, P(C.c_double), P(VebiStepStats)]
    lib.vebi_batch_destroy.argtypes = [vp]
    lib.vebi_set_solver_grid.argtypes = [vp, C.c_int32]
    lib.vebi_dump_async.argtypes = [vp]
    lib.vebi_dump_write.argtypes = [vp, P(VebiDumpInfo), C.c_char_p, C.c_char_p]
    lib.vebi_dump_wait.argtypes = [vp]
    lib.vebi_format_list.argtypes = [C.c_char_p, P(C.c_double), P(C.c_int32), C.c_char_p, C.c_int64]
    lib.vebi_format_list.restype = C.c_int64
    lib.vebi_set_weissenberg.argtypes = [vp, C.c_double]
    lib.vebi_set_velocity_limit.argtypes = [vp, C.c_double]
    lib.vebi_set_velocity_limit.restype = C.c_int
    lib.vebi_set_coarse_block_rows.argtypes = [vp, C.c_int32]
    lib.vebi_set_coarse_block_rows.restype = C.c_int
    lib.vebi_adjoint_create.argtypes = [vp, C.c_int32, C.c_int32, P(vp)]
    lib.vebi_adjoint_record.argtypes = [vp, C.c_int32, P(VebiStepStats)]
    lib.vebi_adjoint_replay.argtypes = [vp, C.c_int32, P(VebiStepStats)]
    lib.vebi_adjoint_restore.argtypes = [vp, C.c_int32]
    lib.vebi_adjoint_reverse.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_double), C.c_int32,
                                         P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                         P(C.c_int32)]
    lib.vebi_adjoint_destroy.argtypes = [vp]
    lib.vebi_test_barrier_timeout.argtypes = [C.c_int32, C.c_int64, P(C.c_int32), P(C.c_double)]
    lib.vebi_test_barrier_timeout.restype = C.c_int
    lib.vebi_test_conversions.argtypes = [C.c_int64, C.c_uint64, P(C.c_int64), P(C.c_int64)]
    lib.vebi_test_conversions.restype = C.c_int
    for fn in ("vebi_set_weissenberg", "vebi_adjoint_create", "vebi_adjoint_record", "vebi_adjoint_replay",
               "vebi_adjoint_restore", "vebi_adjoint_reverse", "vebi_adjoint_destroy"):
        getattr(lib, fn).restype = C.c_int
    for fn in ("vebi_batch_create", "vebi_batch_get", "vebi_batch_step", "vebi_batch_destroy", "vebi_set_solver_grid"):
        getattr(lib, fn).restype = C.c_int
    lib.vebi_version.restype = C.c_char_p
    lib.vebi_last_error.restype = C.c_char_p
    for fn in ("vebi_create", "vebi_upload_state", "vebi_step", "vebi_run_steps", "vebi_download_state",
               "vebi_destroy", "vebi_pin_host", "vebi_unpin_host", "vebi_set_timing", "vebi_debug_size",
               "vebi_debug_get"):
        getattr(lib, fn).restype = C.c_int
    _lib = lib
    return lib
