"""ctypes binding of libsph_gb300.so (include/sph_gb300.h).

The library is the only compute path: there is no CPU fallback.  If it has
not been built, loading raises (build it with ``sph.build.build()``).
"""
import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

# enums of include/sph_gb300.h
FLUID, BOUNDARY, TEMP_BOUNDARY, COUPLED = 0, 1, 2, 3
KERNEL_CUBIC, KERNEL_GAUSSIAN, KERNEL_WENDLAND = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
INTEGRATOR_PEC, INTEGRATOR_EULER, INTEGRATOR_VERLET = 0, 1, 2

SPH_OK = 0
STATUS_CELL_OVERFLOW = 1 << 0
STATUS_GRID_COARSENED = 1 << 1
STATUS_NONFINITE = 1 << 2
STATUS_GRID_TOO_LARGE = 1 << 3
STATUS_NO_FLUID = 1 << 4
STATUS_SMALL_DT = 1 << 5
#: status bits that are informational, not errors
STATUS_INFO = STATUS_GRID_COARSENED | STATUS_SMALL_DT

FIELDS = ("m", "rho", "p", "c", "drho", "h", "x", "y", "vx", "vy", "ax", "ay",
          "xsphx", "xsphy", "x0", "y0", "vx0", "vy0", "rho0")


class Wcsph(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("rho0", "gamma", "co", "B", "Pb", "alpha", "beta", "epsilon",
                                          "r0", "D", "p1", "p2", "height")] + \
               [("use_xsph", C.c_int32), ("use_summation_density", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("precision", C.c_int32), ("integrator", C.c_int32),
                ("pec_use_xsph", C.c_int32), ("pec_strict", C.c_int32), ("pad0", C.c_int32),
                ("nn_scale", C.c_double), ("h_fixed", C.c_double), ("cfl_c", C.c_double),
                ("cfl_f", C.c_double), ("damping", C.c_double), ("dt_fixed", C.c_double)]


class Particles(C.Structure):
    _fields_ = [("n", C.c_int64), ("label", C.c_void_p)] + [(k, C.c_void_p) for k in FIELDS]


BLOCK_ARRAYS = ("m", "p", "rho", "h", "c", "r", "w", "dw_x", "dw_y", "x", "y", "vx", "vy")


class Block(C.Structure):
    """sph_block_t: one neighbour block in computed_dtype layout (device)."""
    _fields_ = [("n", C.c_int64), ("label", C.c_void_p)] + [(k, C.c_void_p) for k in BLOCK_ARRAYS]


class Workspace(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("bytes", C.c_size_t), ("n_cap", C.c_int64), ("max_cells", C.c_int64)]


ADJOINT_ARRAYS = ("xb", "yb", "vxb", "vyb", "rhob", "axb", "ayb", "drhob", "alphab",
                  "lax", "lay", "lad", "xhb", "yhb", "vxhb", "vyhb", "rhohb", "alb")


class Adjoint(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ADJOINT_ARRAYS] + [("reuse_build", C.c_int32), ("pad0", C.c_int32),
                                                            ("omega", C.c_double), ("wall_x", C.c_double)]


#: every function include/sph_gb300.h declares
EXPORTS = ("sph_abi_version", "sph_workspace_size", "sph_default_max_cells", "sph_workspace_init",
           "sph_get_status", "sph_status_string", "sph_status_bit_string", "sph_initialize", "sph_eos", "sph_nn_update",
           "sph_nn_count", "sph_nn_export", "sph_compute", "sph_timestep", "sph_predict", "sph_correct",
           "sph_run", "sph_kernel_eval", "sph_kernel_grad", "sph_gauss_deriv", "sph_run_profiled",
           "sph_compute_static", "sph_run_wall_load", "sph_adjoint_step", "sph_batch_workspace_size",
           "sph_batch_setup", "sph_batch_instance_cells", "sph_batch_run", "sph_nn_probe_count",
           "sph_nn_probe_export", "sph_probe_density", "sph_newmark_predict", "sph_newmark_correct",
           "sph_newmark_work_size", "sph_newmark_acceleration", "sph_selftest_staging",
           "sph_block_equations")
SPH_ERR_STATIC_LIMIT = 5
STATIC_MAX_PARTICLES = 32768
STATIC_MAX_CELLS = 131072

STAGES = ("timestep", "predict", "build", "records", "pair", "correct")

_lib = None


class SphError(RuntimeError):
    pass


def load():
    """Load libsph_gb300.so; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SphError("libsph_gb300.so is not built (expected at %s); run sph.build.build() -- "
                       "the WCSPH step has no CPU fallback" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, PP, WP, CP, WS = C.c_void_p, C.POINTER(Particles), C.POINTER(Wcsph), C.POINTER(Config), C.POINTER(Workspace)
    sig = {
        "sph_abi_version": (C.c_int, []),
        "sph_workspace_size": (C.c_int, [C.c_int64, C.c_int64, C.POINTER(C.c_size_t)]),
        "sph_default_max_cells": (C.c_int64, [C.c_int64]),
        "sph_workspace_init": (C.c_int, [WS, vp]),
        "sph_get_status": (C.c_int, [WS, C.POINTER(C.c_uint32), vp]),
        "sph_status_string": (C.c_char_p, [C.c_int]),
        "sph_status_bit_string": (C.c_char_p, [C.c_uint32]),
        "sph_initialize": (C.c_int, [PP, WP, CP, vp]),
        "sph_eos": (C.c_int, [PP, WP, vp]),
        "sph_nn_update": (C.c_int, [PP, CP, WS, vp]),
        "sph_nn_count": (C.c_int, [PP, CP, WS, vp, vp]),
        "sph_nn_export": (C.c_int, [PP, CP, WS, vp, vp, vp]),
        "sph_compute": (C.c_int, [PP, WP, CP, WS, vp]),
        "sph_timestep": (C.c_int, [PP, WP, CP, WS, vp, vp]),
        "sph_predict": (C.c_int, [PP, CP, vp, vp]),
        "sph_correct": (C.c_int, [PP, CP, vp, vp]),
        "sph_run": (C.c_int, [PP, WP, CP, WS, C.c_int64, vp, vp]),
        "sph_kernel_eval": (C.c_int, [C.c_int, C.c_int64, vp, vp, vp, vp]),
        "sph_kernel_grad": (C.c_int, [C.c_int, C.c_int64, vp, vp, vp, vp, vp]),
        "sph_gauss_deriv": (C.c_int, [C.c_int64, vp, vp, vp, vp]),
        "sph_run_profiled": (C.c_int, [PP, WP, CP, WS, C.c_int64, C.POINTER(C.c_double), vp]),
        "sph_compute_static": (C.c_int, [PP, WP, CP, vp, vp]),
        "sph_run_wall_load": (C.c_int, [PP, WP, CP, WS, C.c_int64, C.c_double, vp, vp, vp]),
        "sph_adjoint_step": (C.c_int, [PP, PP, WP, CP, WS, C.POINTER(Adjoint), vp]),
        "sph_batch_workspace_size": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_size_t)]),
        "sph_batch_setup": (C.c_int, [WS, C.c_int64, C.POINTER(C.c_int64), WP, C.POINTER(C.c_double), CP,
                                      C.c_int32, vp]),
        "sph_batch_instance_cells": (C.c_int64, [WS, C.c_int64, C.POINTER(C.c_int64), C.c_int64]),
        "sph_batch_run": (C.c_int, [PP, CP, WS, C.c_int64, C.c_int64, vp, C.c_int32, vp]),
        "sph_nn_probe_count": (C.c_int, [PP, WS, C.c_int64, vp, vp, vp, vp, vp]),
        "sph_nn_probe_export": (C.c_int, [PP, WS, C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "sph_probe_density": (C.c_int, [PP, WP, C.c_int, WS, C.c_int64, vp, vp, vp, vp, vp, vp, vp]),
        "sph_selftest_staging": (C.c_int, [vp, vp, vp]),
        "sph_block_equations": (C.c_int, [C.POINTER(Block), C.POINTER(C.c_double), WP, vp, vp]),
        "sph_newmark_predict": (C.c_int, [PP, C.c_double, C.c_double, vp, vp]),
        "sph_newmark_correct": (C.c_int, [PP, C.c_double, C.c_double, vp, vp]),
        "sph_newmark_work_size": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_size_t)]),
        "sph_newmark_acceleration": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, vp, vp, vp, C.c_double, C.c_double,
                                               C.c_double, vp, vp, vp, vp, vp, C.c_size_t, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.sph_abi_version() != 1:
        raise SphError("libsph_gb300 ABI version mismatch")
    _lib = L
    return L


def check(code, what="sph call"):
    if code != SPH_OK:
        msg = load().sph_status_string(code).decode()
        raise SphError("%s failed: %s (code %d)" % (what, msg, code))


def status_names(bits):
    L = load()
    return [L.sph_status_bit_string(1 << b).decode() for b in range(32) if bits & (1 << b)]
