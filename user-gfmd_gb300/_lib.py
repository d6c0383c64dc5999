"""ctypes binding of the gfmd_gb300 C ABI (include/gfmd_gb300.h).

The native library is required: importing the bindings fails loudly when
``libgfmd_gb300.so`` has not been built, and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgfmd_gb300.so")

GFMD_OK = 0
GFMD_EINVAL = 1
GFMD_ENOMEM = 2
GFMD_ECUDA = 3
GFMD_ENONFINITE = 4
GFMD_ETIMEDOUT = 5
GFMD_ENOTCONVERGED = 6
GFMD_ENOPHI = 7

GFMD_PREC_F64 = 0
GFMD_PREC_F32 = 1
GFMD_PHI_FULL = 0
GFMD_PHI_HALF = 1

GFMD_OBST_NONE = 0
GFMD_OBST_SPHERE_EXP = 1
GFMD_OBST_SPHERE_LJ = 2
GFMD_OBST_MAP_EXP = 3
GFMD_OBST_MAP_BICUBIC = 4
GFMD_MIN_CG = 0
GFMD_MIN_FIRE = 1
GFMD_MIN_TR = 2


class Obstacle(ctypes.Structure):
    """gfmd_obstacle_t"""

    _fields_ = [
        ("kind", ctypes.c_int),
        ("center", ctypes.c_double * 3),
        ("radius", ctypes.c_double),
        ("epsilon", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("cutoff", ctypes.c_double),
        ("d_map", ctypes.c_void_p),
        ("map_z0", ctypes.c_double),
        ("norm", ctypes.c_int),
        ("lattice", ctypes.c_double * 2),
        ("nlayer", ctypes.c_int),
        ("layer_offset", (ctypes.c_double * 3) * 8),
        ("fz_ext", ctypes.c_double),
    ]


class MinParams(ctypes.Structure):
    """gfmd_min_params_t"""

    _fields_ = [
        ("method", ctypes.c_int),
        ("ftol", ctypes.c_double),
        ("maxiter", ctypes.c_int),
        ("recompute", ctypes.c_int),
        ("refine", ctypes.c_void_p),
        ("fire_minsteps", ctypes.c_int),
        ("fire_incfac", ctypes.c_double),
        ("fire_decfac", ctypes.c_double),
        ("fire_mix", ctypes.c_double),
        ("fire_mixdec", ctypes.c_double),
        ("fire_dtmax", ctypes.c_double),
        ("fire_dt", ctypes.c_double),
        ("fire_xlimit", ctypes.c_double),
        ("precond", ctypes.c_void_p),
        ("tr_dmax", ctypes.c_double),
        ("tr_rho_tol", ctypes.c_double),
        ("dmax", ctypes.c_double),
    ]


class MinReport(ctypes.Structure):
    """gfmd_min_report_t"""

    _fields_ = [
        ("status", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("force_evals", ctypes.c_int),
        ("energy", ctypes.c_double),
        ("fmax", ctypes.c_double),
        ("fnorm", ctypes.c_double),
        ("seconds", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchItem(ctypes.Structure):
    """gfmd_batch_item_t"""

    _fields_ = [
        ("handle", ctypes.c_void_p),
        ("refine", ctypes.c_void_p),
        ("obstacle", ctypes.POINTER(Obstacle)),
        ("d_u", ctypes.c_void_p),
        ("report", MinReport),
        ("precond", ctypes.c_void_p),
    ]


_NAMES = {
    GFMD_EINVAL: "EINVAL",
    GFMD_ENOMEM: "ENOMEM",
    GFMD_ECUDA: "ECUDA",
    GFMD_ENONFINITE: "ENONFINITE",
    GFMD_ETIMEDOUT: "ETIMEDOUT",
    GFMD_ENOTCONVERGED: "ENOTCONVERGED",
    GFMD_ENOPHI: "ENOPHI",
}


class SurfaceParams(ctypes.Structure):
    """gfmd_surface_params_t."""
    _fields_ = [("lattice", ctypes.c_double), ("hurst", ctypes.c_double),
                ("rms_slope", ctypes.c_double), ("lambda_short", ctypes.c_double),
                ("lambda_long", ctypes.c_double), ("seed", ctypes.c_ulonglong)]


class GFMDError(RuntimeError):
    """A non-zero status from the C ABI, with the library's message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{_NAMES.get(code, code)}] {msg}")
        self.code = code


_c_int, _c_dbl, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
_pi = ctypes.POINTER(ctypes.c_int)
_pd = ctypes.POINTER(ctypes.c_double)

# (name, argtypes) for every entry point of include/gfmd_gb300.h
SIGNATURES = {
    "gfmd_last_error": [],
    "gfmd_version": [],
    "gfmd_create": [_c_int, _c_int, _c_int, _c_int, ctypes.POINTER(_vp)],
    "gfmd_destroy": [_vp],
    "gfmd_set_stream": [_vp, _vp],
    "gfmd_set_phi": [_vp, _vp, _c_int, _vp],
    "gfmd_post_force": [_vp, _vp, _vp, _pd],
    "gfmd_post_force_host": [_vp, _vp, _vp, _pd],
    "gfmd_force_f64": [_vp, _vp, _vp, _vp],
    "gfmd_force_f32": [_vp, _vp, _vp, _vp],
    "gfmd_get_u0": [_vp, _vp],
    "gfmd_memory_usage": [_vp, _pd],
    "gfmd_solver_info": [_vp, _pi, _pi],
    "gfmd_plan_info": [_vp, _pi, _pi],
    "gfmd_force_kernel_times": [_vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float), _c_int, _pi],
    "gfmd_kernel_plan": [_vp, _pi, _pi, _pi],
    "gfmd_phi_pattern": [_vp, _pi, _pi],
    "gfmd_minimize": [_vp, ctypes.POINTER(Obstacle), ctypes.POINTER(MinParams), _vp,
                      ctypes.POINTER(MinReport)],
    "gfmd_make_preconditioner": [_vp, _c_dbl, ctypes.POINTER(_vp)],
    "gfmd_prec_gradient": [_vp, _vp, _vp, _vp],
    "gfmd_prec_gradient_host": [_vp, _vp, _vp, _vp],
    "gfmd_minimize_batch": [_c_int, ctypes.POINTER(BatchItem), ctypes.POINTER(MinParams)],
    "gfmd_run_dynamics": [_vp, ctypes.POINTER(Obstacle), _c_dbl, _c_dbl, _c_int, _vp, _vp, _vp,
                          ctypes.POINTER(MinReport)],
    "gfmd_obstacle_force": [_c_int, _c_int, _c_int, ctypes.POINTER(Obstacle), _vp, _vp, _vp, _vp],
    "gfmd_post_force_noalloc": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp],
    "gfmd_atoms_to_grid": [_c_int, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_int, _c_dbl, _c_dbl, _c_int,
                           _c_int, _vp, _vp, _vp, _pi, _vp],
    "gfmd_grid_to_atoms": [_c_int, _vp, _vp, _c_int, _c_int, _c_int, _vp, _c_int, _pd, _vp],
    "gfmd_rough_surface": [_c_int, _c_int, ctypes.POINTER(SurfaceParams), _vp, _vp],
    "gfmd_ws_create": [_c_int, _c_int, _c_int, ctypes.c_ulonglong, ctypes.POINTER(_vp)],
    "gfmd_ws_destroy": [_vp],
    "gfmd_ws_set_stream": [_vp, _vp],
    "gfmd_ws_num_params": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "gfmd_ws_get_params": [_vp, _vp, _vp],
    "gfmd_ws_set_params": [_vp, _vp],
    "gfmd_ws_forward": [_vp, _c_int, _c_int, _c_int, _vp, _vp],
    "gfmd_ws_loss_grad": [_vp, _c_int, _c_int, _c_int, _vp, _vp, _pd],
    "gfmd_ws_adam_step": [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float],
    "gfmd_ws_to_nhwc": [_vp, _c_int, _c_int, ctypes.c_float, _vp, _vp],
    "gfmd_ws_from_nhwc": [_vp, _c_int, _c_int, _c_dbl, _vp, _vp],
    "gfmd_kernel_create": [ctypes.c_char_p, ctypes.POINTER(_vp)],
    "gfmd_kernel_destroy": [_vp],
    "gfmd_kernel_info": [_vp, _pi, _pi],
    "gfmd_kernel_set_box": [_vp, ctypes.c_double, ctypes.c_double],
    "gfmd_kernel_phi": [_vp, _c_int, _c_int, _c_int, _vp, _vp, _c_int],
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load the native library (once)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"gfmd_gb300 native library not built: {LIB_PATH} is missing "
                "(run __graft_entry__.build())"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_char_p if name in ("gfmd_last_error", "gfmd_version") else _c_int
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != GFMD_OK:
        raise GFMDError(rc, lib().gfmd_last_error().decode(errors="replace"))
