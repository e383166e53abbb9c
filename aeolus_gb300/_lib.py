"""ctypes binding of the C ABI in ``include/aeolus_gb300.h``.

The library is the in-tree ``libaeolus_gb300.so`` built by ``build.py``.  If
it is missing the import of any compute entry point raises: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_long, c_size_t, c_uint, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libaeolus_gb300.so"

OK, ERR_ARG, ERR_CUDA, ERR_WORKSPACE, ERR_STATE = 0, 1, 2, 3, 4
PREC_FP64, PREC_SPLIT_BF16 = 0, 1
TUNING_KNOBS = 5  # AEOLUS_TUNING_KNOBS
(OP_SYNTHESIZE, OP_ANALYZE, OP_JACOBIAN, OP_WINDS, OP_BVE_TENDENCY, OP_SWE_TENDENCY,
 OP_BVE_RK4, OP_SWE_RK4, OP_SWE_VALIDATE, OP_SWE_INVARIANTS,
 OP_SYNTHESIZE_ADJOINT, OP_ANALYZE_ADJOINT, OP_BVE_TENDENCY_ADJOINT, OP_SWE_TENDENCY_ADJOINT,
 OP_BVE_RK4_ADJOINT, OP_SWE_RK4_ADJOINT, OP_VECTOR_CURL_DIV) = range(17)
STATE_NONFINITE, STATE_MONOPOLE, STATE_THICKNESS = 1, 2, 4

# Spectral operator ids of aeolus_spectral_op.
SOP_LAPLACIAN, SOP_INV_LAPLACIAN, SOP_INV_LAPLACIAN_ZERO, SOP_D_LAMBDA = 0, 1, 2, 3
SOP_SIN_THETA_D_THETA, SOP_ADJOINT_SIN_THETA_D_THETA, SOP_TRUNCATE = 4, 5, 6


class BveParams(ctypes.Structure):
    _fields_ = [("radius", c_double), ("omega", c_double), ("viscosity", c_double)]


class PeParams(ctypes.Structure):
    _fields_ = [("radius", c_double), ("omega", c_double), ("r_dry", c_double), ("cp_dry", c_double)]


class SweParams(ctypes.Structure):
    _fields_ = [("radius", c_double), ("omega", c_double), ("gravity", c_double),
                ("mean_depth", c_double), ("nu4", c_double), ("forcing", c_void_p)]


# name -> (restype, argtypes); mirrors include/aeolus_gb300.h exactly.
SIGNATURES = {
    "aeolus_last_error": (c_char_p, []),
    "aeolus_version": (c_int, []),
    "aeolus_profile_enable": (c_int, [c_int]),
    "aeolus_profile_collect": (c_int, [c_char_p, c_size_t]),
    "aeolus_profile_reset": (c_int, []),
    "aeolus_plan_create_gauss": (c_int, [c_int, c_int, c_int, c_double, c_int, POINTER(c_void_p)]),
    "aeolus_plan_create_points": (c_int, [c_long, c_void_p, c_void_p, c_void_p, c_int, c_double, c_int,
                                          POINTER(c_void_p)]),
    "aeolus_plan_destroy": (c_int, [c_void_p]),
    "aeolus_plan_info": (c_int, [c_void_p, POINTER(c_int), POINTER(c_int), POINTER(c_int), POINTER(c_int),
                                 POINTER(c_long)]),
    "aeolus_plan_nodes": (c_int, [c_void_p, c_void_p, c_void_p]),
    "aeolus_plan_set_precision": (c_int, [c_void_p, c_int, c_int]),
    "aeolus_plan_device_error": (c_int, [c_void_p, POINTER(c_int)]),
    "aeolus_rk4_stage": (c_int, [c_int, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_long, c_void_p]),
    "aeolus_selftest_wait_timeout": (c_int, [ctypes.c_ulonglong, POINTER(c_int), POINTER(ctypes.c_ulonglong)]),
    "aeolus_selftest_df_convert": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "aeolus_plan_set_tuning": (c_int, [c_void_p, POINTER(c_int)]),
    "aeolus_plan_get_tuning": (c_int, [c_void_p, POINTER(c_int)]),
    "aeolus_workspace_bytes": (c_int, [c_void_p, c_int, c_int, POINTER(c_size_t)]),
    "aeolus_synthesize": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_analyze": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_vector_curl_div": (c_int, [c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p,
                                       c_size_t, c_void_p]),
    "aeolus_synthesize_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "aeolus_pe_derive": (c_int, [c_void_p, POINTER(PeParams), c_int, c_void_p, c_void_p, c_int, c_void_p]),
    "aeolus_pe_columns": (c_int, [c_void_p, POINTER(PeParams), c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                  c_void_p]),
    "aeolus_pe_spectral": (c_int, [c_int, POINTER(PeParams), c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_int, c_void_p]),
    "aeolus_geodesic_sizes": (c_int, [c_int, POINTER(c_long), POINTER(c_long), POINTER(c_size_t)]),
    "aeolus_geodesic_build": (c_int, [c_int, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_size_t, c_void_p]),
    "aeolus_spectral_op": (c_int, [c_int, c_int, c_double, c_void_p, c_void_p, c_int, c_void_p]),
    "aeolus_jacobian": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_winds": (c_int, [c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t,
                             c_void_p]),
    "aeolus_bve_tendency": (c_int, [c_void_p, POINTER(BveParams), c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                    c_size_t, c_void_p]),
    "aeolus_swe_tendency": (c_int, [c_void_p, POINTER(SweParams), c_void_p, c_void_p, c_int, c_void_p, c_size_t,
                                    c_void_p]),
    "aeolus_bve_rk4": (c_int, [c_void_p, POINTER(BveParams), c_void_p, c_int, c_double, c_int, c_void_p, c_size_t,
                               c_void_p]),
    "aeolus_swe_rk4": (c_int, [c_void_p, POINTER(SweParams), c_void_p, c_int, c_double, c_int, c_void_p, c_void_p,
                               c_size_t, c_void_p]),
    "aeolus_swe_validate": (c_int, [c_void_p, c_void_p, POINTER(SweParams), c_void_p, c_void_p, c_void_p, c_int,
                                    c_void_p, c_size_t, c_void_p]),
    "aeolus_bve_spectral_diagnostics": (c_int, [c_int, c_double, c_double, c_void_p, c_void_p, c_int, c_void_p]),
    "aeolus_swe_invariants": (c_int, [c_void_p, POINTER(SweParams), c_void_p, c_void_p, c_int, c_void_p, c_size_t,
                                      c_void_p]),
    "aeolus_synthesize_adjoint": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_analyze_adjoint": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_bve_tendency_adjoint": (c_int, [c_void_p, POINTER(BveParams), c_void_p, c_void_p, c_void_p, c_int,
                                            c_void_p, c_size_t, c_void_p]),
    "aeolus_swe_tendency_adjoint": (c_int, [c_void_p, POINTER(SweParams), c_void_p, c_void_p, c_void_p, c_int,
                                            c_void_p, c_size_t, c_void_p]),
    "aeolus_bve_rk4_adjoint": (c_int, [c_void_p, POINTER(BveParams), c_void_p, c_void_p, c_int, c_double, c_void_p,
                                       c_size_t, c_void_p]),
    "aeolus_swe_rk4_adjoint": (c_int, [c_void_p, POINTER(SweParams), c_void_p, c_void_p, c_int, c_double, c_void_p,
                                       c_size_t, c_void_p]),
    "aeolus_ensemble_create": (c_int, [c_int, POINTER(c_void_p), POINTER(c_int), POINTER(BveParams),
                                       POINTER(c_void_p)]),
    "aeolus_ensemble_create_swe": (c_int, [c_int, POINTER(c_void_p), POINTER(c_int), POINTER(SweParams),
                                           POINTER(c_void_p)]),
    "aeolus_ensemble_swe_rk4": (c_int, [c_void_p, POINTER(c_void_p), c_double, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_ensemble_destroy": (c_int, [c_void_p]),
    "aeolus_ensemble_workspace_bytes": (c_int, [c_void_p, POINTER(c_size_t)]),
    "aeolus_ensemble_bve_rk4": (c_int, [c_void_p, POINTER(c_void_p), c_double, c_int, c_void_p, c_size_t, c_void_p]),
    "aeolus_ensemble_capture": (c_int, [c_void_p, POINTER(c_void_p), c_double, c_void_p, c_size_t, c_void_p]),
    "aeolus_ensemble_launch": (c_int, [c_void_p, c_int, c_void_p]),
    "aeolus_ensemble_autotune": (c_int, [c_void_p, POINTER(c_void_p), c_void_p, c_size_t, c_void_p, c_char_p,
                                         c_size_t]),
}

_lib = None


class AeolusError(RuntimeError):
    """A nonzero status from the C ABI (message from aeolus_last_error)."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


def load(path: os.PathLike | str | None = None):
    """Load the shared library (once) and declare every signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -m aeolus_gb300.build` "
            "(the GB300 kernels have no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int):
    if status != OK:
        msg = load().aeolus_last_error()
        err = ValueError if status == ERR_ARG else AeolusError
        if err is ValueError:
            raise ValueError(msg.decode() if msg else f"status {status}")
        raise AeolusError(status, msg.decode() if msg else "")
    return status
