"""ctypes binding of ``libapple_gb300.so`` (declared in ``include/apple_gb300.h``).

There is no fallback: if the library is missing or fails to load, importing
any compute entry point raises.  Build it with ``python -m apple_gb300._build``
(or ``__graft_entry__.build()``).
"""

from __future__ import annotations

import ctypes
import pathlib
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_uint, c_void_p

LIB_PATH = pathlib.Path(__file__).resolve().parent / "libapple_gb300.so"

OK = 0
F32, F64 = 0, 1
ARAP, STABLE_NEO_HOOKEAN, STABLE_NEO_HOOKEAN_MUSCLE = 0, 1, 2
FUN, GRAD, HESS_DIAG, HESS_PROD, HESS_QUAD = 1, 2, 4, 8, 16
PRIMARY_SUCCESS, MAX_STEPS_REACHED, LINE_SEARCH_FAILED, NAN_ENCOUNTERED, RUNNING = range(5)


class PncgParams(ctypes.Structure):
    _fields_ = [
        ("max_steps", c_int32),
        ("rtol", c_double),
        ("atol", c_double),
        ("max_backtracking", c_int32),
        ("armijo_c", c_double),
        ("overstep", c_double),
        ("beta_max", c_double),
        ("refresh_ratio", c_double),
    ]


class PncgStats(ctypes.Structure):
    _fields_ = [
        ("result", c_int32),
        ("n_steps", c_int32),
        ("grad_norm", c_double),
        ("grad_norm_first", c_double),
        ("energy", c_double),
        ("alpha", c_double),
        ("beta", c_double),
        ("line_search_steps", c_int32),
        ("line_search_ok", c_int32),
        ("hess_diag_mean", c_double),
    ]


class CgParams(ctypes.Structure):
    _fields_ = [("max_iter", c_int32), ("rtol", c_double), ("atol", c_double)]


class CgStats(ctypes.Structure):
    _fields_ = [("result", c_int32), ("n_iter", c_int32), ("residual", c_double), ("residual_first", c_double)]


class AgbError(RuntimeError):
    """A non-zero status from the C ABI."""


_SIGNATURES = {
    "agb_last_error": (c_char_p, []),
    "agb_version": (c_char_p, []),
    "agb_space_create": (c_int, [c_int32, c_void_p, POINTER(c_void_p)]),
    "agb_space_destroy": (c_int, [c_void_p]),
    "agb_space_order": (c_int, [c_void_p, c_void_p]),
    "agb_region_compute": (c_int, [c_int32, c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_int32)]),
    "agb_fem_create": (
        c_int,
        [c_void_p, c_int, c_int, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
         c_void_p, c_void_p, c_int32, POINTER(c_void_p)],
    ),
    "agb_fem_destroy": (c_int, [c_void_p]),
    "agb_fem_info": (c_int, [c_void_p, POINTER(c_int32), POINTER(c_int32)]),
    "agb_fem_cells": (c_int, [c_void_p, c_void_p, POINTER(ctypes.c_uint32)]),
    "agb_plan_tiles": (c_int, [c_int32, c_int32, c_void_p, c_void_p, c_int32, POINTER(c_int32), POINTER(c_int32),
                               c_void_p, c_void_p, c_void_p]),
    "agb_fem_fun": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_hess_diag": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_hess_prod": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_hess_quad": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_fun_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_eval": (
        c_int,
        [c_void_p, c_uint, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    ),
    "agb_model_create": (
        c_int,
        [c_void_p, c_int, c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, POINTER(c_void_p)],
    ),
    "agb_model_destroy": (c_int, [c_void_p]),
    "agb_model_eval": (
        c_int,
        [c_void_p, c_uint, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    ),
    "agb_dof_to_free": (c_int, [c_int32, ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_dof_to_full": (c_int, [c_int32, ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_pncg_default_params": (None, [POINTER(PncgParams)]),
    "agb_solver_create": (c_int, [c_void_p, POINTER(PncgParams), POINTER(c_void_p)]),
    "agb_solver_destroy": (c_int, [c_void_p]),
    "agb_solver_reset": (c_int, [c_void_p, c_void_p, c_void_p]),
    "agb_solver_iterate": (c_int, [c_void_p, c_int32, c_void_p]),
    "agb_solver_step": (c_int, [c_void_p, c_void_p]),
    "agb_solver_read": (c_int, [c_void_p, c_void_p, POINTER(PncgStats), c_void_p]),
    "agb_solver_read_direction": (c_int, [c_void_p, c_void_p, c_void_p]),
    "agb_solver_read_gradient": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_solver_read_reductions": (c_int, [c_void_p, POINTER(c_double), c_void_p]),
    "agb_pncg_minimize_host": (c_int, [c_void_p, c_void_p, POINTER(PncgStats), c_void_p]),
    "agb_solver_time_passes": (c_int, [c_void_p, c_int32, c_void_p, ctypes.c_size_t, POINTER(ctypes.c_float), c_void_p]),
    "agb_batch_create": (c_int, [c_int32, c_void_p, POINTER(PncgParams), c_int32, POINTER(c_void_p)]),
    "agb_batch_destroy": (c_int, [c_void_p]),
    "agb_batch_info": (c_int, [c_void_p, POINTER(c_int32), POINTER(c_int32)]),
    "agb_batch_reset": (c_int, [c_void_p, c_void_p, c_void_p]),
    "agb_batch_iterate": (c_int, [c_void_p, c_int32, c_void_p]),
    "agb_batch_step": (c_int, [c_void_p, c_void_p]),
    "agb_batch_read": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_cg_default_params": (None, [POINTER(CgParams)]),
    "agb_solver_adjoint": (c_int, [c_void_p, c_void_p, c_void_p, POINTER(CgParams), POINTER(CgStats), c_void_p]),
    "agb_fem_grad_param_vjp": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "agb_fem_set_activation": (c_int, [c_void_p, c_void_p]),
    "agb_solver_step_kernels": (c_int, [c_void_p, POINTER(c_int32)]),
    "agb_solver_checkpoint_size": (c_int, [c_void_p, POINTER(ctypes.c_size_t)]),
    "agb_solver_save": (c_int, [c_void_p, c_void_p, c_void_p]),
    "agb_solver_load": (c_int, [c_void_p, c_void_p, ctypes.c_size_t, c_void_p]),
    "agb_fem_grad_activation_vjp": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load the library (once).  Raises ImportError if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m apple_gb300._build` "
            "(the GPU path has no fallback)"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(rc: int) -> None:
    if rc != OK:
        msg = load().agb_last_error().decode(errors="replace")
        raise AgbError(f"apple_gb300 status {rc}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
