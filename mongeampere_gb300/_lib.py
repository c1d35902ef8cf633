"""ctypes binding of ``libma_gb300.so`` (the C ABI declared in ``include/ma.h``).

The library is built in-tree by :func:`mongeampere_gb300.build.build`.  There is
no fallback: if the library is missing or cannot be loaded, every entry point
raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


class MaSolveOpts(ctypes.Structure):
    _fields_ = [("eps_g", ctypes.c_double), ("maxiter", ctypes.c_int64), ("stop_rule", ctypes.c_int),
                ("precision", ctypes.c_int), ("verbose", ctypes.c_int), ("cg_rtol", ctypes.c_double),
                ("cg_maxiter", ctypes.c_int64), ("precond", ctypes.c_int), ("init", ctypes.c_int)]


class MaStats(ctypes.Structure):
    _fields_ = [("niter", ctypes.c_size_t), ("neval", ctypes.c_size_t), ("cg_iters", ctypes.c_size_t),
                ("linesearch_halvings", ctypes.c_size_t), ("grad_norm", ctypes.c_double),
                ("max_rel_err", ctypes.c_double), ("value", ctypes.c_double), ("t_eval_ms", ctypes.c_double),
                ("t_linsolve_ms", ctypes.c_double), ("neval_fp64", ctypes.c_size_t),
                ("cg_noconv", ctypes.c_size_t)]


class MaProblem(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_void_p), ("n", ctypes.c_int64), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("nu", ctypes.c_void_p), ("w", ctypes.c_void_p), ("status", ctypes.c_int), ("stats", MaStats)]


class MaProfile(ctypes.Structure):
    _fields_ = [("cells_ms", ctypes.c_double), ("cells_launches", ctypes.c_int64),
                ("pieces_ms", ctypes.c_double), ("pieces_launches", ctypes.c_int64),
                ("cells_large_ms", ctypes.c_double), ("cells_large_launches", ctypes.c_int64),
                ("bounds_ms", ctypes.c_double), ("bounds_launches", ctypes.c_int64),
                ("pcg_ms", ctypes.c_double), ("pcg_launches", ctypes.c_int64), ("pcg_iters", ctypes.c_int64),
                ("large_sites", ctypes.c_int64), ("search", ctypes.c_int64 * 6),
                ("amg_fallbacks", ctypes.c_int64), ("amg_setup_ms", ctypes.c_double),
                ("amg_levels", ctypes.c_int64), ("mixed", ctypes.c_int64 * 4)]


# every symbol include/ma.h declares, with its ctypes signature
SIGNATURES = {
    "ma_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ma_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "ma_ctx_destroy": (None, [_vp]),
    "ma_ctx_set_stream": (ctypes.c_int, [_vp, _vp]),
    "ma_ctx_last_error": (ctypes.c_char_p, [_vp]),
    "ma_ctx_launch_count": (ctypes.c_int64, [_vp]),
    "ma_ctx_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
    "ma_ctx_profile_read": (ctypes.c_int, [_vp, ctypes.POINTER(MaProfile)]),
    "ma_mesh_create_grid": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.POINTER(_vp)]),
    "ma_mesh_create_triangles": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip,
                                                ctypes.POINTER(_vp)]),
    "ma_mesh_destroy": (None, [_vp]),
    "ma_mesh_total_mass": (ctypes.c_int, [_vp, _dp]),
    "ma_kantorovich": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _dp,
                                      _vp, _i64p]),
    "ma_hessian_copy": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    "ma_solve_opts_default": (None, [ctypes.POINTER(MaSolveOpts)]),
    "ma_ot_solve": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int,
                                   ctypes.POINTER(MaSolveOpts), ctypes.POINTER(MaStats)]),
    "ma_laplacian_solve": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_int64, _i64p]),
    "ma_laplacian_solve_static": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, ctypes.c_double,
                                                 ctypes.c_int64, _i64p, _vp]),
    "ma_moments": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, _vp, _vp, _vp]),
    "ma_pieces": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
    "ma_pieces_copy": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "ma_polygon_cells": (ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                        _vp]),
    "ma_polygon_cells_copy": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    "ma_ot_solve_batch": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int, _vp, ctypes.c_int, _vp]),
    "ma_draw_laguerre": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        _vp, ctypes.c_int]),
    "ma_mesh_create_image": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "ma_w2_flow": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int64,
                                  ctypes.c_double, _vp, _vp]),
    "ma_mesh_set_values": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int]),
    "ma_kantorovich_vjp": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          _vp, _vp, _vp, _vp, _vp, _vp]),
    "ma_lloyd": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp, ctypes.c_int, _vp, _vp]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"{path} is not built; run mongeampere_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class MaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


MA_OK = 0
MA_ERR_INVALID_ARGUMENT = 1
MA_ERR_NO_DEVICE = 2
MA_ERR_CUDA = 3
MA_ERR_OUT_OF_MEMORY = 4
MA_ERR_CAPACITY = 5
MA_ERR_EXACT_OVERFLOW = 6
MA_EMPTY_CELL = 7
MA_LINESEARCH_FAIL = 8
MA_MAXITER = 9
MA_ERR_BUFFER_TOO_SMALL = 10
MA_CG_NOCONV = 11

MA_MEM_HOST = 0
MA_MEM_DEVICE = 1
MA_FP64 = 0
MA_MIXED = 1
MA_STOP_GRAD_NORM = 0
MA_STOP_MAX_REL = 1
MA_PRECOND_MULTIGRID = 0
MA_PRECOND_JACOBI = 1
MA_INIT_GIVEN = 0
MA_INIT_MULTISCALE = 1
MA_INIT_CONTINUATION = 2
