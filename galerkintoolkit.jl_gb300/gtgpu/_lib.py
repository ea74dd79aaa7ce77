"""ctypes binding of ``libgtgpu.so`` (the C ABI declared in include/gtgpu.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the shared library is missing or no CUDA device exists.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

GT_OK = 0
GT_ERR_INVALID = -1
GT_ERR_CUDA = -2
GT_ERR_OOM = -3
GT_ERR_UNSUPPORTED = -4
GT_ERR_NOT_CONVERGED = -5
GT_ERR_TIMEOUT = -6
GT_ERR_BUDGET = -7

GT_QUAD4, GT_HEX8, GT_TET4 = 1, 2, 3
GT_LAPLACE, GT_MASS, GT_ELASTICITY = 1, 2, 3
GT_INT_VOLUME, GT_INT_POLY, GT_INT_FIELD, GT_INT_L2_NORM2, GT_INT_L2_ERROR2, GT_INT_H1_ERROR2 = 0, 1, 2, 3, 4, 5
GT_FP64, GT_FP32, GT_MIXED = 0, 1, 2
GT_SOLVE_FP64, GT_SOLVE_IR, GT_SOLVE_FP32 = 0, 1, 2

_NAMES = {GT_ERR_INVALID: "GT_ERR_INVALID", GT_ERR_CUDA: "GT_ERR_CUDA", GT_ERR_OOM: "GT_ERR_OOM",
          GT_ERR_UNSUPPORTED: "GT_ERR_UNSUPPORTED", GT_ERR_NOT_CONVERGED: "GT_ERR_NOT_CONVERGED",
          GT_ERR_TIMEOUT: "GT_ERR_TIMEOUT", GT_ERR_BUDGET: "GT_ERR_BUDGET"}


class GTError(RuntimeError):
    """Error status returned by the C ABI."""

    def __init__(self, code, msg):
        super().__init__(f"{_NAMES.get(code, code)}: {msg}")
        self.code = code


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("outer_iterations", C.c_int32), ("rel_residual", C.c_double),
                ("fp64_iterations", C.c_int32), ("reserved", C.c_int32)]


P = C.c_void_p
I32 = C.c_int
I64 = C.c_int64
DBL = C.c_double

# (name, restype, argtypes) of every exported symbol declared in include/gtgpu.h
SIGNATURES = [
    ("gt_ctx_create", I32, [I32, C.POINTER(P)]),
    ("gt_ctx_destroy", I32, [P]),
    ("gt_last_error", C.c_char_p, [P]),
    ("gt_ctx_synchronize", I32, [P]),
    ("gt_ctx_set_stream", I32, [P, P]),
    ("gt_ctx_memory", I32, [P, P, P]),
    ("gt_ctx_trim", I32, [P]),
    ("gt_ctx_barrier_probe", I32, [P, I32, I32, I64]),
    ("gt_ctx_launch_count", I32, [P, P]),
    ("gt_ctx_graph_launch_count", I32, [P, P]),
    ("gt_ctx_fma_rate", I32, [P, I32, P]),
    ("gt_ctx_profile_begin", I32, [P]),
    ("gt_ctx_profile_end", I32, [P, I32, P, P, P]),
    ("gt_mesh_create", I32, [P, I32, I64, P, I64, P, I64, P, I64, P, P, I64, P, C.POINTER(P)]),
    ("gt_mesh_set_coords", I32, [P, P]),
    ("gt_mesh_destroy", I32, [P]),
    ("gt_space_create", I32, [P, I32, I32, I32, P, C.POINTER(P)]),
    ("gt_space_info", I32, [P, P]),
    ("gt_space_cell_dofs", I32, [P, P]),
    ("gt_space_destroy", I32, [P]),
    ("gt_assemble_matrix", I32, [P, I32, P, DBL, I32, C.POINTER(P)]),
    ("gt_assemble_matrix_and_vector", I32, [P, I32, P, DBL, I32, P, P, P, C.POINTER(P)]),
    ("gt_linear_problem", I32, [P, I32, P, DBL, I32, P, P, P, P, C.POINTER(P)]),
    ("gt_assemble_csr", I32, [P, I32, P, DBL, I32, P, P, P, I64, P, P, P, P, C.POINTER(P)]),
    ("gt_update_matrix", I32, [P, I32, P, DBL]),
    ("gt_update_matrix_and_vector", I32, [P, I32, P, DBL, P, P, P]),
    ("gt_update_matrix_noalloc", I32, [P, I32, P, DBL]),
    ("gt_matrix_info", I32, [P, P]),
    ("gt_matrix_download_csr", I32, [P, P, P, P, P]),
    ("gt_matrix_destroy", I32, [P]),
    ("gt_assemble_vector", I32, [P, P, P, P]),
    ("gt_integrate", I32, [P, I32, P, P, P, P]),
    ("gt_assemble_boundary_vector", I32, [P, I32, P, P, P, I32]),
    ("gt_solve", I32, [P, P, P, DBL, I32, I32, C.POINTER(SolveInfo)]),
    ("gt_spmv", I32, [P, P, P]),
    ("gt_batch_create", I32, [P, I32, P, C.POINTER(P)]),
    ("gt_batch_set_lanes", I32, [P, I32]),
    ("gt_batch_set_small_rows", I32, [P, I64]),
    ("gt_batch_info", I32, [P, P]),
    ("gt_batch_solve", I32, [P, P, P, DBL, I32, I32, P]),
    ("gt_batch_destroy", I32, [P]),
    ("gt_device_alloc", I32, [P, I64, C.POINTER(P)]),
    ("gt_device_free", I32, [P, P]),
    ("gt_device_copy", I32, [P, P, P, I64]),
    ("gt_lognormal_cells", I32, [P, I64, DBL, C.c_uint64, P]),
]

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building if needed) libgtgpu.so and declare its prototypes."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or not _build.up_to_date():
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build()")
            _build.build()
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def check(ctx, status):
    if status != GT_OK:
        L = load()
        msg = L.gt_last_error(ctx).decode() if ctx else "invalid argument"
        raise GTError(status, msg)
    return status
