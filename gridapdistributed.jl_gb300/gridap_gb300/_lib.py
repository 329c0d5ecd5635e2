"""ctypes binding of libgdgpu.so (declared in include/gdgpu.h).

Loading fails loudly when the library has not been built: there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "lib" / "libgdgpu.so"

GD_OK = 0
GD_SUB_ASSEMBLED_ROWS = 0
GD_FULLY_ASSEMBLED_ROWS = 1
GD_SOLVE_JACOBI_PCG = 1
GD_SOLVE_MIXED_IR = 2
GD_HOST = 0
GD_DEVICE = 1
GD_QP_FP64 = 0
GD_QP_BF16 = 1
GD_QP_BF16X3 = 2
GD_QP_BF16X6 = 3
QP_PRECISIONS = {"fp64": GD_QP_FP64, "bf16": GD_QP_BF16, "bf16x3": GD_QP_BF16X3, "bf16x6": GD_QP_BF16X6}

STATUS_NAMES = {
    0: "GD_OK", 1: "GD_ERR_ARG", 2: "GD_ERR_OOM", 3: "GD_ERR_CUDA", 4: "GD_ERR_TIMEOUT",
    5: "GD_ERR_STALL", 6: "GD_ERR_STATE", 7: "GD_ERR_UNSUPPORTED", 8: "GD_ERR_NUMERIC",
    9: "GD_ERR_NOTCONVERGED",
}


class GdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class gd_coeffs(C.Structure):
    _fields_ = [("kappa", C.c_void_p), ("f_nodal", C.c_void_p), ("f_const", C.c_double),
                ("degree", C.c_int), ("where", C.c_int)]


class gd_elasticity(C.Structure):
    _fields_ = [("E", C.c_void_p), ("nu", C.c_double), ("force", C.c_double * 3), ("degree", C.c_int),
                ("where", C.c_int)]


class gd_qp_coeffs(C.Structure):
    _fields_ = [("kappa_qp", C.c_void_p), ("f_nodal", C.c_void_p), ("f_const", C.c_double), ("degree", C.c_int),
                ("precision", C.c_int), ("where", C.c_int)]


class gd_elasticity_qp(C.Structure):
    _fields_ = [("E_qp", C.c_void_p), ("nu", C.c_double), ("force", C.c_double * 3), ("degree", C.c_int),
                ("precision", C.c_int), ("where", C.c_int)]


class gd_dg_form(C.Structure):
    _fields_ = [("gamma", C.c_double), ("h", C.c_double), ("degree", C.c_int), ("f_const", C.c_double),
                ("f_qp", C.c_void_p), ("dirichlet_sides", C.c_void_p), ("ud_qp", C.c_void_p),
                ("neumann_sides", C.c_void_p), ("g_qp", C.c_void_p), ("where", C.c_int)]


class gd_solve_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("rel_residual", C.c_double),
                ("seconds", C.c_double)]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
I64P = C.POINTER(C.c_int64)
I32P = C.POINTER(C.c_int32)
DP = C.POINTER(C.c_double)

# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "gd_last_error": [],
    "gd_version": [],
    "gd_ctx_create": [C.c_int, PP],
    "gd_ctx_destroy": [P],
    "gd_ctx_set_stream": [P, P],
    "gd_ctx_synchronize": [P],
    "gd_model_cartesian": [P, C.c_int, I64P, I32P, DP, PP],
    "gd_model_destroy": [P],
    "gd_model_num_parts": [P, I32P],
    "gd_model_part_boxes": [P, C.c_int, I64P, I64P, I64P, I64P],
    "gd_space_create": [P, C.c_int, C.c_int, I32P, PP],
    "gd_space_destroy": [P],
    "gd_space_num_free_dofs": [P, I64P],
    "gd_space_local_sizes": [P, C.c_int, I64P, I64P, I64P],
    "gd_space_get_gids": [P, C.c_int, I64P, I32P],
    "gd_space_dof_nodes": [P, C.c_int, I64P],
    "gd_space_set_dirichlet": [P, DP, C.c_int],
    "gd_assembler_create": [P, P, C.c_int, PP],
    "gd_assembler_destroy": [P],
    "gd_assemble_symbolic": [P],
    "gd_assemble_numeric": [P, C.POINTER(gd_coeffs)],
    "gd_assemble_numeric_async": [P, C.POINTER(gd_coeffs)],
    "gd_assemble_vector": [P, C.POINTER(gd_coeffs), DP, C.c_int],
    "gd_assembler_set_profiling": [P, C.c_int],
    "gd_assembler_phase_times": [P, DP, DP, DP],
    "gd_assembler_counts": [P, I64P, I64P, I64P, I32P],
    "gd_assembler_tuning": [P, I32P, I32P, I32P, C.POINTER(C.c_float), I32P],
    "gd_assembler_set_shape": [P, C.c_int],
    "gd_matrix_sizes": [P, C.c_int, I64P, I64P, I64P, I64P, I64P],
    "gd_matrix_export": [P, C.c_int, I64P, I32P, DP, I64P, I32P, I64P, I32P],
    "gd_vector_export": [P, C.c_int, DP],
    "gd_system_device_ptrs": [P, PP, PP, PP, PP, I64P],
    "gd_system_download": [P, DP, DP],
    "gd_assembler_set_class_sums": [P, C.c_int],
    "gd_assemble_download": [P, C.POINTER(gd_coeffs), DP, DP],
    "gd_spmv": [P, P, P, C.c_int],
    "gd_solve": [P, C.c_int, C.c_double, C.c_int, P, C.c_int, C.POINTER(gd_solve_stats)],
    "gd_fe_function_local": [P, C.c_int, P, C.c_int, DP],
    "gd_solve_rhs": [P, C.c_int, C.c_double, C.c_int, P, P, C.c_int, C.POINTER(gd_solve_stats)],
    "gd_solve_noalloc": [P, C.c_double, C.c_int, P, C.c_int, C.POINTER(gd_solve_stats)],
    "gd_assemble_elasticity": [P, P],
    "gd_assemble_qp": [P, P],
    "gd_assemble_elasticity_qp": [P, P],
    "gd_qp_info": [P, I32P, I32P, I32P, I32P, DP, DP],
    "gd_l2_error": [P, P, P, C.c_int, C.c_int, DP],
    "gd_add_boundary_source": [P, I32P, P, C.c_int, C.c_int],
    "gd_batch_create": [P, P, C.c_int, PP],
    "gd_batch_destroy": [P],
    "gd_batch_assemble": [P],
    "gd_batch_assemble_async": [P],
    "gd_batch_counts": [P, I32P, I64P, I64P],
    "gd_batch_tuning": [P, I32P, I32P, I32P, C.POINTER(C.c_float), I32P],
    "gd_batch_solve": [P, C.c_double, C.c_int, P],
    "gd_batch_solution": [P, C.c_int, P, C.c_int],
    "gd_learned_create": [P, C.c_int, C.c_int, C.c_uint64, PP],
    "gd_learned_levels": [P, I32P],
    "gd_learned_flags": [P, I32P],
    "gd_learned_destroy": [P],
    "gd_learned_num_params": [P, I64P],
    "gd_learned_get_params": [P, C.POINTER(C.c_float)],
    "gd_learned_set_params": [P, C.POINTER(C.c_float)],
    "gd_learned_apply": [P, P, P],
    "gd_learned_apply_reference": [P, P, P],
    "gd_learned_gradient": [P, P, P, C.c_int, DP, C.POINTER(C.c_float)],
    "gd_learned_train_step": [P, P, P, C.c_int, C.c_float, DP],
    "gd_solve_learned": [P, P, C.c_double, C.c_int, P, C.c_int, C.POINTER(gd_solve_stats), I32P],
    "gd_mfield_create": [P, C.c_int, PP],
    "gd_mfield_destroy": [P],
    "gd_mfield_assemble": [P, DP, DP, DP, C.POINTER(gd_coeffs)],
    "gd_mfield_block_export": [P, C.c_int, C.c_int, C.c_int, DP, DP],
    "gd_mfield_gids": [P, C.c_int, I32P, C.c_int, I64P, I32P],
    "gd_mfmat_create": [P, C.c_int, I32P, C.c_int, I32P, PP],
    "gd_mfmat_destroy": [P],
    "gd_mfmat_refresh": [P],
    "gd_mfmat_counts": [P, I64P, I64P],
    "gd_mfmat_sizes": [P, C.c_int, I64P, I64P, I64P, I64P, I64P],
    "gd_mfmat_export": [P, C.c_int, I64P, I32P, DP, I64P, I32P, I64P, I32P, DP],
    "gd_mfmat_spmv": [P, P, P, C.c_int],
    "gd_dg_space_create": [P, C.c_int, PP],
    "gd_dg_space_destroy": [P],
    "gd_dg_num_free_dofs": [P, I64P],
    "gd_dg_local_sizes": [P, C.c_int, I64P, I64P, I64P],
    "gd_dg_get_gids": [P, C.c_int, I64P, I32P],
    "gd_dg_assemble": [P, C.POINTER(gd_dg_form)],
    "gd_dg_set_strategy": [P, C.c_int],
    "gd_dg_matrix_sizes": [P, C.c_int, I64P, I64P, I64P, I64P, I64P],
    "gd_dg_matrix_export": [P, C.c_int, I64P, I32P, DP, I64P, I32P, I64P, I32P, DP],
    "gd_dg_spmv": [P, P, P, C.c_int],
    "gd_dg_solve": [P, C.c_double, C.c_int, P, C.c_int, C.POINTER(gd_solve_stats)],
    "gd_dg_l2_error": [P, P, P, C.c_int, C.c_int, DP],
    "gd_debug_barrier_probe": [P, C.c_int, C.c_int, C.c_double],
}
_RESTYPES = {"gd_last_error": C.c_char_p, "gd_version": C.c_char_p}

_lib = None


def load(path: str | os.PathLike | None = None):
    """Load libgdgpu.so once.  Raises if the library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libgdgpu.so not found at {p}: run __graft_entry__.build() first "
                           "(this package has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def check(status: int):
    if status != GD_OK:
        msg = _lib.gd_last_error().decode() if _lib is not None else ""
        raise GdError(status, msg)


def call(name, *args):
    lib = load()
    check(getattr(lib, name)(*args))


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def vptr(a) -> C.c_void_p:
    """Void pointer of a numpy array (host) or an int device address."""
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(int(a))
