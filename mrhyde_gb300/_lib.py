"""ctypes binding of libmrhyde_gb.so (the C ABI in include/mrhyde_gb300.h).

The structures below mirror the header field by field.  Loading fails loudly when the library is
missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

from .buildlib import LIB_PATH, build

MRG_OK, MRG_EINVAL, MRG_ENOMEM, MRG_ECUDA, MRG_ETIMEOUT, MRG_ENOTSUP, MRG_ENOCONV, MRG_ENUMERIC = range(8)
STATUS_NAMES = {0: "MRG_OK", 1: "MRG_EINVAL", 2: "MRG_ENOMEM", 3: "MRG_ECUDA", 4: "MRG_ETIMEOUT",
                5: "MRG_ENOTSUP", 6: "MRG_ENOCONV", 7: "MRG_ENUMERIC"}

MRG_THERMAL, MRG_DIFFUSION_1PU2 = 0, 1
MRG_SRC_CONST, MRG_SRC_SINPROD = 0, 1
MRG_DBC_CONST, MRG_DBC_NODE = 0, 1
MRG_FACE_XLO, MRG_FACE_XHI, MRG_FACE_YLO, MRG_FACE_YHI, MRG_FACE_ZLO, MRG_FACE_ZHI = 1, 2, 4, 8, 16, 32
MRG_FACE_ALL = 63
MRG_BC_NONE, MRG_BC_NEUMANN, MRG_BC_WEAK_DIRICHLET = 0, 1, 2
MRG_PATH_FACTORED, MRG_PATH_CELL, MRG_PATH_TENSOR, MRG_PATH_STORED = 1, 2, 3, 4

MRG_ASM_RES = 1
MRG_ASM_JAC = 2
MRG_ASM_J_FP32 = 4
MRG_ASM_OVERWRITE = 8
MRG_ASM_FIX_ZERO_ROWS = 16
MRG_ASM_FORCE_CELL = 256
MRG_ASM_ATOMIC = 512
MRG_ASM_ADJOINT = 1024
MRG_ASM_SENS = 2048
MRG_ASM_TENSOR_CORES = 4096
MRG_ASM_CUDA_CORES = 8192
MRG_ASM_NATIVE_FP64 = 16384
MRG_NOALLOC_MAX_DOFS = 1 << 18
MRG_WAIT_LIMIT_MAX_NS = 60_000_000_000


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("order", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nz", C.c_int32), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("vertex_coords", C.POINTER(C.c_double))]


class PhysicsDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("source_kind", C.c_int32), ("source_amp", C.c_double),
                ("source_freq", C.c_double), ("kappa_const", C.c_double),
                ("kappa_cell", C.POINTER(C.c_double)), ("dirichlet_faces", C.c_uint32),
                ("dirichlet_kind", C.c_int32), ("dirichlet_const", C.c_double),
                ("dirichlet_node", C.POINTER(C.c_double)), ("quad_order", C.c_int32), ("reserved", C.c_int32)]


class ProblemInfo(C.Structure):
    _fields_ = [("n_dofs", C.c_int64), ("n_cells", C.c_int64), ("nnz", C.c_int64), ("n_fixed", C.c_int64),
                ("nodes_per_cell", C.c_int32), ("qp_per_cell", C.c_int32), ("path", C.c_int32),
                ("reserved", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("outer_iterations", C.c_int32), ("rel_residual", C.c_double),
                ("abs_residual", C.c_double), ("status", C.c_int32), ("reserved", C.c_int32)]


MRG_KRYLOV_AUTO, MRG_KRYLOV_PCG, MRG_KRYLOV_BICGSTAB = 0, 1, 2
MRG_PREC_JACOBI, MRG_PREC_GMG, MRG_PREC_GMG_SPLIT = 0, 1, 2


class NewtonOpts(C.Structure):
    _fields_ = [("nl_tol", C.c_double), ("max_iters", C.c_int32), ("mixed", C.c_int32),
                ("lin_tol", C.c_double), ("lin_maxiter", C.c_int32), ("reuse_jacobian", C.c_int32),
                ("krylov", C.c_int32), ("gmg_full_setup", C.c_int32)]


class BatchDesc(C.Structure):
    _fields_ = [("n_problems", C.c_int32), ("sizes", C.POINTER(C.c_int32)), ("kappa", C.POINTER(C.c_double)),
                ("dirichlet", C.POINTER(C.c_double)), ("source", C.c_double)]


class BatchInfo(C.Structure):
    _fields_ = [("n_problems", C.c_int32), ("threads", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("reserved", C.c_int32), ("n_cells", C.c_int64), ("n_nodes", C.c_int64), ("nnz", C.c_int64)]


class BatchOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("inner_tol", C.c_double), ("max_outer", C.c_int32), ("max_inner", C.c_int32)]


class BatchStat(C.Structure):
    _fields_ = [("outer_iterations", C.c_int32), ("inner_iterations", C.c_int32), ("rel_residual", C.c_double),
                ("status", C.c_int32), ("reserved", C.c_int32)]


# name -> (restype, argtypes) for every entry point of include/mrhyde_gb300.h
_VP = C.c_void_p
SIGNATURES = {
    "mrg_problem_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(PhysicsDesc), C.POINTER(_VP)]),
    "mrg_problem_create_on_stream": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(PhysicsDesc), _VP, C.POINTER(_VP)]),
    "mrg_problem_destroy": (C.c_int, [_VP]),
    "mrg_problem_get_info": (C.c_int, [_VP, C.POINTER(ProblemInfo)]),
    "mrg_get_graph": (C.c_int, [_VP, _VP, _VP, _VP]),
    "mrg_get_dof_map": (C.c_int, [_VP, _VP, _VP]),
    "mrg_get_fixed_dofs": (C.c_int, [_VP, _VP, _VP, _VP]),
    "mrg_set_kappa": (C.c_int, [_VP, _VP, _VP]),
    "mrg_set_dirichlet": (C.c_int, [_VP, _VP, _VP]),
    "mrg_get_side_points": (C.c_int, [_VP, C.c_int32, C.POINTER(C.c_int64), _VP]),
    "mrg_set_face_bc": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP]),
    "mrg_set_preconditioner": (C.c_int, [_VP, C.c_int32]),
    "mrg_assemble": (C.c_int, [_VP, _VP, _VP, _VP, C.c_uint32, _VP]),
    "mrg_assemble_residual": (C.c_int, [_VP, _VP, _VP, C.c_uint32, _VP]),
    "mrg_spmv": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP, _VP]),
    "mrg_solve_pcg": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP, C.c_double, C.c_int32, C.POINTER(SolveStats), _VP]),
    "mrg_newton": (C.c_int, [_VP, _VP, C.POINTER(NewtonOpts), C.POINTER(SolveStats), _VP]),
    "mrg_solve_bicgstab": (C.c_int, [_VP, _VP, C.c_int32, _VP, _VP, C.c_double, C.c_int32, C.POINTER(SolveStats), _VP]),
    "mrg_solve_pcg_noalloc": (C.c_int, [_VP, _VP, _VP, _VP, C.c_double, C.c_int32, C.POINTER(SolveStats), _VP]),
    "mrg_batch_create": (C.c_int, [C.POINTER(BatchDesc), C.POINTER(_VP)]),
    "mrg_batch_destroy": (C.c_int, [_VP]),
    "mrg_batch_get_info": (C.c_int, [_VP, C.POINTER(BatchInfo), _VP, _VP]),
    "mrg_batch_solve": (C.c_int, [_VP, _VP, _VP, C.POINTER(BatchOpts), _VP, _VP]),
    "mrg_batch_autotune": (C.c_int, [_VP, _VP, _VP, C.POINTER(BatchOpts), _VP]),
    "mrg_batch_set_config": (C.c_int, [_VP, C.c_int32, C.c_int32]),
    "mrg_measure_fma_rates": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), _VP]),
    "mrg_set_wait_policy": (C.c_int, [_VP, C.c_uint64, C.c_int32]),
    "mrg_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "mrg_version": (C.c_char_p, []),
}

_lib = None


class MrgError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")


def lib(rebuild: bool = True):
    """Load libmrhyde_gb.so (building it first if sources changed).  Raises if it cannot be loaded."""
    global _lib
    if _lib is None:
        path = build() if rebuild else LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError(f"libmrhyde_gb.so not found at {path}; run mrhyde_gb300.build.build()")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().mrg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int, where: str):
    if status != MRG_OK:
        raise MrgError(status, where, last_error())
    return status
