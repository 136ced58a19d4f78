"""ctypes binding of libgsgpu.so (include/gsgpu.h). Loading fails loudly when the library is
missing: there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgsgpu.so")

# the exported entry points declared in include/gsgpu.h
EXPORTS = [
    "gsgpu_create", "gsgpu_destroy", "gsgpu_last_error", "gsgpu_set_problem", "gsgpu_refresh", "gsgpu_set_coefs",
    "gsgpu_assemble", "gsgpu_sizes", "gsgpu_matrix_csr", "gsgpu_rhs", "gsgpu_fixed_dofs", "gsgpu_dof_map",
    "gsgpu_solve", "gsgpu_l2_error", "gsgpu_min_jacobian", "gsgpu_assemble_times", "gsgpu_stream",
    "gsgpu_set_profiling", "gsgpu_spmv_stats", "gsgpu_cg_jacobi_noalloc", "gsgpu_set_batch", "gsgpu_batch_info",
    "gsgpu_batch_l2_error", "gsgpu_server_create", "gsgpu_server_submit", "gsgpu_server_wait",
    "gsgpu_server_last_error", "gsgpu_server_destroy", "gsgpu_apply", "gsgpu_mg_apply", "gsgpu_set_fixed_dofs",
    "gsgpu_h1_error", "gsgpu_batch_h1_error", "gsgpu_autotune", "gsgpu_tuned_variants", "gsgpu_tune_save",
    "gsgpu_tune_load", "gsgpu_tune_clear", "gsgpu_server_set_resident", "gsgpu_eval_fields", "gsgpu_mass_csr",
]

# the tuning table measured on GB300 (written by gsgpu_tune_save after gsgpu_autotune runs on the
# benchmark configurations); loaded with the library, so contexts take their kernel variants from it
TUNING_PATH = os.path.join(HERE, "tuning.txt")

OK, ERR_INVALID, ERR_CUDA, ERR_BUDGET, ERR_NOT_CONVERGED, ERR_JACOBIAN, ERR_STATE, ERR_TIMEOUT = range(8)
SOLVER_CG_JACOBI, SOLVER_CG_MG = 0, 1
PREC_FP64, PREC_MIXED = 0, 1


class Problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("npatches", C.c_int),
        ("degree", C.POINTER(C.c_int)), ("nknots", C.POINTER(C.c_int)), ("knots", C.POINTER(C.c_double)),
        ("gdegree", C.POINTER(C.c_int)), ("gnknots", C.POINTER(C.c_int)), ("gknots", C.POINTER(C.c_double)),
        ("coefs", C.POINTER(C.c_double)),
        ("ninterfaces", C.c_int), ("interfaces", C.POINTER(C.c_int)),
        ("ndirichlet", C.c_int), ("dirichlet", C.POINTER(C.c_int)),
        ("kappa_fourier", C.c_int), ("kappa_const", C.c_double), ("kappa_alpha", C.c_double),
        ("kappa_scale", C.c_double), ("kappa_nmodes", C.c_int), ("kappa_amp", C.POINTER(C.c_double)),
        ("kappa_k", C.POINTER(C.c_int)), ("kappa_phase", C.POINTER(C.c_double)),
        ("ufreq", C.c_int), ("quA", C.c_double), ("quB", C.c_int), ("dirichlet_strategy", C.c_int),
        ("nneumann", C.c_int), ("neumann", C.POINTER(C.c_int)),
    ]


class SolverOpts(C.Structure):
    _fields_ = [
        ("method", C.c_int), ("precision", C.c_int), ("tol", C.c_double), ("max_iters", C.c_int),
        ("mg_levels", C.c_int), ("mg_npre", C.c_int), ("mg_npost", C.c_int), ("mg_damping", C.c_double),
        ("inner_tol", C.c_double), ("mg_cycles", C.c_int), ("mg_cgc_damping", C.c_double),
    ]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("relres", C.c_double), ("refinements", C.c_int), ("t_solve_ms", C.c_double)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("nfree", C.c_int), ("iterations", C.c_int), ("relres", C.c_double),
                ("t_submit", C.c_double), ("t_start", C.c_double), ("t_done", C.c_double), ("batch_size", C.c_int),
                ("batch_id", C.c_longlong), ("est_bytes", C.c_double), ("ms_setup", C.c_double),
                ("ms_assemble", C.c_double), ("ms_solve", C.c_double), ("resident", C.c_int)]


class GsGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gsgpu error {code}: {msg}")
        self.code = code


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.gsgpu_create.argtypes = [C.POINTER(vp), C.c_int]
        L.gsgpu_destroy.argtypes = [vp]
        L.gsgpu_last_error.argtypes = [vp]
        L.gsgpu_last_error.restype = C.c_char_p
        L.gsgpu_set_problem.argtypes = [vp, C.POINTER(Problem)]
        L.gsgpu_refresh.argtypes = [vp]
        L.gsgpu_set_coefs.argtypes = [vp, vp]
        L.gsgpu_assemble.argtypes = [vp, C.c_int]
        L.gsgpu_sizes.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gsgpu_matrix_csr.argtypes = [vp, vp, vp, vp]
        L.gsgpu_rhs.argtypes = [vp, vp]
        L.gsgpu_fixed_dofs.argtypes = [vp, vp]
        L.gsgpu_set_fixed_dofs.argtypes = [vp, vp, C.c_int]
        L.gsgpu_dof_map.argtypes = [vp, vp]
        L.gsgpu_solve.argtypes = [vp, C.POINTER(SolverOpts), vp, C.POINTER(SolveInfo)]
        L.gsgpu_l2_error.argtypes = [vp, C.POINTER(C.c_double)]
        L.gsgpu_h1_error.argtypes = [vp, C.POINTER(C.c_double)]
        L.gsgpu_batch_h1_error.argtypes = [vp, vp]
        L.gsgpu_set_batch.argtypes = [vp, C.c_int, vp]
        L.gsgpu_batch_info.argtypes = [vp, vp, vp, vp]
        L.gsgpu_batch_l2_error.argtypes = [vp, vp]
        L.gsgpu_server_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]
        L.gsgpu_server_submit.argtypes = [vp, C.POINTER(Problem), C.c_double, C.POINTER(C.c_longlong)]
        L.gsgpu_server_wait.argtypes = [vp, C.c_longlong, vp, C.c_int, C.POINTER(RequestInfo)]
        L.gsgpu_server_last_error.argtypes = [vp]
        L.gsgpu_server_last_error.restype = C.c_char_p
        L.gsgpu_server_destroy.argtypes = [vp]
        L.gsgpu_server_set_resident.argtypes = [vp, C.c_double]
        L.gsgpu_apply.argtypes = [vp, vp, vp]
        L.gsgpu_mg_apply.argtypes = [vp, C.POINTER(SolverOpts), vp, vp]
        L.gsgpu_min_jacobian.argtypes = [vp, C.POINTER(C.c_double)]
        L.gsgpu_assemble_times.argtypes = [vp, vp]
        L.gsgpu_stream.argtypes = [vp, C.POINTER(vp)]
        L.gsgpu_set_profiling.argtypes = [vp, C.c_int]
        L.gsgpu_spmv_stats.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.gsgpu_cg_jacobi_noalloc.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_double, C.c_int, vp,
                                               C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.gsgpu_autotune.argtypes = [vp, vp]
        L.gsgpu_tuned_variants.argtypes = [vp, vp]
        L.gsgpu_tune_save.argtypes = [C.c_char_p]
        L.gsgpu_tune_load.argtypes = [C.c_char_p]
        L.gsgpu_tune_clear.argtypes = []
        L.gsgpu_eval_fields.argtypes = [C.POINTER(Problem), C.c_int, vp, vp, vp, vp]
        L.gsgpu_mass_csr.argtypes = [vp, vp]
        for name in EXPORTS:
            if name != "gsgpu_last_error":
                getattr(L, name).restype = C.c_int
        if os.path.exists(TUNING_PATH) and not os.environ.get("GSGPU_NO_TUNING_TABLE"):
            if L.gsgpu_tune_load(TUNING_PATH.encode()) != OK:
                raise ImportError(f"{TUNING_PATH} is not a valid tuning table")
        _LIB = L
    return _LIB
