"""ctypes binding of libpmgpu.so (the C ABI declared in include/pmgpu.h).

The library is built in-tree by mymoonmd_gb300/build.py. There is no CPU
fallback: importing this module without the built library raises ImportError.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libpmgpu.so"

PM_OK = 0
PM_E_INVALID = 1
PM_E_OOM = 2
PM_E_DIVERGED = 3
PM_E_BREAKDOWN = 4
PM_E_MAXIT = 5
PM_E_CUDA = 6
PM_E_TIMEOUT = 7
PM_E_UNSUPPORTED = 8

_STATUS_NAMES = {
    PM_E_INVALID: "PM_E_INVALID", PM_E_OOM: "PM_E_OOM", PM_E_DIVERGED: "PM_E_DIVERGED",
    PM_E_BREAKDOWN: "PM_E_BREAKDOWN", PM_E_MAXIT: "PM_E_MAXIT", PM_E_CUDA: "PM_E_CUDA",
    PM_E_TIMEOUT: "PM_E_TIMEOUT", PM_E_UNSUPPORTED: "PM_E_UNSUPPORTED",
}


class PmError(RuntimeError):
    """Failure reported by the library (the reference throws std::runtime_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class CdCoeffs(C.Structure):
    _fields_ = [("eps", C.c_double), ("b", C.c_double * 3), ("c", C.c_double),
                ("manufactured", C.c_int), ("f_const", C.c_double), ("poly", C.c_double * 10),
                ("poly_src", C.c_double * 10)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("geometry", C.c_int), ("root_n", C.c_int), ("n_refine", C.c_int),
                ("n_levels", C.c_int), ("elem", C.c_int), ("coeffs", CdCoeffs), ("nu", C.c_double),
                ("solution_out", C.POINTER(C.c_double)), ("tag", C.c_uint64)]


class Result(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("status", C.c_int), ("iterations", C.c_int), ("residual", C.c_double),
                ("initial_residual", C.c_double), ("n_dofs", C.c_int), ("worker", C.c_int),
                ("cache_hit", C.c_int), ("queue_ms", C.c_double), ("setup_ms", C.c_double),
                ("run_ms", C.c_double), ("latency_ms", C.c_double)]


def _load() -> C.CDLL:
    if not _LIB_PATH.exists():
        raise ImportError(
            f"{_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (there is no CPU fallback)")
    return C.CDLL(str(_LIB_PATH))


lib = _load()

vp = C.c_void_p
i32 = C.c_int
i64 = C.c_int64
f64 = C.c_double
pi32 = C.POINTER(C.c_int)
pf64 = C.POINTER(C.c_double)

_SIGS = {
    "pm_version": (i32, []),
    "pm_ctx_create": (i32, [i32, C.POINTER(vp)]),
    "pm_ctx_destroy": (None, [vp]),
    "pm_last_error": (C.c_char_p, [vp]),
    "pm_ctx_synchronize": (i32, [vp]),
    "pm_ctx_set_option": (i32, [vp, C.c_char_p, i32]),
    "pm_ctx_kernel_launches": (i32, [vp, C.POINTER(C.c_uint64)]),
    "pm_ctx_time_begin": (i32, [vp]),
    "pm_ctx_time_end": (i32, [vp, C.POINTER(C.c_float)]),
    "pm_dev_alloc": (i32, [vp, C.c_size_t, C.POINTER(vp)]),
    "pm_dev_free": (i32, [vp, vp]),
    "pm_memcpy_h2d": (i32, [vp, vp, vp, C.c_size_t]),
    "pm_memcpy_d2h": (i32, [vp, vp, vp, C.c_size_t]),
    "pm_memset_dev": (i32, [vp, vp, i32, C.c_size_t]),
    "pm_host_alloc": (i32, [vp, C.c_size_t, C.POINTER(vp)]),
    "pm_host_free": (i32, [vp, vp]),
    "pm_matrix_create_csr": (i32, [vp, i32, i32, i32, vp, vp, vp, C.POINTER(vp)]),
    "pm_matrix_destroy": (None, [vp]),
    "pm_matrix_set_blocks": (i32, [vp, i32, vp, vp]),
    "pm_matrix_info": (i32, [vp, pi32, pi32, pi32, C.POINTER(i64)]),
    "pm_matrix_set_values": (i32, [vp, vp]),
    "pm_matrix_get_values": (i32, [vp, vp]),
    "pm_matrix_get_structure": (i32, [vp, vp, vp]),
    "pm_matrix_apply_scaled_add": (i32, [vp, vp, vp, f64]),
    "pm_matrix_apply": (i32, [vp, vp, vp]),
    "pm_matrix_get_diagonal": (i32, [vp, vp]),
    "pm_matrix_make_fp32": (i32, [vp]),
    "pm_matrix_make_sliced64": (i32, [vp]),
    "pm_matrix_apply_f32": (i32, [vp, vp, vp]),
    "pm_matrix_set_kernel": (i32, [vp, i32, i32]),
    "pm_matrix_bench_apply": (i32, [vp, i32, vp, vp, i32, C.POINTER(C.c_float), pf64]),
    "pm_dot": (i32, [vp, i32, vp, vp, pf64]),
    "pm_norm": (i32, [vp, i32, vp, pf64]),
    "pm_axpy": (i32, [vp, i32, f64, vp, vp]),
    "pm_scal": (i32, [vp, i32, f64, vp]),
    "pm_solver_create": (i32, [vp, C.c_char_p, C.POINTER(vp)]),
    "pm_solver_destroy": (None, [vp]),
    "pm_solver_update_matrix": (i32, [vp, vp]),
    "pm_solver_set_multigrid_level": (i32, [vp, i32, i32, vp, i32, i32, vp, vp, vp]),
    "pm_solver_solve": (i32, [vp, vp, vp]),
    "pm_solver_solve_host": (i32, [vp, vp, vp, i32]),
    "pm_solver_last_info": (i32, [vp, pi32, pf64, pf64]),
    "pm_solver_residual_history": (i32, [vp, vp, i32, pi32]),
    "pm_solver_apply_preconditioner": (i32, [vp, vp, vp]),
    "pm_disc_create": (i32, [i32, i32, i32, i32, i32, i32, C.POINTER(vp)]),
    "pm_disc_create_bc": (i32, [i32, i32, i32, i32, i32, i32, i32, C.POINTER(vp)]),
    "pm_disc_create_device": (i32, [vp, i32, i32, i32, i32, i32, i32, i32, C.POINTER(vp)]),
    "pm_disc_destroy": (None, [vp]),
    "pm_disc_level_info": (i32, [vp, i32, i32, pi32, pi32, pi32, pi32, C.POINTER(i64)]),
    "pm_disc_dofmap": (i32, [vp, i32, i32, vp]),
    "pm_disc_cell_vertices": (i32, [vp, i32, vp]),
    "pm_disc_structure": (i32, [vp, i32, vp, vp]),
    "pm_disc_prolongation_info": (i32, [vp, i32, pi32, pi32, C.POINTER(i64)]),
    "pm_disc_prolongation": (i32, [vp, i32, vp, vp, vp]),
    "pm_assemble_cd": (i32, [vp, vp, i32, C.POINTER(CdCoeffs), i32, vp, vp]),
    "pm_assemble_cd_noalloc": (i32, [vp, i32, C.POINTER(CdCoeffs), vp, vp]),
    "pm_problem_create_cd": (i32, [vp, vp, C.POINTER(CdCoeffs), i32, C.c_char_p, C.POINTER(vp)]),
    "pm_problem_destroy": (None, [vp]),
    "pm_problem_create_stokes": (i32, [vp, vp, f64, C.c_char_p, C.POINTER(vp)]),
    "pm_problem_assemble": (i32, [vp]),
    "pm_problem_solve": (i32, [vp]),
    "pm_problem_reset_solution": (i32, [vp]),
    "pm_problem_size": (i32, [vp, pi32, pi32]),
    "pm_problem_get_solution": (i32, [vp, vp]),
    "pm_problem_get_rhs": (i32, [vp, vp]),
    "pm_problem_set_solution": (i32, [vp, vp]),
    "pm_problem_matrix": (i32, [vp, i32, C.POINTER(vp)]),
    "pm_problem_solver": (i32, [vp, C.POINTER(vp)]),
    "pm_problem_solution_dev": (i32, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "pm_problem_run_host": (i32, [vp, C.POINTER(CdCoeffs), vp, vp]),
    "pm_problem_errors": (i32, [vp, vp]),
    "pm_problem_assemble_nonlinear": (i32, [vp]),
    "pm_problem_residuals": (i32, [vp, vp]),
    "pm_problem_solve_nonlinear": (i32, [vp, i32, vp, pi32]),
    "pm_problem_last_info": (i32, [vp, pi32, pf64, pf64]),
    "pm_problem_solve_batched": (i32, [vp, i32, i32, pi32]),
    "pm_tcd_create": (i32, [vp, vp, C.POINTER(CdCoeffs), vp, i32, C.c_char_p, C.POINTER(vp)]),
    "pm_tcd_destroy": (None, [vp]),
    "pm_tcd_assemble_initial_time": (i32, [vp]),
    "pm_tcd_next_step": (i32, [vp]),
    "pm_tcd_assemble": (i32, [vp]),
    "pm_tcd_solve": (i32, [vp]),
    "pm_tcd_state": (i32, [vp, pf64, pi32]),
    "pm_tcd_problem": (i32, [vp, C.POINTER(vp)]),
    "pm_server_create": (i32, [i32, i32, C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(vp)]),
    "pm_server_destroy": (None, [vp]),
    "pm_server_submit": (i32, [vp, C.POINTER(Request)]),
    "pm_server_poll": (i32, [vp, C.POINTER(Result), i32, i32, pi32]),
    "pm_server_drain": (i32, [vp]),
    "pm_server_stats": (i32, [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "pm_ctx_probe": (i32, [vp, i64]),
    "pm_ctx_probe_result": (i32, [vp, pi32, pf64, pf64]),
}

for _name, (_res, _args) in _SIGS.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def check(rc: int, ctx=None) -> None:
    if rc != PM_OK:
        msg = lib.pm_last_error(ctx).decode(errors="replace")
        raise PmError(rc, msg)


def declared_symbols() -> list[str]:
    return sorted(_SIGS)
