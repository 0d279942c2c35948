"""ctypes mirror of include/coolpdlp_cuda.h and the loader of libcoolpdlp_cuda.

The shared library is built in-tree by ``coolpdlp.build.build_library()``
(nvcc, sm_103a).  Loading fails loudly when it is missing: there is no CPU
fallback in this package.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_char_p, c_double, c_int32, c_int64,
                    c_uint64, c_void_p)

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libcoolpdlp_cuda.so")
HEADER_PATH = os.path.join(os.path.dirname(PKG_ROOT), "include", "coolpdlp_cuda.h")

# status codes
OK = 0
ERR_ARGUMENT = 1
ERR_DIMENSION = 2
ERR_CUDA = 3
ERR_OUT_OF_MEMORY = 4
ERR_TIMEOUT = 5
ERR_NOT_FOUND = 6
ERR_UNSUPPORTED = 7

# enums
OPTIMAL, TIME_LIMIT, ITERATION_LIMIT, STILL_RUNNING = 0, 1, 2, 3
# extensions (infeasibility_tol > 0)
PRIMAL_INFEASIBLE, DUAL_INFEASIBLE = 4, 5
ALGO_PDLP, ALGO_PDHG = 0, 1
VAL_F64, VAL_F32, VAL_PM1 = 0, 1, 2
# tile_flags bits: CPDLP_TILE_NO_NARROW keeps scaled values for a +-1 matrix;
# CPDLP_TILE_DENSITY_ORDER / _NO_DENSITY_ORDER force the density order on / off
TILE_NO_NARROW = 1
TILE_DENSITY_ORDER = 2
TILE_NO_DENSITY_ORDER = 4
FMT_AUTO, FMT_CSR, FMT_ELL, FMT_COO = -1, 0, 1, 2
VEC_SOL, VEC_SOL_LAST, VEC_SOL_AVG, VEC_SOL_AVG_LAST, VEC_SOL_RESTART = 0, 1, 2, 3, 4


class KKTErrorsC(Structure):
    _fields_ = [(name, c_double) for name in
                ("primal", "primal_scale", "dual", "dual_scale", "gap", "gap_scale")]


class ParamsC(Structure):
    _fields_ = [
        ("algorithm", c_int32),
        ("float_type", c_int32),
        ("chambolle_pock_alpha", c_double),
        ("ruiz_iter", c_int32),
        ("invnorm_scaling", c_double),
        ("primal_weight_damping", c_double),
        ("zero_tol", c_double),
        ("sufficient_decay", c_double),
        ("necessary_decay", c_double),
        ("artificial_decay", c_double),
        ("show_progress", c_int32),
        ("check_every", c_int32),
        ("record_error_history", c_int32),
        ("termination_reltol", c_double),
        ("max_kkt_passes", c_int64),
        ("time_limit", c_double),
        ("power_tol_override", c_double),
        ("power_maxiter_override", c_int64),
        ("power_seed", c_uint64),
        ("refine_reltol", c_double),
        ("tile_nnz", c_int32),
        ("tile_flags", c_int32),
        ("infeasibility_tol", c_double),
        ("matrix_type", c_int32),
    ]


class LPC(Structure):
    _fields_ = [
        ("m", c_int64), ("n", c_int64), ("nnz", c_int64),
        ("colptr", POINTER(c_int64)), ("rowval", POINTER(c_int64)),
        ("nzval", POINTER(c_double)),
        ("c", POINTER(c_double)), ("lv", POINTER(c_double)), ("uv", POINTER(c_double)),
        ("lc", POINTER(c_double)), ("uc", POINTER(c_double)),
    ]


class StatsC(Structure):
    _fields_ = [
        ("err", KKTErrorsC),
        ("time_elapsed", c_double),
        ("kkt_passes", c_int64),
        ("termination_status", c_int32),
        ("restart_from_avg", c_int32),
        ("outer", c_int64), ("inner", c_int64), ("total", c_int64),
        ("eta", c_double), ("eta_sum", c_double), ("omega", c_double),
        ("history_length", c_int64),
        ("power_iterations", c_int64),
        ("refine_kkt_passes", c_int64),
        ("setup_seconds", c_double),
        ("kernel_launches", c_int64),
    ]


def default_params_py(algorithm: int = ALGO_PDLP) -> ParamsC:
    """Pure-Python copy of cpdlp_params_default (common.jl:53-116, pdhg.jl:6-16),
    usable without the CUDA library (e.g. by CPU tests)."""
    p = ParamsC()
    nan = float("nan")
    p.algorithm = algorithm
    p.float_type = VAL_F64
    p.chambolle_pock_alpha = 1.0
    p.ruiz_iter = 10 if algorithm == ALGO_PDLP else 0
    p.invnorm_scaling = 0.9
    p.primal_weight_damping = 0.5 if algorithm == ALGO_PDLP else nan
    p.zero_tol = 1e-8
    p.sufficient_decay = 0.2 if algorithm == ALGO_PDLP else nan
    p.necessary_decay = 0.8 if algorithm == ALGO_PDLP else nan
    p.artificial_decay = 0.36 if algorithm == ALGO_PDLP else nan
    p.show_progress = 0
    p.check_every = 100
    p.record_error_history = 1
    p.termination_reltol = 1e-4
    p.max_kkt_passes = 10 ** 5
    p.time_limit = 100.0
    p.power_tol_override = 0.0
    p.power_maxiter_override = 0
    p.power_seed = 0
    p.refine_reltol = 0.0
    p.tile_nnz = 0
    p.tile_flags = 0
    p.infeasibility_tol = 0.0
    p.matrix_type = FMT_AUTO
    return p


class CpdlpError(RuntimeError):
    """A non-zero status from libcoolpdlp_cuda."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class DimensionMismatch(CpdlpError, ValueError):
    """Mirror of Julia's DimensionMismatch (milp.jl:72-76)."""


class ArgumentError(CpdlpError, ValueError):
    """Mirror of Julia's ArgumentError (milp.jl:83-90, device.jl:9)."""


def raise_for(code: int, message: str):
    if code == OK:
        return
    if code == ERR_DIMENSION:
        raise DimensionMismatch(code, message)
    if code == ERR_ARGUMENT:
        raise ArgumentError(code, message)
    raise CpdlpError(code, message)


# Every symbol the header declares; the CPU tests check that the library exports them.
EXPORTED_SYMBOLS = (
    "cpdlp_abi_version", "cpdlp_params_default", "cpdlp_create", "cpdlp_destroy",
    "cpdlp_last_error", "cpdlp_synchronize", "cpdlp_stream",
    "cpdlp_matrix_from_csc", "cpdlp_matrix_destroy", "cpdlp_matrix_shape",
    "cpdlp_matrix_export", "cpdlp_spmv",
    "cpdlp_problem_create", "cpdlp_problem_destroy", "cpdlp_problem_scaling",
    "cpdlp_state_create", "cpdlp_state_destroy", "cpdlp_state_solve", "cpdlp_state_step",
    "cpdlp_state_kkt", "cpdlp_state_vectors", "cpdlp_state_solution", "cpdlp_state_stats",
    "cpdlp_state_history", "cpdlp_solve", "cpdlp_solve_history", "cpdlp_problem_spectral_norm",
    "cpdlp_problem_layout", "cpdlp_problem_order", "cpdlp_reduced_costs",
    "cpdlp_batch_solve", "cpdlp_state_solve_blocks", "cpdlp_state_profile",
    "cpdlp_state_kernel_bytes", "cpdlp_spmv_csr_noalloc",
    "cpdlp_submit", "cpdlp_poll", "cpdlp_wait", "cpdlp_cancel", "cpdlp_collect",
    "cpdlp_job_count", "cpdlp_job_destroy", "cpdlp_batch_footprint", "cpdlp_job_ready",
    "cpdlp_collect_lp", "cpdlp_sort_rows_columns",
)

_LIB = None


def _declare(lib):
    H = c_void_p
    P64 = POINTER(c_int64)
    PD = POINTER(c_double)
    sig = {
        "cpdlp_abi_version": (c_int32, []),
        "cpdlp_params_default": (None, [POINTER(ParamsC), c_int32]),
        "cpdlp_create": (c_int32, [c_int32, POINTER(H)]),
        "cpdlp_destroy": (c_int32, [H]),
        "cpdlp_last_error": (c_char_p, [H]),
        "cpdlp_synchronize": (c_int32, [H]),
        "cpdlp_stream": (c_void_p, [H]),
        "cpdlp_matrix_from_csc": (c_int32, [H, c_int64, c_int64, c_int64, P64, P64, PD,
                                            c_int32, c_int32, POINTER(H)]),
        "cpdlp_matrix_destroy": (c_int32, [H]),
        "cpdlp_matrix_shape": (c_int32, [H, P64, P64, P64, P64]),
        "cpdlp_matrix_export": (c_int32, [H, H, P64, P64, PD]),
        "cpdlp_spmv": (c_int32, [H, H, c_void_p, c_void_p, c_double, c_double]),
        "cpdlp_problem_create": (c_int32, [H, POINTER(LPC), POINTER(ParamsC), POINTER(H)]),
        "cpdlp_problem_destroy": (c_int32, [H]),
        "cpdlp_problem_scaling": (c_int32, [H, H, PD, PD]),
        "cpdlp_state_create": (c_int32, [H, H, POINTER(ParamsC), PD, PD, POINTER(H)]),
        "cpdlp_state_destroy": (c_int32, [H]),
        "cpdlp_state_solve": (c_int32, [H, H, POINTER(StatsC)]),
        "cpdlp_state_step": (c_int32, [H, H, c_int64]),
        "cpdlp_state_kkt": (c_int32, [H, H, c_int32, POINTER(KKTErrorsC)]),
        "cpdlp_state_vectors": (c_int32, [H, H, c_int32, PD, PD]),
        "cpdlp_state_solution": (c_int32, [H, H, PD, PD]),
        "cpdlp_state_stats": (c_int32, [H, H, POINTER(StatsC)]),
        "cpdlp_state_history": (c_int32, [H, P64, POINTER(KKTErrorsC), c_int64, P64]),
        "cpdlp_solve": (c_int32, [H, POINTER(LPC), POINTER(ParamsC), PD, PD, PD, PD,
                                  POINTER(StatsC)]),
        "cpdlp_solve_history": (c_int32, [H, P64, POINTER(KKTErrorsC), c_int64, P64]),
        "cpdlp_problem_layout": (c_int32, [H, POINTER(c_int32), POINTER(c_int32), P64]),
        "cpdlp_problem_order": (c_int32, [H, H, POINTER(c_int32), P64, P64]),
        "cpdlp_reduced_costs": (c_int32, [H, POINTER(LPC), PD, PD, PD]),
        "cpdlp_problem_spectral_norm": (c_int32, [H, H, POINTER(ParamsC), PD, P64]),
        "cpdlp_batch_solve": (c_int32, [H, c_int64, POINTER(LPC), POINTER(ParamsC),
                                        POINTER(PD), POINTER(PD), POINTER(StatsC)]),
        "cpdlp_state_solve_blocks": (c_int32, [H, H, c_int64, POINTER(StatsC)]),
        "cpdlp_state_profile": (c_int32, [H, H, c_int32, PD]),
        "cpdlp_state_kernel_bytes": (c_int32, [H, PD]),
        "cpdlp_spmv_csr_noalloc": (c_int32, [H, c_int64, c_int64, c_int64, c_void_p, c_void_p,
                                             c_void_p, c_int32, c_void_p, c_void_p, c_double,
                                             c_double]),
        "cpdlp_submit": (c_int32, [H, c_int64, POINTER(LPC), POINTER(ParamsC), PD,
                                   POINTER(PD), POINTER(PD), c_int64, POINTER(H)]),
        "cpdlp_poll": (c_int32, [H, H, POINTER(c_int32)]),
        "cpdlp_wait": (c_int32, [H, H]),
        "cpdlp_cancel": (c_int32, [H, H]),
        "cpdlp_collect": (c_int32, [H, H, POINTER(PD), POINTER(PD), POINTER(StatsC)]),
        "cpdlp_job_count": (c_int64, [H]),
        "cpdlp_job_ready": (c_int32, [H, H, POINTER(c_int32)]),
        "cpdlp_collect_lp": (c_int32, [H, H, c_int64, PD, PD, POINTER(StatsC)]),
        "cpdlp_job_destroy": (c_int32, [H]),
        "cpdlp_batch_footprint": (c_int64, [c_int64, POINTER(LPC), POINTER(ParamsC)]),
        "cpdlp_sort_rows_columns": (c_int32, [H, POINTER(LPC), P64, P64, P64, P64, PD, PD, PD,
                                              PD, PD, PD]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load_library(path: str | None = None):
    """Load libcoolpdlp_cuda.so (in-tree build).  Raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libcoolpdlp_cuda.so not found at {p}: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = _declare(ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL))
    if path is None:
        _LIB = lib
    return lib
