"""coolpdlp -- a GB300-native (sm_103a) PDLP/PDHG LP solver with CoolPDLP.jl's API.

Exports mirror src/CoolPDLP.jl:53-63.  The numerical work runs in the CUDA
library libcoolpdlp_cuda (coolpdlp.jl_gb300/lib/), built by
``coolpdlp.build.build_library()``; there is no CPU fallback.
"""
from . import _abi
from ._abi import ArgumentError, CpdlpError, DimensionMismatch
from .algorithms import (ITERATION_LIMIT, OPTIMAL, STILL_RUNNING, TIME_LIMIT, PDHG, PDLP,
                         Algorithm, ConvergenceStats, DeviceMILP, KKTErrors, SolverState,
                         TerminationStatus, absolute, get_solution, initialize, preprocess,
                         relative, solve, solve_, solve_inplace)
from .matrices import GPUSparseMatrixCOO, GPUSparseMatrixCSR, GPUSparseMatrixELL
from .problems import (CSCMatrix, MILP, PrimalDualSolution, axpby, is_feasible, nbcons,
                       nbcons_eq, nbcons_ineq, nbvar, nbvar_cont, nbvar_int, objective_value,
                       sort_rows_columns)

__all__ = [
    "GPUSparseMatrixCOO", "GPUSparseMatrixCSR", "GPUSparseMatrixELL",
    "MILP", "nbvar", "nbvar_int", "nbvar_cont", "nbcons", "nbcons_eq", "nbcons_ineq",
    "PrimalDualSolution", "preprocess", "initialize", "solve", "solve_", "solve_inplace",
    "PDHG", "PDLP", "Algorithm", "is_feasible", "objective_value", "TerminationStatus",
    "KKTErrors", "ConvergenceStats", "OPTIMAL", "TIME_LIMIT", "ITERATION_LIMIT",
    "STILL_RUNNING", "DimensionMismatch", "ArgumentError", "CpdlpError", "CSCMatrix",
    "sort_rows_columns",
]
