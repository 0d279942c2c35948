"""Algorithm configuration and the solve entry points.

Mirror of src/algorithms/common.jl, pdlp.jl, pdhg.jl and the parameter structs
of src/components/*.jl.  All numerical work runs in libcoolpdlp_cuda on the
GPU; this module only builds parameter structs and moves host arrays.
"""
from __future__ import annotations

import dataclasses
import enum
import math
import time

import numpy as np

from . import _abi as A
from . import native
from .problems import MILP, PrimalDualSolution


class TerminationStatus(enum.IntEnum):
    """termination.jl:13 (same order and values)."""
    OPTIMAL = A.OPTIMAL
    TIME_LIMIT = A.TIME_LIMIT
    ITERATION_LIMIT = A.ITERATION_LIMIT
    STILL_RUNNING = A.STILL_RUNNING
    # extensions of this library (infeasibility_tol > 0); the reference has none
    PRIMAL_INFEASIBLE = A.PRIMAL_INFEASIBLE
    DUAL_INFEASIBLE = A.DUAL_INFEASIBLE


OPTIMAL = TerminationStatus.OPTIMAL
TIME_LIMIT = TerminationStatus.TIME_LIMIT
ITERATION_LIMIT = TerminationStatus.ITERATION_LIMIT
STILL_RUNNING = TerminationStatus.STILL_RUNNING

# FP32 iterates whose relative KKT error has not halved over this many checks
# continue in FP64 when refine_reltol > 0 (the library's rule, solver.cuh)
STALL_CHECKS = 30


@dataclasses.dataclass(frozen=True)
class KKTErrors:
    """errors.jl:8-21 (unscaled units)."""
    primal: float = math.nan
    primal_scale: float = math.nan
    dual: float = math.nan
    dual_scale: float = math.nan
    gap: float = math.nan
    gap_scale: float = math.nan

    @classmethod
    def from_c(cls, e) -> "KKTErrors":
        return cls(e.primal, e.primal_scale, e.dual, e.dual_scale, e.gap, e.gap_scale)

    def isapprox(self, other: "KKTErrors", rtol: float = 1.4901161193847656e-08) -> bool:
        return all(math.isclose(getattr(self, f), getattr(other, f), rel_tol=rtol)
                   for f in ("primal", "dual", "gap", "primal_scale", "dual_scale", "gap_scale"))

    def __str__(self):
        return (f"KKT relative errors: primal {self.primal / self.primal_scale:.3e}, "
                f"dual {self.dual / self.dual_scale:.3e}, gap {self.gap / self.gap_scale:.3e}")


def relative(err: KKTErrors) -> float:
    """errors.jl:55-58"""
    return max(err.primal / err.primal_scale, err.dual / err.dual_scale, err.gap / err.gap_scale)


def absolute(err: KKTErrors, omega: float) -> float:
    """errors.jl:60-63"""
    return math.sqrt(omega ** 2 * err.primal ** 2 + err.dual ** 2 / omega ** 2 + err.gap ** 2)


@dataclasses.dataclass
class ConvergenceStats:
    """termination.jl:44-76 plus the iteration counter and step sizes."""
    err: KKTErrors
    starting_time: float
    time_elapsed: float
    kkt_passes: int
    termination_status: TerminationStatus
    error_history: list
    outer: int = 0
    inner: int = 0
    total: int = 0
    eta: float = math.nan
    omega: float = math.nan
    power_iterations: int = 0
    setup_seconds: float = 0.0
    refine_kkt_passes: int = 0

    def __str__(self):
        return (f"Convergence stats with termination status {self.termination_status.name}:\n"
                f"- {self.err}\n- time elapsed: {self.time_elapsed:.3f} seconds \n"
                f"- KKT passes: {self.kkt_passes}")


class Algorithm:
    """Algorithm{A}(T, Ti, M; kwargs...) (common.jl:8-116).

    name: "PDLP" or "PDHG"; T: np.float64 / np.float32 (iterate precision);
    Ti: index type (the device always uses int32 indices, so only its range is
    checked); M: the matrix type of the solve's products (conversion.jl:37-55):
    "CSR" (the CSR tile engine), "ELL" (the reference's ELL layout, one thread
    per row), "COO" (solved on the CSR engine: the reference's COO product
    sums with atomics in a run-dependent order), a GPUSparseMatrix* class, or
    None / "AUTO" (default): the autotuner picks per matrix among CSR tile
    shapes and ELL for matrices of at least 2^21 nonzeros."""

    KEYWORDS = ("chambolle_pock_alpha", "ruiz_iter", "invnorm_scaling", "primal_weight_damping",
                "zero_tol", "sufficient_decay", "necessary_decay", "artificial_decay",
                "show_progress", "check_every", "record_error_history", "termination_reltol",
                "max_kkt_passes", "time_limit", "power_tol_override", "power_maxiter_override",
                "power_seed", "refine_reltol", "tile_nnz", "tile_flags", "infeasibility_tol")

    FORMATS = {"AUTO": A.FMT_AUTO, "CSR": A.FMT_CSR, "ELL": A.FMT_ELL, "COO": A.FMT_COO}

    def __init__(self, name: str = "PDLP", T=np.float64, Ti=np.int64, M=None, *, device: int = 0,
                 backend=None, **kw):
        name = name.upper()
        if name not in ("PDLP", "PDHG"):
            raise A.ArgumentError(A.ERR_ARGUMENT, f"unknown algorithm {name}")
        self.name = name
        T = np.dtype(T).type
        if T not in (np.float64, np.float32):
            raise A.ArgumentError(A.ERR_ARGUMENT, "T must be Float64 or Float32")
        self.T = T
        self.Ti = Ti
        if M is None:
            M = "AUTO"
        self.M = (M if isinstance(M, str) else getattr(M, "FORMAT", "CSR")).upper()
        if self.M not in self.FORMATS:
            raise A.ArgumentError(A.ERR_ARGUMENT, f"unknown matrix type {M}")
        self.device = device if backend is None else int(getattr(backend, "device", backend))
        algo = A.ALGO_PDLP if name == "PDLP" else A.ALGO_PDHG
        p = A.default_params_py(algo)
        p.float_type = A.VAL_F32 if T is np.float32 else A.VAL_F64
        p.matrix_type = self.FORMATS[self.M]
        for k, v in kw.items():
            if k not in self.KEYWORDS:
                raise TypeError(f"unexpected keyword {k}")
            setattr(p, k, type(getattr(p, k))(v) if not isinstance(getattr(p, k), float) else float(v))
        self.params = p

    def kwargs(self) -> dict:
        return {k: getattr(self.params, k) for k in self.KEYWORDS}

    def __repr__(self):
        kw = ", ".join(f"{k}={v}" for k, v in self.kwargs().items())
        return f"{self.name} algorithm (T={self.T.__name__}, M={self.M}): {kw}"


def PDLP(T=np.float64, Ti=np.int64, M=None, **kw) -> Algorithm:
    """pdlp.jl:6-11"""
    return Algorithm("PDLP", T, Ti, M, **kw)


def PDHG(T=np.float64, Ti=np.int64, M=None, **kw) -> Algorithm:
    """pdhg.jl:6-16: ruiz_iter = 0 and NaN restart / primal-weight parameters."""
    kw.setdefault("ruiz_iter", 0)
    return Algorithm("PDHG", T, Ti, M, **kw)


# ---------------------------------------------------------------------------
class DeviceMILP:
    """The preprocessed MILP resident on the GPU (result of `preprocess`)."""

    def __init__(self, milp: MILP, algo: Algorithm, handle: native.Handle | None = None):
        self.milp = milp
        self.algo = algo
        self.handle = handle or native.default_handle(algo.device)
        self.lp = native.LPStruct(milp.A.m, milp.A.n, milp.A.colptr, milp.A.rowval, milp.A.nzval,
                                  milp.c, milp.lv, milp.uv, milp.lc, milp.uc)
        self.problem = native.Problem(self.handle, self.lp, algo.params)

    @property
    def D1(self):
        return self.problem.scaling()[0]

    @property
    def D2(self):
        return self.problem.scaling()[1]


class SolverState:
    """PDLPState / PDHGState (pdlp.jl:20-43, pdhg.jl:25-38) on the device."""

    def __init__(self, dmilp: DeviceMILP, sol: PrimalDualSolution, algo: Algorithm,
                 starting_time: float | None = None):
        self.dmilp = dmilp
        self.algo = algo
        self.native = native.State(dmilp.problem, algo.params, sol.x, sol.y)
        self.starting_time = time.time() if starting_time is None else starting_time

    def stats(self) -> ConvergenceStats:
        return _stats_from(self.native.stats(), self.native.history(), self.starting_time)

    def solution(self) -> PrimalDualSolution:
        x, y = self.native.solution()
        return PrimalDualSolution(x, y)


def _stats_from(st, hist, starting_time) -> ConvergenceStats:
    return ConvergenceStats(
        err=KKTErrors.from_c(st.err), starting_time=starting_time, time_elapsed=st.time_elapsed,
        kkt_passes=st.kkt_passes, termination_status=TerminationStatus(st.termination_status),
        error_history=[(p, KKTErrors.from_c(e)) for p, e in hist], outer=st.outer,
        inner=st.inner, total=st.total, eta=st.eta, omega=st.omega,
        power_iterations=st.power_iterations, setup_seconds=st.setup_seconds,
        refine_kkt_passes=st.refine_kkt_passes)


def preprocess(milp: MILP, sol: PrimalDualSolution, algo: Algorithm):
    """common.jl:154-169: scaling, conversion and upload happen on the GPU."""
    return DeviceMILP(milp, algo), sol


def initialize(dmilp: DeviceMILP, sol: PrimalDualSolution, algo: Algorithm,
               starting_time: float | None = None) -> SolverState:
    """pdlp.jl:45-67 / pdhg.jl:40-54 (step size by power method, primal weight)."""
    return SolverState(dmilp, sol, algo, starting_time)


def solve_inplace(state: SolverState, dmilp: DeviceMILP | None = None,
                  algo: Algorithm | None = None) -> SolverState:
    """solve!(state, milp, algo) (pdlp.jl:69-94, pdhg.jl:56-74)."""
    state.native.solve()
    return state


solve_ = solve_inplace


def get_solution(state: SolverState, dmilp: DeviceMILP | None = None) -> PrimalDualSolution:
    """common.jl:233-235"""
    return state.solution()


def solve(milp: MILP, *args):
    """solve(milp, algo) or solve(milp, sol, algo) (common.jl:186-209).

    Returns (PrimalDualSolution, ConvergenceStats); the solution is
    unpreconditioned and on the host, stats.error_history is filled."""
    if len(args) == 1:
        algo = args[0]
        sol = PrimalDualSolution(np.zeros_like(milp.lv), np.zeros_like(milp.lc))
    elif len(args) == 2:
        sol, algo = args
    else:
        raise TypeError("solve(milp, algo) or solve(milp, sol, algo)")
    t0 = time.time()
    if nbcons_zero_cost(milp):
        # early exit for a problem without constraints and with zero cost
        # (common.jl:194-198), inside cpdlp_solve
        handle = native.default_handle(algo.device)
        lp = native.LPStruct(milp.A.m, milp.A.n, milp.A.colptr, milp.A.rowval, milp.A.nzval,
                             milp.c, milp.lv, milp.uv, milp.lc, milp.uc)
        x, y, st = native.solve_lp(handle, lp, algo.params, sol.x, sol.y)
        return PrimalDualSolution(x, y), _stats_from(st, [], t0)
    p = algo.params
    if p.float_type == A.VAL_F32 and p.refine_reltol > 0:
        # mixed precision (FP32 phase, then refinement rounds on the residual
        # LP with FP64 residuals and KKT errors) runs inside cpdlp_solve
        handle = native.default_handle(algo.device)
        lp = native.LPStruct(milp.A.m, milp.A.n, milp.A.colptr, milp.A.rowval, milp.A.nzval,
                             milp.c, milp.lv, milp.uv, milp.lc, milp.uc)
        x, y, st = native.solve_lp(handle, lp, p, sol.x, sol.y)
        return PrimalDualSolution(x, y), _stats_from(st, native.solve_history(handle), t0)
    dmilp, sol = preprocess(milp, sol, algo)
    state = initialize(dmilp, sol, algo, starting_time=t0)
    solve_inplace(state)
    return state.solution(), state.stats()


def nbcons_zero_cost(milp: MILP) -> bool:
    return milp.A.m == 0 and not np.any(milp.c != 0)
