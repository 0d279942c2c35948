"""The MathOptInterface optimizer of CoolPDLP.jl (src/moi.jl), mirrored for Python.

``Model`` is a small JuMP-like builder (variables with bounds, affine
constraints in the four supported sets, an affine objective with a sense);
``Optimizer.optimize(model)`` does what ``MOI.optimize!`` does (moi.jl:168-246):

* constraint rows are grouped by set in the order EqualTo, GreaterThan,
  LessThan, Interval (the ``RHS`` product of sets, moi.jl:1-7), each group in
  the order its constraints were added;
* a maximisation negates c, solves, and negates the objectives back; the
  objective constant is added to both objectives;
* the solve is ``coolpdlp.solve(milp, algo)`` on the GPU, with ``algo`` built
  from the raw attributes (``algorithm``, ``float_type``, ``int_type``,
  ``matrix_type`` and every ``Algorithm`` keyword) and ``show_progress =
  !silent``; a float_type other than the model's warns, like moi.jl:200-203;
* afterwards z = proj_multiplier(c - A'y, lv, uv) and the dual objective
  l'|y|+ - u'|y|- + lv'|z|+ - uv'|z|- (safeprod_left for infinite bounds) are
  computed on the host from the returned solution, as moi.jl:217-227 does;
* statuses map as moi.jl:230-241: OPTIMAL -> (OPTIMAL, FEASIBLE_POINT,
  FEASIBLE_POINT), TIME_LIMIT / ITERATION_LIMIT -> (that, UNKNOWN, UNKNOWN),
  STILL_RUNNING -> (OTHER_ERROR, NO_SOLUTION, NO_SOLUTION).
"""
from __future__ import annotations

import dataclasses
import enum
import math
import warnings

import numpy as np

from . import algorithms as alg
from . import native
from .problems import CSCMatrix, MILP


class TerminationStatusCode(enum.Enum):
    OPTIMIZE_NOT_CALLED = "OPTIMIZE_NOT_CALLED"
    OPTIMAL = "OPTIMAL"
    TIME_LIMIT = "TIME_LIMIT"
    ITERATION_LIMIT = "ITERATION_LIMIT"
    OTHER_ERROR = "OTHER_ERROR"
    INFEASIBLE = "INFEASIBLE"            # infeasibility_tol > 0 only
    DUAL_INFEASIBLE = "DUAL_INFEASIBLE"  # infeasibility_tol > 0 only


class ResultStatusCode(enum.Enum):
    UNKNOWN_RESULT_STATUS = "UNKNOWN_RESULT_STATUS"
    FEASIBLE_POINT = "FEASIBLE_POINT"
    NO_SOLUTION = "NO_SOLUTION"
    INFEASIBILITY_CERTIFICATE = "INFEASIBILITY_CERTIFICATE"


class Sense(enum.Enum):
    MIN = "MIN_SENSE"
    MAX = "MAX_SENSE"


# the four supported sets (moi.jl SUPPORTED_SET_TYPE)
@dataclasses.dataclass(frozen=True)
class EqualTo:
    value: float


@dataclasses.dataclass(frozen=True)
class GreaterThan:
    lower: float


@dataclasses.dataclass(frozen=True)
class LessThan:
    upper: float


@dataclasses.dataclass(frozen=True)
class Interval:
    lower: float
    upper: float


_SET_ORDER = (EqualTo, GreaterThan, LessThan, Interval)


def _bounds(s) -> tuple[float, float]:
    if isinstance(s, EqualTo):
        return s.value, s.value
    if isinstance(s, GreaterThan):
        return s.lower, math.inf
    if isinstance(s, LessThan):
        return -math.inf, s.upper
    if isinstance(s, Interval):
        return s.lower, s.upper
    raise TypeError(f"unsupported set {type(s).__name__}")


@dataclasses.dataclass(frozen=True)
class VariableIndex:
    value: int  # 1-based, as MOI


@dataclasses.dataclass(frozen=True)
class ConstraintIndex:
    kind: str   # "affine" or "variable"
    set_type: type
    value: int  # affine: position within its set group (1-based); variable: the variable


class Model:
    """Variables, affine constraints and an affine objective (the subset of
    MOI that moi.jl supports)."""

    def __init__(self):
        self.lower: list[float] = []
        self.upper: list[float] = []
        self.names: list[str] = []
        self.affine: dict[type, list[tuple[dict[int, float], object]]] = {t: [] for t in _SET_ORDER}
        self.obj_terms: dict[int, float] = {}
        self.obj_constant = 0.0
        self.sense = Sense.MIN
        self.var_sets: dict[int, object] = {}

    def add_variable(self, lower: float = -math.inf, upper: float = math.inf,
                     name: str = "") -> VariableIndex:
        self.lower.append(float(lower))
        self.upper.append(float(upper))
        self.names.append(name)
        vi = VariableIndex(len(self.lower))
        if math.isfinite(lower) and math.isfinite(upper):
            self.var_sets[vi.value] = (EqualTo(lower) if lower == upper else Interval(lower, upper))
        elif math.isfinite(lower):
            self.var_sets[vi.value] = GreaterThan(lower)
        elif math.isfinite(upper):
            self.var_sets[vi.value] = LessThan(upper)
        return vi

    def add_constraint(self, terms, s) -> ConstraintIndex:
        """terms: {VariableIndex: coefficient} or [(VariableIndex, coefficient)];
        s: EqualTo / GreaterThan / LessThan / Interval.  Repeated variables add up."""
        if type(s) not in _SET_ORDER:
            raise TypeError(f"unsupported set {type(s).__name__}")
        items = terms.items() if isinstance(terms, dict) else terms
        row: dict[int, float] = {}
        for v, a in items:
            j = v.value if isinstance(v, VariableIndex) else int(v)
            if not 1 <= j <= len(self.lower):
                raise IndexError(f"unknown variable {j}")
            row[j] = row.get(j, 0.0) + float(a)
        group = self.affine[type(s)]
        group.append((row, s))
        return ConstraintIndex("affine", type(s), len(group))

    def set_objective(self, terms, constant: float = 0.0, sense: Sense = Sense.MIN):
        items = terms.items() if isinstance(terms, dict) else terms
        self.obj_terms = {}
        for v, a in items:
            j = v.value if isinstance(v, VariableIndex) else int(v)
            self.obj_terms[j] = self.obj_terms.get(j, 0.0) + float(a)
        self.obj_constant = float(constant)
        self.sense = sense

    # ---- conversion to the solver's LP (moi.jl:176-196) ----------------------
    def rows(self, ci: ConstraintIndex) -> int:
        """0-based row of an affine constraint (MOI.Utilities.rows)."""
        off = 0
        for t in _SET_ORDER:
            if t is ci.set_type:
                return off + ci.value - 1
            off += len(self.affine[t])
        raise KeyError(ci)

    def to_milp(self) -> tuple[MILP, np.ndarray]:
        n = len(self.lower)
        cols: list[list[tuple[int, float]]] = [[] for _ in range(n)]
        lc, uc = [], []
        r = 0
        for t in _SET_ORDER:
            for row, s in self.affine[t]:
                for j, a in sorted(row.items()):
                    cols[j - 1].append((r, a))
                lo, hi = _bounds(s)
                lc.append(lo)
                uc.append(hi)
                r += 1
        m = r
        colptr = np.ones(n + 1, dtype=np.int64)
        rowval, nzval = [], []
        for j in range(n):
            for i, a in sorted(cols[j]):
                rowval.append(i + 1)
                nzval.append(a)
            colptr[j + 1] = colptr[j] + len(cols[j])
        c = np.zeros(n)
        for j, a in self.obj_terms.items():
            c[j - 1] += a
        if self.sense == Sense.MAX:
            c = -c
        A = CSCMatrix(m, n, colptr, np.array(rowval, dtype=np.int64), np.array(nzval, dtype=np.float64))
        milp = MILP(c=c, lv=np.array(self.lower), uv=np.array(self.upper), A=A,
                    lc=np.array(lc, dtype=np.float64), uc=np.array(uc, dtype=np.float64))
        return milp, c


class Optimizer:
    """CoolPDLP.Optimizer{T} (moi.jl:16-47): options are the keyword arguments of
    ``Algorithm`` plus ``algorithm``, ``float_type``, ``int_type``,
    ``matrix_type`` and ``backend`` (device index here)."""

    def __init__(self, T=np.float64):
        self.T = np.dtype(T).type
        self.silent = False
        self.options: dict[str, object] = {}
        self.empty()

    # ---- MOI.empty! / is_empty (moi.jl:49-76) --------------------------------
    def empty(self):
        self.x = np.zeros(0)
        self.y = np.zeros(0)
        self.z = np.zeros(0)
        self.obj_value = math.nan
        self.dual_obj_value = math.nan
        self.termination_status = TerminationStatusCode.OPTIMIZE_NOT_CALLED
        self.primal_status = ResultStatusCode.UNKNOWN_RESULT_STATUS
        self.dual_status = ResultStatusCode.UNKNOWN_RESULT_STATUS
        self.solve_time = 0.0
        self.model: Model | None = None

    def is_empty(self) -> bool:
        return (self.x.size == 0 and self.y.size == 0 and self.z.size == 0
                and math.isnan(self.obj_value) and math.isnan(self.dual_obj_value)
                and self.termination_status == TerminationStatusCode.OPTIMIZE_NOT_CALLED
                and self.solve_time == 0.0 and self.model is None)

    # ---- attributes ----------------------------------------------------------
    def set_attribute(self, name: str, value):
        self.options[name] = value

    def get_attribute(self, name: str):
        return self.options[name]

    def set_silent(self, value: bool = True):
        self.silent = bool(value)

    def set_time_limit_sec(self, value):
        if value is None:
            self.options.pop("time_limit", None)
        else:
            self.options["time_limit"] = float(value)

    def get_time_limit_sec(self):
        return self.options.get("time_limit")

    solver_name = "CoolPDLP"

    # ---- optimize! (moi.jl:168-246) ------------------------------------------
    def optimize(self, model: Model):
        self.empty()
        milp, c = model.to_milp()
        opts = dict(self.options)
        name = opts.pop("algorithm", "PDLP")
        if isinstance(name, alg.Algorithm):
            name = name.name
        float_type = np.dtype(opts.pop("float_type", self.T)).type
        if float_type is not self.T:
            warnings.warn(f"Got mismatched float type: solving in {float_type.__name__} but "
                          f"returning the solution in {self.T.__name__}.")
        int_type = opts.pop("int_type", np.int64)
        matrix_type = opts.pop("matrix_type", None)
        device = int(opts.pop("backend", 0) or 0)
        kw = {"show_progress": not self.silent}
        kw.update(opts)
        algo = alg.Algorithm(str(name), float_type, int_type, matrix_type, device=device, **kw)
        sol, stats = alg.solve(milp, algo)
        self.model = model
        self.x = np.asarray(sol.x, dtype=np.float64)
        self.y = np.asarray(sol.y, dtype=np.float64)
        # z and the dual objective (moi.jl:215-227) on the device
        lps = native.LPStruct(milp.A.m, milp.A.n, milp.A.colptr, milp.A.rowval, milp.A.nzval,
                              c, milp.lv, milp.uv, milp.lc, milp.uc)
        self.z, raw_dual = native.reduced_costs(native.default_handle(device), lps, self.y)
        raw_obj = float(np.dot(c, self.x))
        mx = model.sense == Sense.MAX
        self.obj_value = (-raw_obj if mx else raw_obj) + model.obj_constant
        self.dual_obj_value = (-float(raw_dual) if mx else float(raw_dual)) + model.obj_constant
        self.solve_time = float(stats.time_elapsed)
        cts = stats.termination_status
        if cts == alg.OPTIMAL:
            ts, ps, ds = (TerminationStatusCode.OPTIMAL, ResultStatusCode.FEASIBLE_POINT,
                          ResultStatusCode.FEASIBLE_POINT)
        elif cts == alg.TIME_LIMIT:
            ts, ps, ds = (TerminationStatusCode.TIME_LIMIT, ResultStatusCode.UNKNOWN_RESULT_STATUS,
                          ResultStatusCode.UNKNOWN_RESULT_STATUS)
        elif cts == alg.ITERATION_LIMIT:
            ts, ps, ds = (TerminationStatusCode.ITERATION_LIMIT,
                          ResultStatusCode.UNKNOWN_RESULT_STATUS,
                          ResultStatusCode.UNKNOWN_RESULT_STATUS)
        elif cts == alg.TerminationStatus.PRIMAL_INFEASIBLE:
            # extension: the returned y is the dual ray
            ts, ps, ds = (TerminationStatusCode.INFEASIBLE, ResultStatusCode.NO_SOLUTION,
                          ResultStatusCode.INFEASIBILITY_CERTIFICATE)
        elif cts == alg.TerminationStatus.DUAL_INFEASIBLE:
            # extension: the returned x is the primal ray
            ts, ps, ds = (TerminationStatusCode.DUAL_INFEASIBLE,
                          ResultStatusCode.INFEASIBILITY_CERTIFICATE, ResultStatusCode.NO_SOLUTION)
        else:
            assert cts == alg.STILL_RUNNING
            ts, ps, ds = (TerminationStatusCode.OTHER_ERROR, ResultStatusCode.NO_SOLUTION,
                          ResultStatusCode.NO_SOLUTION)
        self.termination_status, self.primal_status, self.dual_status = ts, ps, ds
        return stats

    # ---- results (moi.jl:104-166) --------------------------------------------
    @property
    def result_count(self) -> int:
        return 0 if self.termination_status == TerminationStatusCode.OPTIMIZE_NOT_CALLED else 1

    @property
    def raw_status_string(self) -> str:
        return self.termination_status.value

    def _check(self, result_index: int = 1):
        if not 1 <= result_index <= self.result_count:
            raise IndexError(f"result index {result_index} out of bounds (result count "
                             f"{self.result_count})")

    def get_primal_status(self, result_index: int = 1) -> ResultStatusCode:
        return (ResultStatusCode.NO_SOLUTION if result_index > self.result_count
                else self.primal_status)

    def get_dual_status(self, result_index: int = 1) -> ResultStatusCode:
        return (ResultStatusCode.NO_SOLUTION if result_index > self.result_count
                else self.dual_status)

    def objective_value(self, result_index: int = 1) -> float:
        self._check(result_index)
        return self.obj_value

    def dual_objective_value(self, result_index: int = 1) -> float:
        self._check(result_index)
        return self.dual_obj_value

    def variable_primal(self, vi: VariableIndex, result_index: int = 1) -> float:
        self._check(result_index)
        return float(self.x[vi.value - 1])

    def constraint_dual(self, ci, result_index: int = 1) -> float:
        """ScalarAffineFunction rows: y[row]; variable bounds: the reduced cost z,
        its positive part for GreaterThan and minus its negative part for LessThan
        (moi.jl:123-156).  ci is a ConstraintIndex, or a VariableIndex with a set
        type for the variable-bound constraint of that variable."""
        self._check(result_index)
        if isinstance(ci, ConstraintIndex) and ci.kind == "affine":
            return float(self.y[self.model.rows(ci)])
        if isinstance(ci, tuple):
            vi, set_type = ci
        else:
            vi, set_type = VariableIndex(ci.value), ci.set_type
        zj = float(self.z[vi.value - 1])
        if set_type is GreaterThan:
            return max(zj, 0.0)
        if set_type is LessThan:
            return -max(-zj, 0.0)
        return zj


def _proj_multiplier(g: float, l: float, u: float) -> float:
    """linalg.jl: 0 if both bounds infinite, the <=0 part if only u is finite,
    the >=0 part if only l is finite, g if both are finite."""
    lf, uf = math.isfinite(l), math.isfinite(u)
    if not lf and not uf:
        return 0.0
    if lf and not uf:
        return max(g, 0.0)
    if uf and not lf:
        return min(g, 0.0)
    return g


def _safeprod_left(l, r):
    """safeprod_left(l, r) = isinf(l) ? r : l*r (linalg.jl:17), elementwise."""
    l = np.asarray(l, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    with np.errstate(invalid="ignore"):
        return np.where(np.isinf(l), r, l * r)
