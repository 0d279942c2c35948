"""Problem and solution types: mirror of src/problems/milp.jl and solution.jl."""
from __future__ import annotations

import dataclasses
import warnings

import numpy as np

from ._abi import ArgumentError, DimensionMismatch
from . import _abi as A


def _as_float_vector(v, what: str) -> np.ndarray:
    a = np.asarray(v)
    if a.dtype == object or not (np.issubdtype(a.dtype, np.floating) or
                                 np.issubdtype(a.dtype, np.integer)):
        raise ArgumentError(A.ERR_ARGUMENT, f"Abstract type parameter ({what} has dtype {a.dtype})")
    if a.ndim != 1:
        raise DimensionMismatch(A.ERR_DIMENSION, f"{what} must be a vector")
    return np.ascontiguousarray(a, dtype=np.float64)


class CSCMatrix:
    """A SparseMatrixCSC-like container: 1-based int64 colptr/rowval, float64 nzval."""

    def __init__(self, m: int, n: int, colptr, rowval, nzval):
        self.m, self.n = int(m), int(n)
        self.colptr = np.ascontiguousarray(colptr, dtype=np.int64)
        self.rowval = np.ascontiguousarray(rowval, dtype=np.int64)
        self.nzval = np.ascontiguousarray(nzval, dtype=np.float64)

    @property
    def shape(self):
        return (self.m, self.n)

    @property
    def nnz(self) -> int:
        return int(self.nzval.size)

    @classmethod
    def from_any(cls, A_) -> "CSCMatrix":
        if isinstance(A_, CSCMatrix):
            return A_
        try:
            import scipy.sparse as sp
        except ImportError:  # pragma: no cover
            sp = None
        if sp is not None and sp.issparse(A_):
            csc = sp.csc_matrix(A_)
            csc.sum_duplicates()
            csc.sort_indices()
            return cls(csc.shape[0], csc.shape[1], csc.indptr.astype(np.int64) + 1,
                       csc.indices.astype(np.int64) + 1, csc.data.astype(np.float64))
        D = np.asarray(A_)
        if D.ndim != 2:
            raise DimensionMismatch(A.ERR_DIMENSION, "constraint matrix must be 2-D")
        if D.dtype == object:
            raise ArgumentError(A.ERR_ARGUMENT, "Abstract type parameter (matrix)")
        m, n = D.shape
        rows, cols = np.nonzero(D.T)  # column-major order: (col, row)
        colptr = np.zeros(n + 1, dtype=np.int64)
        np.add.at(colptr, rows + 1, 1)  # rows here index columns of D
        colptr = np.cumsum(colptr) + 1
        return cls(m, n, colptr, cols + 1, D[cols, rows].astype(np.float64))

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.nzval, self.rowval - 1, self.colptr - 1), shape=(self.m, self.n))

    def transpose(self) -> "CSCMatrix":
        """convert(typeof(A), transpose(A)) (milp.jl:60)."""
        t = self.to_scipy().T.tocsc()
        t.sort_indices()
        return CSCMatrix(self.n, self.m, t.indptr + 1, t.indices + 1, t.data)

    def matvec(self, x) -> np.ndarray:
        return self.to_scipy() @ np.asarray(x, dtype=np.float64)


class MILP:
    """LP/MILP in "cuPDLPx form" (milp.jl:20-115):

        min c'x  s.t.  lv <= x <= uv,  lc <= A x <= uc

    Raises DimensionMismatch / ArgumentError like the reference constructor."""

    def __init__(self, *, c, lv, uv, A, lc, uc, At=None, D1=None, D2=None, int_var=None,
                 var_names=None, dataset: str = "", name: str = "", path: str = ""):
        self.c = _as_float_vector(c, "c")
        self.lv = _as_float_vector(lv, "lv")
        self.uv = _as_float_vector(uv, "uv")
        self.lc = _as_float_vector(lc, "lc")
        self.uc = _as_float_vector(uc, "uc")
        self.A = CSCMatrix.from_any(A)
        self.At = CSCMatrix.from_any(At) if At is not None else self.A.transpose()
        m, n = self.A.shape
        self.D1 = _as_float_vector(D1, "D1") if D1 is not None else np.ones(m)
        self.D2 = _as_float_vector(D2, "D2") if D2 is not None else np.ones(n)
        self.int_var = (np.zeros(n, dtype=bool) if int_var is None
                        else np.asarray(int_var, dtype=bool))
        self.var_names = list(var_names) if var_names is not None else [str(i + 1) for i in range(n)]
        if not (n == self.c.size == self.lv.size == self.uv.size == self.D2.size ==
                self.int_var.size == len(self.var_names)):
            raise DimensionMismatch(A_ERR_DIM, "Variable size not consistent")
        if not (m == self.lc.size == self.uc.size == self.D1.size):
            raise DimensionMismatch(A_ERR_DIM, "Constraint size not consistent")
        if self.At.shape != (n, m):
            raise DimensionMismatch(A_ERR_DIM, "Transposed matrix size not consistent")
        self.dataset = str(dataset)
        self.path = str(path)
        if not name and path:
            import os
            name = os.path.splitext(os.path.basename(path))[0]
        self.name = str(name)

    @classmethod
    def from_lpdata(cls, lp, **kw) -> "MILP":
        return cls(c=lp.c, lv=lp.lv, uv=lp.uv,
                   A=CSCMatrix(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval), lc=lp.lc, uc=lp.uc,
                   name=kw.pop("name", getattr(lp, "name", "")), **kw)

    @classmethod
    def from_qps(cls, qps, **kw) -> "MILP":
        """MILP(qps::QPSData) (milp.jl:117-136): A = sparse(arows, acols, avals)
        (duplicate entries summed, as Julia's sparse does), int_var from the
        Binary / Integer variable types, var_names from the QPS names.  The
        objective constant and sense are not carried, as in the reference."""
        import scipy.sparse as sp
        from .qps import VTYPE_Binary, VTYPE_Integer
        m, n = len(qps.lcon), len(qps.lvar)
        A_ = sp.coo_matrix((qps.avals, (qps.arows - 1, qps.acols - 1)), shape=(m, n)).tocsc()
        A_.sum_duplicates()
        A_.sort_indices()
        vt = np.asarray(qps.vartypes, dtype=np.int64)
        return cls(c=qps.c, lv=qps.lvar, uv=qps.uvar, A=A_, lc=qps.lcon, uc=qps.ucon,
                   int_var=(vt == VTYPE_Binary) | (vt == VTYPE_Integer),
                   var_names=list(qps.varnames), name=kw.pop("name", qps.name), **kw)

    def __repr__(self):
        return (f"MILP instance {self.name} from dataset {self.dataset}:\n"
                f"- variables: {nbvar(self)}\n  - {nbvar_cont(self)} continuous\n"
                f"  - {nbvar_int(self)} integer\n- constraints: {nbcons(self)}\n"
                f"  - {nbcons_ineq(self)} inequalities\n  - {nbcons_eq(self)} equalities\n"
                f"- nonzeros: {self.A.nnz}")

    def isapprox(self, other: "MILP", rtol: float = 1.4901161193847656e-08) -> bool:
        def close(a, b):
            return a.shape == b.shape and np.allclose(a, b, rtol=rtol, atol=0.0, equal_nan=True)
        return (close(self.c, other.c) and close(self.lv, other.lv) and close(self.uv, other.uv)
                and close(self.A.to_scipy().toarray(), other.A.to_scipy().toarray())
                and close(self.lc, other.lc) and close(self.uc, other.uc)
                and close(self.D1, other.D1) and close(self.D2, other.D2)
                and np.array_equal(self.int_var, other.int_var))


A_ERR_DIM = A.ERR_DIMENSION


def nbvar(milp: MILP) -> int:
    """milp.jl:164"""
    return int(milp.c.size)


def nbvar_int(milp: MILP) -> int:
    return int(np.sum(milp.int_var))


def nbvar_cont(milp: MILP) -> int:
    return nbvar(milp) - nbvar_int(milp)


def nbcons(milp: MILP) -> int:
    return int(milp.A.m)


def nbcons_eq(milp: MILP) -> int:
    """Equality rows are lc == uc (milp.jl:192)."""
    return int(np.sum(milp.lc == milp.uc))


def nbcons_ineq(milp: MILP) -> int:
    return nbcons(milp) - nbcons_eq(milp)


@dataclasses.dataclass
class PrimalDualSolution:
    """solution.jl:49-54"""
    x: np.ndarray
    y: np.ndarray

    def copy(self) -> "PrimalDualSolution":
        return PrimalDualSolution(np.array(self.x, copy=True), np.array(self.y, copy=True))

    def zero(self) -> "PrimalDualSolution":
        return PrimalDualSolution(np.zeros_like(self.x), np.zeros_like(self.y))

    def isapprox(self, other: "PrimalDualSolution", rtol: float = 1.4901161193847656e-08) -> bool:
        return (np.allclose(self.x, other.x, rtol=rtol, atol=0) and
                np.allclose(self.y, other.y, rtol=rtol, atol=0))


def axpby(a: float, x: PrimalDualSolution, b: float, y: PrimalDualSolution) -> PrimalDualSolution:
    """LinearAlgebra.axpby! on both halves (solution.jl:84-90): y = a*x + b*y."""
    y.x[:] = x.x * a + y.x * b
    y.y[:] = x.y * a + y.y * b
    return y


def is_feasible(x, milp: MILP, cons_tol: float = 1e-6, int_tol: float = 1e-5,
                verbose: bool = True) -> bool:
    """solution.jl:12-33"""
    x = np.asarray(x, dtype=np.float64)
    bounds_err = max(np.max(x - milp.uv, initial=-np.inf), np.max(milp.lv - x, initial=-np.inf))
    Ax = milp.A.matvec(x)
    cons_err = max(np.max(Ax - milp.uc, initial=-np.inf), np.max(milp.lc - Ax, initial=-np.inf))
    xint = x[milp.int_var]
    int_err = np.max(np.abs(xint - np.round(xint)), initial=-np.inf) if xint.size else -np.inf
    if bounds_err > cons_tol:
        if verbose:
            warnings.warn(f"Variable bounds not satisfied: bounds_err={bounds_err}")
        return False
    if cons_err > cons_tol:
        if verbose:
            warnings.warn(f"Constraints not satisfied: cons_err={cons_err}")
        return False
    if int_err > int_tol:
        if verbose:
            warnings.warn(f"Integrality not satisfied: int_err={int_err}")
        return False
    return True


def objective_value(x, milp: MILP) -> float:
    """solution.jl:40"""
    return float(np.dot(np.asarray(x, dtype=np.float64), milp.c))


def sort_rows_columns(milp: MILP) -> MILP:
    """sort_rows_columns(milp) (permutation.jl:16-46): a new MILP whose variables
    are ordered by increasing column length and whose constraints by increasing
    row length (stable), through cpdlp_sort_rows_columns."""
    from ctypes import byref
    from . import native
    m, n, nnz = milp.A.m, milp.A.n, milp.A.nnz
    lp = native.LPStruct(m, n, milp.A.colptr, milp.A.rowval, milp.A.nzval, milp.c, milp.lv,
                         milp.uv, milp.lc, milp.uc)
    pv = np.empty(max(n, 1), dtype=np.int64)
    pc = np.empty(max(m, 1), dtype=np.int64)
    colptr = np.empty(n + 1, dtype=np.int64)
    rowval = np.empty(max(nnz, 1), dtype=np.int64)
    nzval = np.empty(max(nnz, 1))
    c, lv, uv = np.empty(max(n, 1)), np.empty(max(n, 1)), np.empty(max(n, 1))
    lc, uc = np.empty(max(m, 1)), np.empty(max(m, 1))
    lib = A.load_library()
    rc = lib.cpdlp_sort_rows_columns(None, byref(lp.s), native._p64(pv), native._p64(pc),
                                     native._p64(colptr), native._p64(rowval), native._pd(nzval),
                                     native._pd(c), native._pd(lv), native._pd(uv),
                                     native._pd(lc), native._pd(uc))
    if rc != A.OK:
        A.raise_for(rc, "sort_rows_columns: invalid LP")
    pv, pc = pv[:n] - 1, pc[:m] - 1
    return MILP(c=c[:n], lv=lv[:n], uv=uv[:n],
                A=CSCMatrix(m, n, colptr, rowval[:nnz], nzval[:nnz]), lc=lc[:m], uc=uc[:m],
                D1=milp.D1[pc], D2=milp.D2[pv], int_var=milp.int_var[pv],
                var_names=[milp.var_names[j] for j in pv], dataset=milp.dataset, name=milp.name,
                path=milp.path)
