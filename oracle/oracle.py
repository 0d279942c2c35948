"""ctypes bindings of the CPU oracle (oracle/cpdlp_oracle.c) -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py use this module, always as the checker of libcoolpdlp_cuda, never
as a code path of the product.  It restates CoolPDLP.jl's solve path in
Float64; see the header of cpdlp_oracle.c for what is and is not pinned.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int32, c_int64, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "liboracle.so")


def _abi():
    import importlib
    import sys
    pkg = os.path.join(os.path.dirname(HERE), "coolpdlp.jl_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    return importlib.import_module("coolpdlp._abi")


A = _abi()
PD = POINTER(c_double)
P64 = POINTER(c_int64)


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "cpdlp_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["bash", os.path.join(HERE, "build_oracle.sh")])
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "orc_proj_box": (c_double, [c_double, c_double, c_double]),
            "orc_proj_multiplier": (c_double, [c_double, c_double, c_double]),
            "orc_combine": (c_double, [c_double, c_double]),
            "orc_safeprod_left": (c_double, [c_double, c_double]),
            "orc_positive_part": (c_double, [c_double]),
            "orc_negative_part": (c_double, [c_double]),
            "orc_gaussian_vector": (None, [c_uint64, c_int64, PD]),
            "orc_csc_transpose": (None, [c_int64, c_int64, P64, P64, PD, P64, P64, PD, P64]),
            "orc_ell_width": (c_int64, [c_int64, P64]),
            "orc_ell_from_csr": (None, [c_int64, c_int64, P64, P64, PD, P64, PD]),
            "orc_coo_from_csc": (None, [c_int64, P64, P64, PD, P64, P64, PD]),
            "orc_spmv_csc": (None, [c_int64, c_int64, P64, P64, PD, PD, PD, c_double, c_double]),
            "orc_spmv_csr": (None, [c_int64, P64, P64, PD, PD, PD, c_double, c_double]),
            "orc_spmv_ell": (None, [c_int64, c_int64, P64, PD, PD, PD, c_double, c_double]),
            "orc_spmv_coo": (None, [c_int64, c_int64, P64, P64, PD, PD, PD, c_double, c_double]),
            "orc_powm_default_tol": (c_double, [c_int64, c_int32]),
            "orc_err_relative": (c_double, [POINTER(A.KKTErrorsC)]),
            "orc_err_absolute": (c_double, [POINTER(A.KKTErrorsC), c_double]),
            "orc_state_create": (c_void_p, [POINTER(A.LPC), POINTER(A.ParamsC), PD, PD]),
            "orc_state_destroy": (None, [c_void_p]),
            "orc_state_step": (None, [c_void_p, c_int64]),
            "orc_state_solve": (c_int32, [c_void_p]),
            "orc_state_solve_blocks": (c_int32, [c_void_p, c_int64]),
            "orc_state_stats": (None, [c_void_p, POINTER(A.StatsC)]),
            "orc_state_vectors": (None, [c_void_p, c_int32, PD, PD]),
            "orc_state_kkt": (None, [c_void_p, c_int32, POINTER(A.KKTErrorsC)]),
            "orc_state_kkt_of": (None, [c_void_p, PD, PD, POINTER(A.KKTErrorsC)]),
            "orc_state_solution": (None, [c_void_p, PD, PD]),
            "orc_state_history": (c_int64, [c_void_p, P64, POINTER(A.KKTErrorsC), c_int64]),
            "orc_state_scaled": (None, [c_void_p] + [PD] * 9),
            "orc_solve": (c_int32, [POINTER(A.LPC), POINTER(A.ParamsC), PD, PD, PD, PD,
                                    POINTER(A.StatsC), POINTER(c_void_p)]),
            "orc_num_threads": (c_int32, []),
            "orc_set_num_threads": (None, [c_int32]),
            "orc_lp_preconditioner": (None, [POINTER(A.LPC), c_int32, c_double, c_int32, PD, PD]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _pd(a):
    return a.ctypes.data_as(PD) if a is not None else None


def _p64(a):
    return a.ctypes.data_as(P64) if a is not None else None


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


class LPRef:
    """Keeps the numpy arrays alive while a cpdlp_lp struct points at them."""

    def __init__(self, lp):
        self.arrays = [i64(lp.colptr), i64(lp.rowval), f64(lp.nzval), f64(lp.c), f64(lp.lv),
                       f64(lp.uv), f64(lp.lc), f64(lp.uc)]
        cp, rv, nz, c, lv, uv, lc, uc = self.arrays
        self.s = A.LPC(lp.m, lp.n, nz.size, _p64(cp), _p64(rv), _pd(nz), _pd(c), _pd(lv),
                       _pd(uv), _pd(lc), _pd(uc))


def params(algorithm=A.ALGO_PDLP, **kw) -> "A.ParamsC":
    p = A.default_params_py(algorithm)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def kkt_dict(e) -> dict:
    return {k: getattr(e, k) for k, _ in A.KKTErrorsC._fields_}


def stats_dict(s) -> dict:
    d = {k: getattr(s, k) for k, _ in A.StatsC._fields_ if k != "err"}
    d["err"] = kkt_dict(s.err)
    return d


class OracleState:
    """preprocess + initialize on the oracle; step / solve / read back."""

    def __init__(self, lp, prm, x0=None, y0=None):
        self.lp = lp
        self.ref = LPRef(lp)
        self.prm = prm
        self.m, self.n = lp.m, lp.n
        x0 = None if x0 is None else f64(x0)
        y0 = None if y0 is None else f64(y0)
        self.h = lib().orc_state_create(ctypes.byref(self.ref.s), ctypes.byref(prm), _pd(x0),
                                        _pd(y0))

    def close(self):
        if self.h:
            lib().orc_state_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, k: int):
        lib().orc_state_step(self.h, k)

    def solve(self) -> int:
        return lib().orc_state_solve(self.h)

    def solve_blocks(self, max_blocks: int) -> int:
        return lib().orc_state_solve_blocks(self.h, max_blocks)

    def stats(self) -> dict:
        s = A.StatsC()
        lib().orc_state_stats(self.h, ctypes.byref(s))
        return stats_dict(s)

    def vectors(self, which=A.VEC_SOL):
        x = np.empty(self.n)
        y = np.empty(self.m)
        lib().orc_state_vectors(self.h, which, _pd(x), _pd(y))
        return x, y

    def kkt(self, which=A.VEC_SOL) -> dict:
        e = A.KKTErrorsC()
        lib().orc_state_kkt(self.h, which, ctypes.byref(e))
        return kkt_dict(e)

    def kkt_of(self, x, y) -> dict:
        e = A.KKTErrorsC()
        lib().orc_state_kkt_of(self.h, _pd(f64(x)), _pd(f64(y)), ctypes.byref(e))
        return kkt_dict(e)

    def solution(self):
        x = np.empty(self.n)
        y = np.empty(self.m)
        lib().orc_state_solution(self.h, _pd(x), _pd(y))
        return x, y

    def history(self):
        cap = self.stats()["history_length"]
        passes = np.empty(max(cap, 1), dtype=np.int64)
        errs = (A.KKTErrorsC * max(cap, 1))()
        lib().orc_state_history(self.h, _p64(passes), errs, cap)
        return [(int(passes[i]), kkt_dict(errs[i])) for i in range(cap)]

    def scaled(self) -> dict:
        m, n, nnz = self.m, self.n, self.lp.nnz
        out = {k: np.empty(n) for k in ("D2", "c", "lv", "uv")}
        out.update({k: np.empty(m) for k in ("D1", "lc", "uc")})
        out["gA"] = np.empty(nnz)
        out["gAt"] = np.empty(nnz)
        lib().orc_state_scaled(self.h, *[_pd(out[k]) for k in
                                         ("D1", "D2", "c", "lv", "uv", "lc", "uc", "gA", "gAt")])
        return out


def solve(lp, prm=None, x0=None, y0=None):
    """solve(milp, sol, algo) on the oracle: returns (x, y, stats dict)."""
    prm = prm if prm is not None else params()
    ref = LPRef(lp)
    x = np.empty(lp.n)
    y = np.empty(lp.m)
    st = A.StatsC()
    x0 = None if x0 is None else f64(x0)
    y0 = None if y0 is None else f64(y0)
    lib().orc_solve(ctypes.byref(ref.s), ctypes.byref(prm), _pd(x0), _pd(y0), _pd(x), _pd(y),
                    ctypes.byref(st), None)
    return x, y, stats_dict(st)


# ---- sparse helpers (0-based in, 1-based out where the reference is 1-based) ----

def csr_from_csc(lp):
    """GPUSparseMatrixCSR(A) fields, 1-based (mat_csr.jl:58-61)."""
    cp0 = i64(lp.colptr) - 1
    rv0 = i64(lp.rowval) - 1
    nz = f64(lp.nzval)
    ptr = np.empty(lp.m + 1, dtype=np.int64)
    idx = np.empty(max(nz.size, 1), dtype=np.int64)
    val = np.empty(max(nz.size, 1))
    lib().orc_csc_transpose(lp.m, lp.n, _p64(cp0), _p64(rv0), _pd(nz), _p64(ptr), _p64(idx),
                            _pd(val), None)
    return ptr + 1, idx[:nz.size] + 1, val[:nz.size]


def ell_from_csc(lp):
    """GPUSparseMatrixELL(A) fields (mat_ell.jl:54-70): width d, colval (m*d,
    column-major, 1-based, 0 padding), nzval."""
    ptr1, idx1, val = csr_from_csc(lp)
    ptr0 = i64(ptr1 - 1)
    idx0 = i64(idx1 - 1)
    d = lib().orc_ell_width(lp.m, _p64(ptr0))
    col = np.empty(max(lp.m * d, 1), dtype=np.int64)
    v = np.empty(max(lp.m * d, 1))
    lib().orc_ell_from_csr(lp.m, d, _p64(ptr0), _p64(idx0), _pd(f64(val)), _p64(col), _pd(v))
    return int(d), col[:lp.m * d], v[:lp.m * d]


def coo_from_csc(lp):
    """GPUSparseMatrixCOO(A) = findnz(A) (mat_coo.jl:50-53), 1-based."""
    nnz = lp.nnz
    r = np.empty(max(nnz, 1), dtype=np.int64)
    c = np.empty(max(nnz, 1), dtype=np.int64)
    v = np.empty(max(nnz, 1))
    lib().orc_coo_from_csc(lp.n, _p64(i64(lp.colptr) - 1), _p64(i64(lp.rowval) - 1),
                           _pd(f64(lp.nzval)), _p64(r), _p64(c), _pd(v))
    return r[:nnz] + 1, c[:nnz] + 1, v[:nnz]


def spmv_csc(lp, b, c, alpha, beta):
    out = f64(c).copy()
    lib().orc_spmv_csc(lp.m, lp.n, _p64(i64(lp.colptr) - 1), _p64(i64(lp.rowval) - 1),
                       _pd(f64(lp.nzval)), _pd(f64(b)), _pd(out), alpha, beta)
    return out


def spmv_csr(m, ptr1, idx1, val, b, c, alpha, beta):
    out = f64(c).copy()
    lib().orc_spmv_csr(m, _p64(i64(ptr1) - 1), _p64(i64(idx1) - 1), _pd(f64(val)), _pd(f64(b)),
                       _pd(out), alpha, beta)
    return out


def spmv_ell(m, d, col1, val, b, c, alpha, beta):
    out = f64(c).copy()
    lib().orc_spmv_ell(m, d, _p64(i64(col1)), _pd(f64(val)), _pd(f64(b)), _pd(out), alpha, beta)
    return out


def spmv_coo(m, row1, col1, val, b, c, alpha, beta):
    out = f64(c).copy()
    lib().orc_spmv_coo(m, int(np.asarray(val).size), _p64(i64(row1) - 1), _p64(i64(col1) - 1),
                       _pd(f64(val)), _pd(f64(b)), _pd(out), alpha, beta)
    return out


def preconditioner(lp, ruiz_iter: int, alpha: float = 1.0, with_cp: bool = True):
    """(D1, D2) of ruiz_preconditioner (with_cp=False) or pdlp_preconditioner."""
    ref = LPRef(lp)
    d1 = np.empty(max(lp.m, 1))
    d2 = np.empty(max(lp.n, 1))
    lib().orc_lp_preconditioner(ctypes.byref(ref.s), ruiz_iter, alpha, int(with_cp), _pd(d1),
                                _pd(d2))
    return d1[:lp.m], d2[:lp.n]


def gaussian_vector(seed: int, n: int) -> np.ndarray:
    out = np.empty(n)
    lib().orc_gaussian_vector(seed, n, _pd(out))
    return out


def scalar(name, *args):
    return getattr(lib(), "orc_" + name)(*args)


def sort_rows_columns(lp):
    """sort_rows_columns (src/components/permutation.jl:1-46) restated with
    numpy/scipy: perm_var = stable sortperm of the column lengths of A
    (increasing_column_order, :1-4), perm_cons = the same for A' (its column
    lengths are A's row lengths); the permuted matrix is A[perm_cons, perm_var]
    (permute_rows_columns, :6-14).  Returns 0-based permutations and the 1-based
    CSC arrays with rows ascending per column."""
    import scipy.sparse as sp
    A_ = sp.csc_matrix((lp.nzval, lp.rowval - 1, lp.colptr - 1), shape=(lp.m, lp.n))
    collen = np.diff(lp.colptr)
    rowlen = np.bincount(lp.rowval - 1, minlength=lp.m) if lp.nnz else np.zeros(lp.m, np.int64)
    pv = np.argsort(collen, kind="stable")
    pc = np.argsort(rowlen, kind="stable")
    B = A_[pc][:, pv].tocsc()
    B.sort_indices()
    return (pv, pc, B.indptr.astype(np.int64) + 1, B.indices.astype(np.int64) + 1,
            B.data.astype(np.float64))
