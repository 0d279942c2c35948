"""Pluggable sparse matrices on the GPU: GPUSparseMatrixCSR / ELL / COO.

Mirror of src/utils/mat_csr.jl, mat_ell.jl and mat_coo.jl: the constructor
takes a CSC matrix (scipy.sparse, a dense array or problems.CSCMatrix),
builds the format on the device, and `mul` is LinearAlgebra.mul!(c, A, b,
alpha, beta) on CUDA tensors (torch) of the matrix eltype.  The stored index
arrays read back 1-based, exactly as the Julia struct fields."""
from __future__ import annotations

import ctypes
import sys
from ctypes import byref, c_int64, c_void_p

import numpy as np

from . import _abi as A
from . import native
from .problems import CSCMatrix


class _GPUSparseMatrix:
    FORMAT_ID = A.FMT_CSR
    FORMAT = "CSR"

    def __init__(self, Acsc, dtype=np.float64, device: int = 0, handle=None, narrow: bool = False):
        """narrow=True (CSR, float32, every value exactly +-1): the signs are
        stored in the column indices and no value array exists."""
        C = CSCMatrix.from_any(Acsc)
        self.handle = handle or native.default_handle(device)
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.dtype(np.float64), np.dtype(np.float32)):
            raise A.ArgumentError(A.ERR_ARGUMENT, "matrix eltype must be float64 or float32")
        if narrow and self.dtype != np.float32:
            raise A.ArgumentError(A.ERR_ARGUMENT, "narrow +-1 storage has Float32 vectors")
        self.narrow = bool(narrow)
        vt = A.VAL_PM1 if narrow else (A.VAL_F64 if self.dtype == np.float64 else A.VAL_F32)
        ptr = c_void_p()
        cp, rv, nz = native.i64(C.colptr), native.i64(C.rowval), native.f64(C.nzval)
        self.handle.check(self.handle.lib.cpdlp_matrix_from_csc(
            self.handle.h, C.m, C.n, nz.size, native._p64(cp), native._p64(rv), native._pd(nz),
            self.FORMAT_ID, vt, byref(ptr)), f"GPUSparseMatrix{self.FORMAT}")
        self.ptr = ptr
        m, n, nnz, w = c_int64(), c_int64(), c_int64(), c_int64()
        self.handle.lib.cpdlp_matrix_shape(ptr, byref(m), byref(n), byref(nnz), byref(w))
        self.m, self.n, self._nnz, self.width = m.value, n.value, nnz.value, w.value

    @property
    def shape(self):
        return (self.m, self.n)

    def nnz(self) -> int:
        return self._nnz

    def export(self):
        """The stored arrays, 1-based (ptr, idx, val) as in cpdlp_matrix_export."""
        raise NotImplementedError

    def mul(self, c, b, alpha: float = 1.0, beta: float = 0.0):
        """mul!(c, A, b, alpha, beta) with torch CUDA tensors; beta == 0 does not read c."""
        import torch
        tdt = torch.float64 if self.dtype == np.float64 else torch.float32
        if not (b.is_cuda and c.is_cuda) or b.dtype != tdt or c.dtype != tdt:
            raise A.ArgumentError(A.ERR_ARGUMENT, "b and c must be CUDA tensors of the matrix eltype")
        if b.numel() != self.n or c.numel() != self.m:
            raise A.DimensionMismatch(A.ERR_DIMENSION, "mul!: vector sizes do not match the matrix")
        if not (b.is_contiguous() and c.is_contiguous()):
            raise A.ArgumentError(A.ERR_ARGUMENT, "vectors must be contiguous")
        # order the library's stream after torch's current stream
        torch.cuda.current_stream(b.device).synchronize()
        self.handle.check(self.handle.lib.cpdlp_spmv(self.handle.h, self.ptr, c_void_p(b.data_ptr()),
                                                     c_void_p(c.data_ptr()), float(alpha),
                                                     float(beta)), "mul!")
        return c

    def close(self):
        if getattr(self, "ptr", None):
            self.handle.lib.cpdlp_matrix_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down:
        # the process releases the device memory itself
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    def _export_raw(self, n_ptr, n_idx, n_val):
        p = np.empty(max(n_ptr, 1), dtype=np.int64)
        i = np.empty(max(n_idx, 1), dtype=np.int64)
        v = np.empty(max(n_val, 1))
        self.handle.check(self.handle.lib.cpdlp_matrix_export(
            self.handle.h, self.ptr, native._p64(p) if n_ptr else None,
            native._p64(i) if n_idx else None, native._pd(v) if n_val else None))
        return p[:n_ptr], i[:n_idx], v[:n_val]


class GPUSparseMatrixCSR(_GPUSparseMatrix):
    """mat_csr.jl:8-92: rowptr (m+1), colval, nzval; colval ascending per row."""
    FORMAT_ID = A.FMT_CSR
    FORMAT = "CSR"

    def export(self):
        rowptr, colval, nzval = self._export_raw(self.m + 1, self._nnz, self._nnz)
        return rowptr, colval, nzval

    def to_dense(self) -> np.ndarray:
        rowptr, colval, nzval = self.export()
        D = np.zeros((self.m, self.n))
        for i in range(self.m):
            for k in range(rowptr[i] - 1, rowptr[i + 1] - 1):
                D[i, colval[k] - 1] = nzval[k]
        return D


class GPUSparseMatrixELL(_GPUSparseMatrix):
    """mat_ell.jl:8-102: colval / nzval are m x d column-major, 0 = padding."""
    FORMAT_ID = A.FMT_ELL
    FORMAT = "ELL"

    def nnz(self) -> int:
        """SparseArrays.nnz = count of nonzero colval (mat_ell.jl:22)."""
        _, colval, _ = self.export()
        return int(np.count_nonzero(colval))

    def export(self):
        md = self.m * self.width
        _, colval, nzval = self._export_raw(0, md, md)
        return None, colval.reshape((self.m, self.width), order="F"), nzval.reshape(
            (self.m, self.width), order="F")

    def to_dense(self) -> np.ndarray:
        _, colval, nzval = self.export()
        D = np.zeros((self.m, self.n))
        for i in range(self.m):
            for k in range(self.width):
                if colval[i, k] != 0:
                    D[i, colval[i, k] - 1] = nzval[i, k]
        return D


class GPUSparseMatrixCOO(_GPUSparseMatrix):
    """mat_coo.jl:8-80: findnz order (column-major)."""
    FORMAT_ID = A.FMT_COO
    FORMAT = "COO"

    def export(self):
        rowval, colval, nzval = self._export_raw(self._nnz, self._nnz, self._nnz)
        return rowval, colval, nzval

    def to_dense(self) -> np.ndarray:
        r, c, v = self.export()
        D = np.zeros((self.m, self.n))
        D[r - 1, c - 1] = v
        return D
