"""cpdlp_spmv_csr_noalloc: the CSR product for callers that may not call
cudaMalloc when they need it (a fixed, pre-reserved device budget, a host
callback or finalizer, or a CuArray-backed GPUSparseMatrixCSR whose arrays
should be used in place).  It reads the caller's own 1-based device arrays and
keeps its scratch in a fixed device array of the library.

Checked against the existing entry point (cpdlp_spmv on a cpdlp_matrix built
from the same CSC) within the SpMV tolerance of the other tests, on two calls
in a row (the calls share the scratch array), with rows that cross several
512-nonzero warp ranges, empty rows and beta == 0 (c must not be read)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrix(seed=5):
    from coolpdlp import generators as G
    st = G.Stream(seed, 0)
    m, n = 3000, 4000
    lens = st.integers(m, 0, 9)              # short rows, some empty
    lens[st.integers(12, 0, m)] = st.integers(12, 600, 3000)   # rows crossing warp ranges
    lens[:5] = 0
    cols = G._distinct_per_group(st, lens.astype(np.int64), n)
    rows = np.repeat(np.arange(m, dtype=np.int64), lens)
    colptr, rowval, nzval = G.csc_from_triplets(m, n, rows, cols, st.normal(rows.size))
    return m, n, colptr, rowval, nzval


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_spmv_matches_cpdlp_spmv(handle, dtype):
    import torch
    import coolpdlp as cp
    from coolpdlp import _abi as A
    m, n, colptr, rowval, nzval = _matrix()
    M = cp.GPUSparseMatrixCSR(cp.CSCMatrix(m, n, colptr, rowval, nzval), dtype=dtype, handle=handle)
    rowptr1, colval1, vals = M.export()
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    d_rowptr = torch.tensor(rowptr1.astype(np.int32), device="cuda")
    d_colval = torch.tensor(colval1.astype(np.int32), device="cuda")
    d_val = torch.tensor(vals.astype(dtype), device="cuda")
    vt = A.VAL_F64 if dtype == np.float64 else A.VAL_F32
    gen = np.random.default_rng(11)
    absA = np.abs(M.to_dense())
    tol = 1e-12 if dtype == np.float64 else 1e-5
    for call, (alpha, beta) in enumerate([(0.75, 0.5), (1.0, 0.0), (-1.25, 2.0)]):
        b = gen.standard_normal(n).astype(dtype)
        c0 = gen.standard_normal(m).astype(dtype)
        bt = torch.tensor(b, device="cuda")
        c_ref = torch.tensor(c0, device="cuda")
        c_new = torch.tensor(c0, device="cuda")
        if beta == 0.0:
            c_new[0] = float("nan")  # beta == 0 must not read c
        M.mul(c_ref, bt, alpha, beta)
        torch.cuda.synchronize()
        rc = handle.lib.cpdlp_spmv_csr_noalloc(
            handle.h, m, n, int(vals.size), ctypes.c_void_p(d_rowptr.data_ptr()),
            ctypes.c_void_p(d_colval.data_ptr()), ctypes.c_void_p(d_val.data_ptr()), vt,
            ctypes.c_void_p(bt.data_ptr()), ctypes.c_void_p(c_new.data_ptr()), alpha, beta)
        handle.check(rc, "cpdlp_spmv_csr_noalloc")
        got = c_new.cpu().numpy().astype(np.float64)
        ref = c_ref.cpu().numpy().astype(np.float64)
        scale = absA @ np.abs(b.astype(np.float64)) + abs(beta) * np.abs(c0.astype(np.float64)) + 1e-300
        assert np.all(np.isfinite(got)), call
        assert np.max(np.abs(got - ref) / scale) <= tol, (call, np.max(np.abs(got - ref) / scale))


def test_noalloc_spmv_rejects_oversize(handle):
    from coolpdlp import _abi as A
    rc = handle.lib.cpdlp_spmv_csr_noalloc(handle.h, 10, 10, 33554433, None, None, None, A.VAL_F64,
                                           None, None, 1.0, 0.0)
    assert rc == A.ERR_UNSUPPORTED
    assert b"33554432" in handle.lib.cpdlp_last_error(handle.h)
