"""cpdlp_spmv_csr_noalloc: the CSR product for callers that may not call
cudaMalloc when they need it (a fixed, pre-reserved device budget, a host
callback or finalizer, or a CuArray-backed GPUSparseMatrixCSR whose arrays
should be used in place).  It reads the caller's own 1-based device arrays and
keeps its scratch in a fixed device array of the library.

Checked against the oracle's CPU CSR product (the restatement of the
reference's spmv_csr!, on the CSR the oracle builds from the same CSC) within
the SpMV tolerance of the other tests, on consecutive calls (the calls share
the scratch array), with rows that cross several 512-nonzero warp ranges, runs
of empty rows and beta == 0 (c must not be read).  Also checked: invalid CSR
input returns CPDLP_ERR_ARGUMENT and the next valid call succeeds, oversize
input is rejected, and repeated calls leave the device's free memory
unchanged.  This file is collected last, so a run that stops at the first
failure has run every other test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lp(seed=5):
    from coolpdlp import generators as G
    st = G.Stream(seed, 0)
    m, n = 3000, 4000
    lens = st.integers(m, 0, 9)              # short rows, some empty
    lens[st.integers(12, 0, m)] = st.integers(12, 600, 3000)   # rows crossing warp ranges
    lens[:5] = 0
    lens[1200:1900] = 0                      # a long run of empty rows
    cols = G._distinct_per_group(st, lens.astype(np.int64), n)
    rows = np.repeat(np.arange(m, dtype=np.int64), lens)
    colptr, rowval, nzval = G.csc_from_triplets(m, n, rows, cols, st.normal(rows.size))
    return G.LPData(m=m, n=n, colptr=colptr, rowval=rowval, nzval=nzval,
                    c=np.zeros(n), lv=np.zeros(n), uv=np.ones(n), lc=np.zeros(m),
                    uc=np.ones(m))


def _call(handle, m, n, nnz, d_rowptr, d_colval, d_val, vt, bt, ct, alpha, beta):
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    return handle.lib.cpdlp_spmv_csr_noalloc(handle.h, m, n, nnz, ptr(d_rowptr), ptr(d_colval),
                                             ptr(d_val), vt, ptr(bt), ptr(ct), alpha, beta)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_spmv_matches_oracle(handle, oracle, dtype):
    import torch
    from coolpdlp import _abi as A
    lp = _lp()
    m, n = lp.m, lp.n
    ptr1, idx1, vals = oracle.csr_from_csc(lp)
    vals_t = vals.astype(dtype)
    d_rowptr = torch.tensor(ptr1.astype(np.int32), device="cuda")
    d_colval = torch.tensor(idx1.astype(np.int32), device="cuda")
    d_val = torch.tensor(vals_t, device="cuda")
    vt = A.VAL_F64 if dtype == np.float64 else A.VAL_F32
    gen = np.random.default_rng(11)
    dense_abs = np.zeros((m, n))
    rows = np.repeat(np.arange(m), np.diff(ptr1))
    np.add.at(dense_abs, (rows, idx1 - 1), np.abs(vals_t.astype(np.float64)))
    tol = 1e-12 if dtype == np.float64 else 1e-5
    cases = [(0.75, 0.5), (1.0, 0.0), (-1.25, 2.0)]
    bs = [gen.standard_normal(n).astype(dtype) for _ in cases]
    cs = [gen.standard_normal(m).astype(dtype) for _ in cases]
    d_b = [torch.tensor(b, device="cuda") for b in bs]
    d_c = [torch.tensor(c, device="cuda") for c in cs]
    torch.cuda.synchronize()
    for call, (alpha, beta) in enumerate(cases):
        b, c0 = bs[call], cs[call]
        if beta == 0.0:
            d_c[call][0] = float("nan")  # beta == 0 must not read c
        handle.check(_call(handle, m, n, int(vals.size), d_rowptr, d_colval, d_val, vt,
                           d_b[call], d_c[call], alpha, beta), "cpdlp_spmv_csr_noalloc")
        got = d_c[call].cpu().numpy().astype(np.float64)
        ref = oracle.spmv_csr(m, ptr1, idx1, vals_t.astype(np.float64), b.astype(np.float64),
                              c0.astype(np.float64), alpha, beta)
        scale = (dense_abs @ np.abs(b.astype(np.float64))
                 + abs(beta) * np.abs(c0.astype(np.float64)) + 1e-300)
        assert np.all(np.isfinite(got)), call
        assert np.max(np.abs(got - ref) / scale) <= tol, (call, np.max(np.abs(got - ref) / scale))


def test_noalloc_spmv_invalid_input_then_valid(handle, oracle):
    import torch
    from coolpdlp import _abi as A
    lp = _lp(seed=6)
    m, n = lp.m, lp.n
    ptr1, idx1, vals = oracle.csr_from_csc(lp)
    b = np.linspace(-1.0, 1.0, n)
    d_b = torch.tensor(b, device="cuda")
    d_val = torch.tensor(vals, device="cuda")
    d_c = torch.zeros(m, dtype=torch.float64, device="cuda")
    # a column index outside 1..n (skipped by the kernel, reported after the call)
    bad_col = idx1.astype(np.int32).copy()
    bad_col[len(bad_col) // 2] = n + 7
    d_ptr = torch.tensor(ptr1.astype(np.int32), device="cuda")
    d_col = torch.tensor(bad_col, device="cuda")
    rc = _call(handle, m, n, int(vals.size), d_ptr, d_col, d_val, A.VAL_F64, d_b, d_c, 1.0, 0.0)
    assert rc == A.ERR_ARGUMENT
    # a decreasing row pointer (values stay inside 1..nnz+1)
    bad_ptr = ptr1.astype(np.int32).copy()
    k = int(np.argmax(np.diff(ptr1) > 2)) + 1
    bad_ptr[k] = bad_ptr[k - 1] - 1 if bad_ptr[k - 1] > 1 else bad_ptr[k + 1] + 1
    assert np.any(np.diff(bad_ptr) < 0)
    d_ptr_bad = torch.tensor(bad_ptr, device="cuda")
    d_col_ok = torch.tensor(idx1.astype(np.int32), device="cuda")
    rc = _call(handle, m, n, int(vals.size), d_ptr_bad, d_col_ok, d_val, A.VAL_F64, d_b, d_c,
               1.0, 0.0)
    assert rc == A.ERR_ARGUMENT
    # the flag is cleared: the next valid call succeeds with the right product
    handle.check(_call(handle, m, n, int(vals.size), d_ptr, d_col_ok, d_val, A.VAL_F64, d_b, d_c,
                       1.0, 0.0), "valid call after invalid ones")
    ref = oracle.spmv_csr(m, ptr1, idx1, vals, b, np.zeros(m), 1.0, 0.0)
    got = d_c.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_noalloc_spmv_allocates_nothing(handle, oracle):
    import torch
    from coolpdlp import _abi as A
    lp = _lp(seed=8)
    m, n = lp.m, lp.n
    ptr1, idx1, vals = oracle.csr_from_csc(lp)
    d_ptr = torch.tensor(ptr1.astype(np.int32), device="cuda")
    d_col = torch.tensor(idx1.astype(np.int32), device="cuda")
    d_val = torch.tensor(vals, device="cuda")
    d_b = torch.ones(n, dtype=torch.float64, device="cuda")
    d_c = torch.zeros(m, dtype=torch.float64, device="cuda")
    args = (handle, m, n, int(vals.size), d_ptr, d_col, d_val, A.VAL_F64, d_b, d_c, 1.0, 0.0)
    handle.check(_call(*args), "warm-up call")   # the first call on the device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        handle.check(_call(*args), "cpdlp_spmv_csr_noalloc")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_spmv_rejects_oversize(handle):
    from coolpdlp import _abi as A
    rc = handle.lib.cpdlp_spmv_csr_noalloc(handle.h, 10, 10, 33554433, None, None, None, A.VAL_F64,
                                           None, None, 1.0, 0.0)
    assert rc == A.ERR_UNSUPPORTED
    assert b"33554432" in handle.lib.cpdlp_last_error(handle.h)
