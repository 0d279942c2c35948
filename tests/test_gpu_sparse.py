"""GPU parity of the pluggable sparse formats and mul! (src/utils/mat_*.jl)
against the CPU oracle's restatement, through the C ABI.

Index arrays must be bit-identical to the reference conversions; Float64
SpMV must match within 1e-12 relative (bit-identical when every row fits one
warp tile, since both sum each row in ascending column order without FMA)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shapes():
    out = []
    for m in (10, 20, 30):
        for n in (10, 20, 30):
            for p in (0.01, 0.1, 0.2, 0.3):
                out.append((m, n, p))
    return out


def _random_csc(m, n, p, seed):
    from coolpdlp import generators as G
    lp, _, _ = G.random_milp_and_sol(m, n, p, seed=seed)
    return lp


def _special_mats():
    """Edge cases: empty, single row/col, empty rows and columns, long rows
    that take the split (multi-warp) path, a power-law row profile."""
    from coolpdlp import generators as G
    mats = []
    # empty
    mats.append(G.LPData(5, 7, np.ones(8, dtype=np.int64), np.zeros(0, dtype=np.int64),
                         np.zeros(0), np.zeros(7), np.zeros(7), np.zeros(7), np.zeros(5), np.zeros(5)))
    st = G.Stream(99, 0)
    for (m, n, dens) in ((1, 50, 0.5), (50, 1, 0.5), (40, 3000, 0.4), (3, 30000, 0.9)):
        mask = st.uniform(m * n) < dens
        flat = np.nonzero(mask)[0]
        cols, rows = flat // m, flat % m
        colptr, rowval, nzval = G.csc_from_triplets(m, n, rows, cols, st.normal(flat.size))
        mats.append(G.LPData(m, n, colptr, rowval, nzval, np.zeros(n), np.zeros(n), np.zeros(n),
                             np.zeros(m), np.zeros(m)))
    mats.append(G.powerlaw_lp(2000, 4000, 24000, seed=5, cap=3000))
    return mats


def _all_mats():
    mats = [_random_csc(m, n, p, seed=i) for i, (m, n, p) in enumerate(_shapes())]
    return mats + _special_mats()


@pytest.mark.parametrize("fmt", ["CSR", "ELL", "COO"])
def test_format_indices_bit_exact(handle, oracle, fmt):
    import coolpdlp as cp
    cls = {"CSR": cp.GPUSparseMatrixCSR, "ELL": cp.GPUSparseMatrixELL,
           "COO": cp.GPUSparseMatrixCOO}[fmt]
    for lp in _all_mats():
        A = cls(cp.CSCMatrix(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval), handle=handle)
        assert A.shape == (lp.m, lp.n)
        if fmt == "CSR":
            ptr, idx, val = A.export()
            optr, oidx, oval = oracle.csr_from_csc(lp)
            assert np.array_equal(ptr, optr) and np.array_equal(idx, oidx)
            assert np.array_equal(val, oval)
            assert A.nnz() == lp.nnz
        elif fmt == "ELL":
            if lp.m * max(1, lp.nnz) > 5e7:
                continue
            _, col, val = A.export()
            d, ocol, oval = oracle.ell_from_csc(lp)
            assert A.width == d
            assert np.array_equal(col.ravel(order="F"), ocol)
            assert np.array_equal(val.ravel(order="F"), oval)
            assert A.nnz() == np.count_nonzero(ocol)
        else:
            r, c, v = A.export()
            orow, ocol, oval = oracle.coo_from_csc(lp)
            assert np.array_equal(r, orow) and np.array_equal(c, ocol) and np.array_equal(v, oval)
        dense = lp.to_scipy().toarray()
        if lp.m * lp.n <= 200000:
            assert np.array_equal(A.to_dense(), dense)
        A.close()


@pytest.mark.parametrize("fmt", ["CSR", "ELL", "COO"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_mul_matches_oracle(handle, oracle, fmt, dtype):
    """mul!(c, A, b, alpha, beta) (mat_*.jl) incl. the strong zero beta == 0."""
    import torch
    import coolpdlp as cp
    from coolpdlp import generators as G
    cls = {"CSR": cp.GPUSparseMatrixCSR, "ELL": cp.GPUSparseMatrixELL,
           "COO": cp.GPUSparseMatrixCOO}[fmt]
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    st = G.Stream(7, 1)
    alpha, beta = 0.7310585786300049, 0.2689414213699951
    for k, lp in enumerate(_all_mats()):
        if fmt == "ELL" and lp.m * max(1, lp.nnz) > 5e7:
            continue
        A = cls(cp.CSCMatrix(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval), dtype=dtype,
                handle=handle)
        b = st.normal(lp.n)
        c = st.normal(lp.m)
        vals = lp.nzval.astype(dtype).astype(np.float64)
        lp32 = G.LPData(lp.m, lp.n, lp.colptr, lp.rowval, vals, lp.c, lp.lv, lp.uv, lp.lc, lp.uc)
        bq = b.astype(dtype).astype(np.float64)
        cq = c.astype(dtype).astype(np.float64)
        for (al, be) in ((alpha, beta), (1.0, 0.0)):
            ref = oracle.spmv_csc(lp32, bq, cq, al, be)
            bt = torch.tensor(b.astype(dtype), device="cuda")
            ct = torch.tensor(c.astype(dtype), device="cuda")
            if be == 0.0 and lp.m > 0:
                ct[0] = float("nan")  # beta == false must not read c
            A.mul(ct, bt, al, be)
            got = ct.cpu().numpy().astype(np.float64)
            scale = np.abs(lp32.to_scipy()) @ np.abs(bq) + abs(be) * np.abs(cq) + 1e-300
            tol = 1e-12 if dtype == np.float64 else 1e-5
            err = np.max(np.abs(got - ref) / scale) if lp.m else 0.0
            assert np.all(np.isfinite(got)), (fmt, k)
            assert err <= tol, (fmt, k, err)
            if dtype == np.float64 and fmt in ("CSR", "ELL"):
                # the reference's CSR/ELL kernels: c[i] = alpha*s + beta*c[i] with s summed
                # in column order; rows of at most 64 nonzeros follow that order exactly
                rowlen = np.bincount(lp.rowval - 1, minlength=lp.m) if lp.nnz else np.zeros(lp.m)
                if rowlen.max(initial=0) <= 64:
                    optr, oidx, oval = oracle.csr_from_csc(lp)
                    exact = oracle.spmv_csr(lp.m, optr, oidx, oval, bq, cq, al, be)
                    if be == 0.0 and lp.m > 0:
                        exact = oracle.spmv_csr(lp.m, optr, oidx, oval, bq, np.zeros(lp.m), al, be)
                    assert np.array_equal(got, exact), (fmt, k, "sequential rows must be bit-exact")
        A.close()


def test_invalid_csc_is_argument_error(handle):
    import coolpdlp as cp
    with pytest.raises(cp.ArgumentError):
        cp.GPUSparseMatrixCSR(cp.CSCMatrix(2, 2, [1, 3, 3], [2, 1], [1.0, 2.0]), handle=handle)
    with pytest.raises(cp.ArgumentError):
        cp.GPUSparseMatrixCSR(cp.CSCMatrix(2, 2, [1, 2, 3], [1, 5], [1.0, 2.0]), handle=handle)
    with pytest.raises(cp.ArgumentError):
        cp.GPUSparseMatrixCSR(cp.CSCMatrix(2, 2, [1, 3, 2], [1, 2], [1.0, 2.0]), handle=handle)
    with pytest.raises(cp.DimensionMismatch):
        cp.GPUSparseMatrixCSR(cp.CSCMatrix(2, 2, [1, 2, 4], [1, 2], [1.0, 2.0]), handle=handle)


def test_mul_dimension_mismatch(handle):
    import torch
    import coolpdlp as cp
    A = cp.GPUSparseMatrixCSR(np.eye(3), handle=handle)
    with pytest.raises(cp.DimensionMismatch):
        A.mul(torch.zeros(3, dtype=torch.float64, device="cuda"),
              torch.zeros(4, dtype=torch.float64, device="cuda"))
