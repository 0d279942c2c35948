"""sort_rows_columns (src/components/permutation.jl:1-46) through the C ABI,
against the oracle's numpy restatement: the permutations, the permuted CSC
arrays and vectors must be identical (integer and copied values: bit-exact).
The entry point is host code, so these tests run without a GPU.  Cases follow
test/components/permutation.jl:5-15 (m, n in 10/20/30, p in 0.01/0.1/0.3),
plus empty rows/columns, ties and an empty matrix."""
import numpy as np
import pytest


def _lps():
    from coolpdlp import generators as G
    out = []
    k = 0
    for m in (10, 20, 30):
        for n in (10, 20, 30):
            for p in (0.01, 0.1, 0.3):
                lp, _, _ = G.random_milp_and_sol(m, n, p, seed=100 + k)
                out.append(lp)
                k += 1
    out.append(G.LPData(4, 3, np.ones(4, dtype=np.int64), np.zeros(0, dtype=np.int64),
                        np.zeros(0), np.arange(3.0), np.zeros(3), np.ones(3), np.zeros(4),
                        np.ones(4)))
    out.append(G.multicommodity_flow_lp(side=4, K=2, seed=3))
    return out


def test_sort_rows_columns_matches_oracle(oracle):
    import coolpdlp as cp
    for k, lp in enumerate(_lps()):
        milp = cp.MILP.from_lpdata(lp)
        got = cp.sort_rows_columns(milp)
        pv, pc, colptr, rowval, nzval = oracle.sort_rows_columns(lp)
        assert np.array_equal(got.A.colptr, colptr), k
        assert np.array_equal(got.A.rowval, rowval), k
        assert np.array_equal(got.A.nzval, nzval), k
        for name, perm in (("c", pv), ("lv", pv), ("uv", pv), ("lc", pc), ("uc", pc)):
            assert np.array_equal(getattr(got, name), getattr(milp, name)[perm]), (k, name)
        assert got.var_names == [milp.var_names[j] for j in pv]
        # the properties the reference's test checks (permutation.jl:11-13)
        D, Ds = milp.A.to_scipy().toarray(), got.A.to_scipy().toarray()
        assert np.array_equal(D[:, pv][pc, :], Ds)
        assert np.all(np.diff(np.count_nonzero(Ds, axis=0)) >= 0)
        assert np.all(np.diff(np.count_nonzero(Ds, axis=1)) >= 0)


def test_sort_rows_columns_is_stable_and_rejects_bad_csc():
    import coolpdlp as cp
    from coolpdlp import _abi as A
    # every column and row of length 1: the identity permutation (ties keep order)
    n = 5
    milp = cp.MILP(c=np.arange(n, dtype=float), lv=np.zeros(n), uv=np.ones(n), A=np.eye(n),
                   lc=np.zeros(n), uc=np.ones(n))
    got = cp.sort_rows_columns(milp)
    assert np.array_equal(got.c, milp.c) and np.array_equal(got.A.rowval, milp.A.rowval)
    bad = cp.MILP(c=np.zeros(2), lv=np.zeros(2), uv=np.ones(2), A=np.eye(2), lc=np.zeros(2),
                  uc=np.ones(2))
    bad.A.rowval = np.array([2, 1], dtype=np.int64)  # descending rows are fine per column...
    bad.A.colptr = np.array([1, 3, 3], dtype=np.int64)  # ...but not inside one column
    with pytest.raises(A.ArgumentError):
        cp.sort_rows_columns(bad)


def test_density_order_preserves_the_solution(oracle):
    """The property the solver's density order rests on: the LP in the order of
    sort_rows_columns is the same LP, so the Float64 oracle solves it to the
    same status and objective (within 1e-6 relative; the reductions run in
    another order), and its solution mapped back through the permutations is a
    solution of the original LP."""
    from coolpdlp import generators as G
    for lp in (G.random_sparse_lp(300, 600, 5, seed=8), G.powerlaw_lp(400, 800, 4800, seed=2,
                                                                     cap=400)):
        pv, pc, colptr, rowval, nzval = oracle.sort_rows_columns(lp)
        sl = G.LPData(lp.m, lp.n, colptr, rowval, nzval, lp.c[pv], lp.lv[pv], lp.uv[pv],
                      lp.lc[pc], lp.uc[pc])
        prm = oracle.params(termination_reltol=1e-8, max_kkt_passes=1 << 40)
        x0, _, s0 = oracle.solve(lp, prm)
        x1, _, s1 = oracle.solve(sl, prm)
        assert s0["termination_status"] == s1["termination_status"] == 0
        o0, o1 = float(lp.c @ x0), float(sl.c @ x1)
        assert abs(o0 - o1) <= 1e-6 * max(1.0, abs(o0)), (o0, o1)
        x = np.empty(lp.n)
        x[pv] = x1
        ax = lp.to_scipy() @ x
        viol = np.maximum(lp.lc - ax, 0.0) + np.maximum(ax - lp.uc, 0.0)
        assert np.max(viol) <= 1e-5 * (1.0 + np.max(np.abs(np.where(np.isfinite(lp.uc), lp.uc,
                                                                        0.0))))
