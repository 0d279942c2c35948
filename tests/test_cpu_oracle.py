"""CPU tests: the oracle against the known answers the reference's own test
suite holds (test/utils/linalg.jl, test/components/*.jl, test/moi.jl,
test/algorithms/all.jl), against scipy (SpMV, conversions) and HiGHS
(objective), plus the host-side API logic.  No GPU needed."""
import math

import numpy as np
import pytest


def test_projections_known_answers(oracle):
    """test/utils/linalg.jl:6-39"""
    S = oracle.scalar
    st = np.random.default_rng(0)
    for x in st.standard_normal(100):
        assert math.isclose(x, S("positive_part", x) - S("negative_part", x))
        assert S("positive_part", x) >= 0 and S("negative_part", x) >= 0
        a = st.standard_normal()
        l, u = a - st.random(), a + st.random()
        p = S("proj_box", x, l, u)
        assert l <= p <= u
        if l <= x <= u:
            assert p == x
        elif x >= u:
            assert p == u
        else:
            assert p == l
        assert S("proj_multiplier", x, -np.inf, np.inf) == 0
        assert S("proj_multiplier", x, -np.inf, 3.0) == -S("negative_part", x)
        assert S("proj_multiplier", x, -3.0, np.inf) == S("positive_part", x)
        assert S("proj_multiplier", x, -3.0, 3.0) == x
    assert S("combine", 1.0, 2.0) == 2
    assert S("combine", 3.0, 3.0) == 3
    assert S("combine", -np.inf, 2.0) == 2
    assert S("combine", 3.0, np.inf) == 3
    assert S("combine", -np.inf, np.inf) == 0
    assert S("safeprod_left", np.inf, 2.5) == 2.5
    assert S("safeprod_left", 2.0, 2.5) == 5.0


def test_two_variable_lp(oracle):
    """test/moi.jl:38-53: objective 205 within 1e-2."""
    from coolpdlp import generators as G
    lp = G.two_variable_lp()
    x, y, st = oracle.solve(lp)
    assert st["termination_status"] == 0
    assert abs(12 * x[0] + 20 * x[1] - 205.0) <= 1e-2


def test_termination_check_not_skipped(oracle):
    from coolpdlp import generators as G
    x, y, st = oracle.solve(G.termination_check_lp())
    assert st["termination_status"] == 0
    assert st["kkt_passes"] == 100


def test_spmv_formats_match_scipy(oracle):
    """test/utils/matrices.jl: mul!(c, M(A), b, a, b) == a*A*b + b*c for the
    three formats, M(A) == A and nnz equal, on 36 random shapes."""
    from coolpdlp import generators as G
    st = G.Stream(5, 0)
    alpha, beta = 0.3, 0.6
    for i, (m, n, p) in enumerate([(m, n, p) for m in (10, 20, 30) for n in (10, 20, 30)
                                   for p in (0.01, 0.1, 0.2, 0.3)]):
        lp, _, _ = G.random_milp_and_sol(m, n, p, seed=i)
        A = lp.to_scipy()
        b, c = st.normal(n), st.normal(m)
        ref = alpha * (A @ b) + beta * c
        ptr, idx, val = oracle.csr_from_csc(lp)
        np.testing.assert_allclose(oracle.spmv_csr(m, ptr, idx, val, b, c, alpha, beta), ref,
                                   rtol=1.5e-8, atol=1e-12)
        csr = A.tocsr()
        csr.sort_indices()
        assert np.array_equal(ptr - 1, csr.indptr) and np.array_equal(idx - 1, csr.indices)
        d, col, v = oracle.ell_from_csc(lp)
        np.testing.assert_allclose(oracle.spmv_ell(m, d, col, v, b, c, alpha, beta), ref,
                                   rtol=1.5e-8, atol=1e-12)
        assert np.count_nonzero(col) == A.nnz
        r, cc, vv = oracle.coo_from_csc(lp)
        np.testing.assert_allclose(oracle.spmv_coo(m, r, cc, vv, b, c, alpha, beta), ref,
                                   rtol=1.5e-8, atol=1e-12)
        np.testing.assert_allclose(oracle.spmv_csc(lp, b, c, alpha, beta), ref, rtol=1.5e-8,
                                   atol=1e-12)
        # CSC scatter (the reference CPU path) and CSR gather are identical bit for bit
        assert np.array_equal(oracle.spmv_csc(lp, b, c, 1.0, 0.0),
                              oracle.spmv_csr(m, ptr, idx, val, b, c, 1.0, 0.0))


def _kkt_closed_forms(lp, x, y):
    """test/components/errors.jl:4-38 closed forms."""
    A = lp.to_scipy()
    c, lv, uv, lc, uc = lp.c, lp.lv, lp.uv, lp.lc, lp.uc
    Aty = A.T @ y
    g = c - Aty
    r = np.where(np.isneginf(lv), np.where(np.isposinf(uv), 0.0, np.minimum(g, 0)),
                 np.where(np.isposinf(uv), np.maximum(g, 0), g))

    def p(v, l, u):
        vp, vm = np.maximum(v, 0), -np.minimum(v, 0)
        us = np.where(np.isposinf(u), np.finfo(float).max, u)
        ls = np.where(np.isneginf(l), -np.finfo(float).max, l)
        return np.dot(vp, us) - np.dot(vm, ls)
    Ax = A @ x
    comb = np.maximum(np.maximum(0, np.where(np.isfinite(lc), np.abs(lc), 0)),
                      np.where(np.isfinite(uc), np.abs(uc), 0))
    return {"primal": np.linalg.norm(Ax - np.clip(Ax, lc, uc)), "dual": np.linalg.norm(g - r),
            "primal_scale": 1 + np.linalg.norm(comb), "dual_scale": 1 + np.linalg.norm(c),
            "r": r, "p": p}


def test_kkt_errors_closed_form_and_invariance(oracle):
    """test/components/errors.jl: the KKT formulas, and the errors of the
    preconditioned problem equal those of the original one."""
    from coolpdlp import generators as G
    lp, x, y = G.random_milp_and_sol(100, 200, 0.4, seed=1)
    S0 = oracle.OracleState(lp, oracle.params(ruiz_iter=0, chambolle_pock_alpha=1.0))
    S = oracle.OracleState(lp, oracle.params())
    sc = S.scaled()
    xs, ys = x / sc["D2"], y / sc["D1"]
    e = S.kkt_of(xs, ys)
    ref = _kkt_closed_forms(lp, x, y)
    for k in ("primal", "dual", "primal_scale", "dual_scale"):
        assert math.isclose(e[k], ref[k], rel_tol=1e-9), k
    sc0 = S0.scaled()
    e0 = S0.kkt_of(x / sc0["D2"], y / sc0["D1"])
    for k in ("primal", "dual", "gap", "primal_scale", "dual_scale", "gap_scale"):
        assert math.isclose(e[k], e0[k], rel_tol=1e-8), k


def test_ruiz_fixed_point(oracle):
    """test/components/preconditioning.jl:26-31: after 10,000 Ruiz passes the
    inf-norms of every scaled column and row are 1 (rtol 1e-2)."""
    from coolpdlp import generators as G
    lp, _, _ = G.random_milp_and_sol(10, 20, 0.4, seed=42)
    d1, d2 = oracle.preconditioner(lp, 10000, with_cp=False)
    A = lp.to_scipy()
    As = abs((A.multiply(d1[:, None])).multiply(d2[None, :])).tocsc()
    cn = As.max(axis=0).toarray().ravel()
    rn = As.max(axis=1).toarray().ravel()
    assert np.allclose(cn[cn > 0], 1, rtol=1e-2) and np.allclose(rn[rn > 0], 1, rtol=1e-2)
    # the full PDLP preconditioner = Ruiz diagonals times Pock-Chambolle (alpha=1)
    r1, r2 = oracle.preconditioner(lp, 10, with_cp=False)
    D1, D2 = oracle.preconditioner(lp, 10, with_cp=True)
    R = abs((A.multiply(r1[:, None])).multiply(r2[None, :])).tocsc()
    rs, cs = np.asarray(R.sum(axis=1)).ravel(), np.asarray(R.sum(axis=0)).ravel()
    np.testing.assert_allclose(D1, r1 / np.sqrt(np.where(rs == 0, 1, rs)), rtol=1e-13)
    np.testing.assert_allclose(D2, r2 / np.sqrt(np.where(cs == 0, 1, cs)), rtol=1e-13)


def test_preconditioning_round_trip(oracle):
    """test/components/preconditioning.jl:44-75: objective and A x invariant."""
    from coolpdlp import generators as G
    lp, x, y = G.random_milp_and_sol(10, 20, 0.4, seed=3)
    S = oracle.OracleState(lp, oracle.params())
    sc = S.scaled()
    xs = x / sc["D2"]
    assert math.isclose(float(np.dot(lp.c, x)), float(np.dot(sc["c"], xs)), rel_tol=1e-12)
    fin = np.isfinite(lp.lv)
    np.testing.assert_allclose((sc["lv"] * sc["D2"])[fin], lp.lv[fin], rtol=1e-14)


def test_pdlp_matches_highs(oracle):
    """test/algorithms/all.jl:20-38: objective vs HiGHS (rtol 1e-2 at 1e-4,
    here 1e-3 at 1e-5)."""
    from scipy.optimize import linprog
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(200, 400, 5, seed=3)
    x, y, st = oracle.solve(lp, oracle.params(termination_reltol=1e-5))
    assert st["termination_status"] == 0
    A = lp.to_scipy()
    eq = lp.lc == lp.uc
    r = linprog(lp.c, A_ub=A[~eq], b_ub=lp.uc[~eq], A_eq=A[eq], b_eq=lp.uc[eq],
                bounds=list(zip(lp.lv, lp.uv)), method="highs")
    assert r.status == 0
    assert abs(r.fun - lp.c @ x) <= 1e-3 * abs(r.fun)


def test_powm_default_tol_wraps_like_julia(oracle):
    """IterativeSolvers' tol = eps(T)*n^3 uses Int64 arithmetic."""
    f = oracle.lib().orc_powm_default_tol
    assert f(2000, 0) == 2.220446049250313e-16 * 8e9
    v = (4177920 ** 3) % 2 ** 64
    v = v - 2 ** 64 if v >= 2 ** 63 else v
    assert f(4177920, 0) == 2.220446049250313e-16 * float(v) < 0
