"""Infeasibility detection (an extension: infeasibility_tol > 0; the reference
has none and runs into its limits).  A primal-infeasible LP must end
PRIMAL_INFEASIBLE with a dual ray that certifies it, an unbounded LP
DUAL_INFEASIBLE with a primal ray; feasible LPs must still end OPTIMAL with
the same iterates as without detection (the check only reads them)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = np.inf


def _lp(A, c, lv, uv, lc, uc):
    from coolpdlp import generators as G
    import scipy.sparse as sp
    M = sp.csc_matrix(np.asarray(A, dtype=float))
    M.sort_indices()
    return G.LPData(M.shape[0], M.shape[1], M.indptr.astype(np.int64) + 1,
                    M.indices.astype(np.int64) + 1, M.data.astype(float), np.asarray(c, float),
                    np.asarray(lv, float), np.asarray(uv, float), np.asarray(lc, float),
                    np.asarray(uc, float))


def _solve(handle, lp, ft, tol, **kw):
    from coolpdlp import native, _abi as A
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    p = A.default_params_py()
    p.float_type = ft
    p.infeasibility_tol = tol
    p.max_kkt_passes = kw.get("max_kkt_passes", 20000)
    return native.solve_lp(handle, L, p)


@pytest.mark.parametrize("ft", [0, 1])
def test_primal_infeasible(handle, ft):
    from coolpdlp import _abi as A
    # x1 + x2 >= 3 with x in [0, 1]^2, plus an equality row that is fine
    lp = _lp([[1, 1, 0], [0, 1, 1]], [1, 1, 1], [0, 0, 0], [1, 1, INF], [3, 1], [INF, 1])
    x, y, st = _solve(handle, lp, ft, 1e-8)
    assert st.termination_status == A.PRIMAL_INFEASIBLE
    # the returned y is a dual ray: y1 > 0 on the >= row, A'y offset only by
    # multipliers of finite bounds, positive ray objective
    assert y[0] > 0
    g = -(np.array([[1, 1, 0], [0, 1, 1]]).T @ y)
    r = np.where(np.isfinite(lp.lv) & (g > 0), g, 0.0) + np.where(np.isfinite(lp.uv) & (g < 0), g, 0.0)
    obj = (np.where(y > 0, lp.lc * y, 0.0) + np.where(y < 0, np.where(np.isfinite(lp.uc), lp.uc, 0) * y, 0.0)).sum() \
        + (np.where(r > 0, lp.lv * r, 0.0) + np.where(r < 0, lp.uv * r, 0.0)).sum()
    assert obj > 0
    assert np.linalg.norm(g - r) <= 1e-6 * obj
    # without detection the reference behaviour: run into the pass limit
    _, _, st0 = _solve(handle, lp, ft, 0.0, max_kkt_passes=3000)
    assert st0.termination_status == A.ITERATION_LIMIT


@pytest.mark.parametrize("ft", [0, 1])
def test_dual_infeasible(handle, ft):
    from coolpdlp import _abi as A
    # min -x1 - x2 s.t. x1 - x2 >= -1, x >= 0: unbounded along x1 = x2 -> inf
    lp = _lp([[1, -1]], [-1, -1], [0, 0], [INF, INF], [-1], [INF])
    x, y, st = _solve(handle, lp, ft, 1e-8)
    assert st.termination_status == A.DUAL_INFEASIBLE
    assert np.all(x >= 0) and float(lp.c @ x) < 0
    assert x[0] - x[1] >= -1e-6 * np.linalg.norm(x)


@pytest.mark.parametrize("ft", [0, 1])
def test_feasible_lps_unchanged(handle, ft):
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    for lp in (G.random_sparse_lp(200, 400, 5, seed=3), G.multicommodity_flow_lp(side=6, K=2, seed=4),
               G.two_variable_lp()):
        x1, y1, s1 = _solve(handle, lp, ft, 1e-8)
        x0, y0, s0 = _solve(handle, lp, ft, 0.0)
        assert s1.termination_status == s0.termination_status == A.OPTIMAL
        assert s1.kkt_passes == s0.kkt_passes
        assert np.array_equal(x1, x0) and np.array_equal(y1, y0)


def test_moi_statuses(cuda_lib):
    from coolpdlp import moi
    # infeasible: x + y >= 3 with x, y in [0, 1]
    m = moi.Model()
    x = m.add_variable(lower=0.0, upper=1.0)
    y = m.add_variable(lower=0.0, upper=1.0)
    m.add_constraint({x: 1.0, y: 1.0}, moi.GreaterThan(3.0))
    m.set_objective({x: 1.0, y: 1.0}, sense=moi.Sense.MIN)
    opt = moi.Optimizer()
    opt.set_silent()
    opt.set_attribute("infeasibility_tol", 1e-8)
    opt.optimize(m)
    assert opt.termination_status == moi.TerminationStatusCode.INFEASIBLE
    assert opt.get_dual_status() == moi.ResultStatusCode.INFEASIBILITY_CERTIFICATE
    # unbounded: max x + y with x - y <= 1, x, y >= 0
    m2 = moi.Model()
    a = m2.add_variable(lower=0.0)
    b = m2.add_variable(lower=0.0)
    m2.add_constraint({a: 1.0, b: -1.0}, moi.LessThan(1.0))
    m2.set_objective({a: 1.0, b: 1.0}, sense=moi.Sense.MAX)
    opt2 = moi.Optimizer()
    opt2.set_silent()
    opt2.set_attribute("infeasibility_tol", 1e-8)
    opt2.optimize(m2)
    assert opt2.termination_status == moi.TerminationStatusCode.DUAL_INFEASIBLE
    assert opt2.get_primal_status() == moi.ResultStatusCode.INFEASIBILITY_CERTIFICATE
