"""Density order inside the solver (CPDLP_TILE_DENSITY_ORDER): the rows and
columns of the problem's matrices in the order of the reference's
sort_rows_columns (src/components/permutation.jl:1-46), each row keeping its
entries in their input order, and every vector crossing the C ABI in the
caller's order.  Checked against the oracle restatement of sort_rows_columns
(the orders), against the Float64 oracle (iterates after 50 steps within
1e-9 relative, whole solves with its status, KKT passes and objective within
1e-6; FP32 solves within 1e-3; a refined FP32 solve to 1e-8 within 1e-6 of the
committed oracle and HiGHS objectives) and against the same solve without
the order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lp_struct(lp):
    from coolpdlp import native
    return native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                           lp.lc, lp.uc)


def _lps():
    from coolpdlp import generators as G
    return [G.powerlaw_lp(2000, 4000, 24000, seed=3, cap=20000),
            G.random_sparse_lp(1000, 2000, 5, seed=0)]


def test_density_order_is_sort_rows_columns(handle, oracle):
    from coolpdlp import _abi as A
    from coolpdlp import native
    for lp in _lps():
        prm = oracle.params()
        prm.tile_flags = A.TILE_DENSITY_ORDER
        P = native.Problem(handle, _lp_struct(lp), prm)
        orow, ocol = P.order()
        pv, pc, *_ = oracle.sort_rows_columns(lp)
        assert np.array_equal(orow, pc) and np.array_equal(ocol, pv), lp.name
        # the scalings come back in the caller's order
        prm0 = oracle.params()
        prm0.tile_flags = A.TILE_NO_DENSITY_ORDER
        P0 = native.Problem(handle, _lp_struct(lp), prm0)
        assert P0.order() is None
        d1, d2 = P.scaling()
        e1, e2 = P0.scaling()
        assert np.array_equal(d1, e1) and np.array_equal(d2, e2)


def test_density_order_steps_match_oracle(handle, oracle):
    """Every row's products and sum are those of the unordered problem, so the
    iterates differ from the oracle's only through the FP64 reductions' order."""
    from coolpdlp import _abi as A
    from coolpdlp import native
    lp = _lps()[0]
    prm = oracle.params()
    prm.tile_flags = A.TILE_DENSITY_ORDER
    P = native.Problem(handle, _lp_struct(lp), prm)
    assert P.order() is not None
    x0 = np.linspace(0.0, 1.0, lp.n)
    y0 = np.linspace(-1.0, 1.0, lp.m)
    st = native.State(P, prm, x0, y0)
    S = oracle.OracleState(lp, prm, x0, y0)
    st.step(50)
    S.step(50)
    for which in (A.VEC_SOL, A.VEC_SOL_AVG):
        xg, yg = st.vectors(which)
        xo, yo = S.vectors(which)
        assert np.max(np.abs(xg - xo)) <= 1e-9 * max(1.0, np.max(np.abs(xo)))
        assert np.max(np.abs(yg - yo)) <= 1e-9 * max(1.0, np.max(np.abs(yo)))
    S.close()


@pytest.mark.parametrize("ft", ["f64", "f32"])
def test_density_order_solves(handle, oracle, ft):
    import coolpdlp as cp
    from coolpdlp import _abi as A
    T = np.float64 if ft == "f64" else np.float32
    for lp in _lps():
        xo, yo, so = oracle.solve(lp, oracle.params(max_kkt_passes=400000))
        milp = cp.MILP.from_lpdata(lp)
        on = cp.PDLP(T, max_kkt_passes=400000, tile_flags=A.TILE_DENSITY_ORDER)
        off = cp.PDLP(T, max_kkt_passes=400000, tile_flags=A.TILE_NO_DENSITY_ORDER)
        sol, st = cp.solve(milp, on)
        sol0, st0 = cp.solve(milp, off)
        og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
        if ft == "f64":
            assert int(st.termination_status) == so["termination_status"], lp.name
            # the FP64 reductions run in another order, which may move a
            # restart decision: the pass count within 2% of the oracle's
            assert abs(st.kkt_passes - so["kkt_passes"]) <= 0.02 * so["kkt_passes"], \
                (lp.name, st.kkt_passes, so["kkt_passes"])
            assert abs(og - oo) <= 1e-6 * max(1.0, abs(oo)), (lp.name, og, oo)
        else:
            assert st.termination_status == cp.OPTIMAL and cp.relative(st.err) <= 1e-4
            assert abs(og - oo) <= 1e-3 * max(1.0, abs(oo)), (lp.name, og, oo)
        # x and y are in the caller's order: the rows' activities of the
        # caller's A lie within the caller's bounds (a wrong order would not)
        ax = lp.to_scipy() @ sol.x
        viol = np.maximum(lp.lc - ax, 0.0) + np.maximum(ax - lp.uc, 0.0)
        viol[~np.isfinite(viol)] = 0.0
        bnd = np.where(np.isfinite(lp.lc), np.abs(lp.lc), 0.0) + \
            np.where(np.isfinite(lp.uc), np.abs(lp.uc), 0.0)
        assert np.linalg.norm(viol) <= 1e-3 * (1.0 + np.linalg.norm(bnd)), lp.name
        assert abs(float(lp.c @ sol0.x) - og) <= 1e-3 * max(1.0, abs(og))


def test_density_order_refined_solve(handle):
    """FP32 iterates with refinement to 1e-8 on the scaled-down power-law LP:
    the FP64 copy of the problem takes the same order, and the objective is
    within 1e-6 of the oracle's and HiGHS's (committed fixtures)."""
    import json
    import os
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    from coolpdlp import native
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "golden.json")) as f:
        g = json.load(f)["powerlaw"]
    lp = G.powerlaw_lp(5000, 10000, 60000, seed=1, cap=20000)
    assert lp.name == g["name"]
    p = native.default_params()
    p.float_type = A.VAL_F32
    p.refine_reltol = 1e-8
    p.max_kkt_passes = 4_000_000
    p.time_limit = 300.0
    p.tile_flags = A.TILE_DENSITY_ORDER
    x, _, st = native.solve_lp(handle, _lp_struct(lp), p)
    e = st.err
    rel = max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)
    assert st.termination_status == A.OPTIMAL and rel <= 1e-8, (st.termination_status, rel)
    obj = float(lp.c @ x)
    for ref in (g["oracle_1e-08"]["objective"], g["highs_objective"]):
        assert abs(obj - ref) <= 1e-6 * max(1.0, abs(ref)), (obj, ref)
