"""GPU: the MOI optimizer mirror end to end (src/moi.jl:168-246, the
reference's test/moi.jl: the two-variable LP with optimum 205 within 1e-2,
Float32 solves with the mismatched-type warning), plus a maximisation with
duals checked against HiGHS."""
import math
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(sense):
    from coolpdlp import moi
    m = moi.Model()
    x = m.add_variable(lower=0.0)
    y = m.add_variable(lower=0.0, upper=3.0)
    c1 = m.add_constraint({x: 6.0, y: 8.0}, moi.GreaterThan(100.0))
    c2 = m.add_constraint({x: 7.0, y: 12.0}, moi.GreaterThan(120.0))
    m.set_objective({x: 12.0, y: 20.0}, sense=sense)
    return m, x, y, c1, c2


def test_two_variable_lp(cuda_lib):
    from coolpdlp import moi
    m, x, y, c1, c2 = _model(moi.Sense.MIN)
    opt = moi.Optimizer()
    opt.set_silent()
    opt.optimize(m)
    assert opt.termination_status == moi.TerminationStatusCode.OPTIMAL
    assert opt.get_primal_status() == moi.ResultStatusCode.FEASIBLE_POINT
    assert abs(opt.objective_value() - 205.0) <= 1e-2
    assert abs(opt.dual_objective_value() - 205.0) <= 1e-1
    # both constraints are >= rows of a minimisation: duals >= 0 (up to the tolerance)
    assert opt.constraint_dual(c1) >= -1e-6 and opt.constraint_dual(c2) >= -1e-6
    assert opt.constraint_dual((x, moi.GreaterThan)) >= 0.0
    assert opt.constraint_dual((y, moi.LessThan)) <= 0.0
    assert opt.solve_time > 0 and opt.result_count == 1


def test_float32_warns_and_returns_float64(cuda_lib):
    from coolpdlp import moi
    m, x, y, *_ = _model(moi.Sense.MIN)
    opt = moi.Optimizer()
    opt.set_silent()
    opt.set_attribute("float_type", np.float32)
    with pytest.warns(UserWarning, match="Got mismatched float type"):
        opt.optimize(m)
    assert opt.termination_status == moi.TerminationStatusCode.OPTIMAL
    assert abs(opt.objective_value() - 205.0) <= 1e-2
    assert isinstance(opt.variable_primal(x), float)
    opt32 = moi.Optimizer(np.float32)
    opt32.set_silent()
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        opt32.optimize(m)
    assert abs(opt32.objective_value() - 205.0) <= 1e-2


def test_maximisation_and_limits_against_highs(cuda_lib):
    from scipy.optimize import linprog
    from coolpdlp import moi
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(60, 120, 4, seed=3)
    m = moi.Model()
    xs = [m.add_variable(lower=lp.lv[j], upper=lp.uv[j]) for j in range(lp.n)]
    A = lp.to_scipy().tocsr()
    for i in range(lp.m):
        row = {xs[j]: A[i, j] for j in A[i].indices}
        s = moi.EqualTo(lp.uc[i]) if lp.lc[i] == lp.uc[i] else moi.LessThan(lp.uc[i])
        m.add_constraint(row, s)
    m.set_objective({xs[j]: -lp.c[j] for j in range(lp.n)}, constant=1.5, sense=moi.Sense.MAX)
    opt = moi.Optimizer()
    opt.set_silent()
    opt.set_attribute("termination_reltol", 1e-8)
    opt.optimize(m)
    eq = lp.lc == lp.uc
    r = linprog(lp.c, A_ub=A[~eq], b_ub=lp.uc[~eq], A_eq=A[eq], b_eq=lp.uc[eq],
                bounds=list(zip(lp.lv, lp.uv)), method="highs")
    want = -r.fun + 1.5
    assert opt.termination_status == moi.TerminationStatusCode.OPTIMAL
    assert abs(opt.objective_value() - want) <= 1e-6 * max(1.0, abs(want))
    assert abs(opt.dual_objective_value() - want) <= 1e-5 * max(1.0, abs(want))
    # an iteration limit maps to ITERATION_LIMIT with unknown result statuses
    opt.set_attribute("termination_reltol", 1e-12)
    opt.set_attribute("max_kkt_passes", 200)
    opt.optimize(m)
    assert opt.termination_status == moi.TerminationStatusCode.ITERATION_LIMIT
    assert opt.get_primal_status() == moi.ResultStatusCode.UNKNOWN_RESULT_STATUS


def test_reduced_costs_on_device_match_host_formula(handle):
    """cpdlp_reduced_costs (z and the dual objective of moi.jl:215-227, FP64
    on the device) against the same formulas evaluated on the host, for a
    random LP with infinite bounds of every kind and a random y."""
    from coolpdlp import generators as G
    from coolpdlp import native
    from coolpdlp.moi import _proj_multiplier, _safeprod_left
    lp, _, _ = G.random_milp_and_sol(300, 500, 0.05, seed=9)
    y = np.random.default_rng(3).standard_normal(lp.m)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    z, dual = native.reduced_costs(handle, L, y)
    At = lp.to_scipy().T.tocsr()
    z_ref = np.array([_proj_multiplier(g, l, u) for g, l, u in zip(lp.c - At @ y, lp.lv, lp.uv)])
    dual_ref = (np.sum(_safeprod_left(lp.lc, np.maximum(y, 0.0)))
                - np.sum(_safeprod_left(lp.uc, np.maximum(-y, 0.0)))
                + np.sum(_safeprod_left(lp.lv, np.maximum(z_ref, 0.0)))
                - np.sum(_safeprod_left(lp.uv, np.maximum(-z_ref, 0.0))))
    scale = 1.0 + np.abs(lp.c) + np.abs(At) @ np.abs(y)
    assert np.max(np.abs(z - z_ref) / scale) <= 1e-13
    assert abs(dual - dual_ref) <= 1e-10 * (1.0 + abs(dual_ref))
