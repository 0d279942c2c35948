"""CPU: the MOI optimizer mirror's model conversion and bookkeeping
(src/moi.jl:1-7 row order by set, :168-196 conversion, :49-76 empty!)."""
import math

import numpy as np
import pytest


def _two_variable_model(sense=None):
    from coolpdlp import moi
    m = moi.Model()
    x = m.add_variable(lower=0.0)
    y = m.add_variable(lower=0.0, upper=3.0)
    c1 = m.add_constraint({x: 6.0, y: 8.0}, moi.GreaterThan(100.0))
    c2 = m.add_constraint([(x, 7.0), (y, 12.0)], moi.GreaterThan(120.0))
    m.set_objective({x: 12.0, y: 20.0}, sense=sense or moi.Sense.MIN)
    return m, x, y, c1, c2


def test_conversion_matches_two_variable_lp():
    from coolpdlp import generators as G
    m, *_ = _two_variable_model()
    milp, c = m.to_milp()
    ref = G.two_variable_lp()
    assert np.array_equal(milp.A.colptr, ref.colptr) and np.array_equal(milp.A.rowval, ref.rowval)
    assert np.array_equal(milp.A.nzval, ref.nzval)
    assert np.array_equal(c, ref.c) and np.array_equal(milp.lv, ref.lv)
    assert np.array_equal(milp.uv, ref.uv) and np.array_equal(milp.lc, ref.lc)
    assert np.array_equal(milp.uc, ref.uc)


def test_rows_grouped_by_set_and_sense():
    from coolpdlp import moi
    m = moi.Model()
    a, b = m.add_variable(), m.add_variable(lower=-1.0, upper=1.0)
    cl = m.add_constraint({a: 1.0}, moi.LessThan(4.0))
    ce = m.add_constraint({a: 1.0, b: 1.0}, moi.EqualTo(2.0))
    ci = m.add_constraint({b: 2.0, a: 1.0, }, moi.Interval(-3.0, 3.0))
    cg = m.add_constraint({b: 1.0, a: 0.5}, moi.GreaterThan(-5.0))
    # EqualTo, GreaterThan, LessThan, Interval
    assert [m.rows(ci_) for ci_ in (ce, cg, cl, ci)] == [0, 1, 2, 3]
    m.set_objective({a: 1.0, b: -2.0, a: 1.0}, constant=3.0, sense=moi.Sense.MAX)
    milp, c = m.to_milp()
    assert np.array_equal(c, [-1.0, 2.0])
    assert np.array_equal(milp.lc, [2.0, -5.0, -np.inf, -3.0])
    assert np.array_equal(milp.uc, [2.0, np.inf, 4.0, 3.0])
    D = milp.A.to_scipy().toarray()
    assert np.array_equal(D, [[1, 1], [0.5, 1], [1, 0], [1, 2]])
    # repeated terms add up
    k = m.add_constraint([(a, 1.0), (a, 2.0)], moi.EqualTo(0.0))
    milp, _ = m.to_milp()
    assert milp.A.to_scipy().toarray()[1, 0] == 3.0


def test_empty_and_attributes():
    from coolpdlp import moi
    opt = moi.Optimizer()
    assert opt.is_empty() and opt.result_count == 0
    assert opt.raw_status_string == "OPTIMIZE_NOT_CALLED"
    opt.set_time_limit_sec(12)
    assert opt.get_time_limit_sec() == 12.0
    opt.set_time_limit_sec(None)
    assert opt.get_time_limit_sec() is None
    opt.set_attribute("termination_reltol", 1e-6)
    assert opt.get_attribute("termination_reltol") == 1e-6
    assert opt.get_primal_status() == moi.ResultStatusCode.NO_SOLUTION
    with pytest.raises(IndexError):
        opt.objective_value()
    with pytest.raises(TypeError):
        moi.Model().add_constraint({}, object())


def test_proj_multiplier_and_safeprod():
    from coolpdlp.moi import _proj_multiplier as pm, _safeprod_left as sp
    assert pm(2.0, -math.inf, math.inf) == 0.0
    assert pm(-2.0, 0.0, math.inf) == 0.0 and pm(2.0, 0.0, math.inf) == 2.0
    assert pm(2.0, -math.inf, 1.0) == 0.0 and pm(-2.0, -math.inf, 1.0) == -2.0
    assert pm(-2.0, 0.0, 1.0) == -2.0
    assert np.array_equal(sp([np.inf, 2.0], [3.0, 3.0]), [3.0, 6.0])
