"""GPU parity of the solve path (preconditioning, step size, step!, KKT errors,
restarts, termination) against the Float64 CPU oracle, through the C ABI.

Tolerances: scaling diagonals bit-identical (max/one-norm sums in the
reference's order); step iterates within 1e-10 relative; full Float64 solves
must reach the same termination status after the same number of KKT passes
with the objective within 1e-6 relative and KKT errors within 1e-6 relative
(the reference's own CPU/GPU coherence standard, test/algorithms/all.jl:64-73).
Float32 solves must reach OPTIMAL with the objective within 1e-3 relative of
the Float64 oracle."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _native_problem(handle, lp, prm):
    from coolpdlp import native
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    return L, native.Problem(handle, L, prm)


def _lps(solvable_only: bool = False):
    """Feasible, bounded LPs (solve parity) plus, for the scaling / step tests,
    a random LP with random infinite bounds that PDLP does not solve."""
    from coolpdlp import generators as G
    out = [G.random_sparse_lp(200, 400, 5, seed=3), G.random_sparse_lp(1000, 2000, 5, seed=0),
           G.multicommodity_flow_lp(side=8, K=3, seed=2)]
    if not solvable_only:
        lp, _, _ = G.random_milp_and_sol(60, 120, 0.1, seed=4)
        out.append(lp)
    return out


def test_scaling_bit_exact(handle, oracle):
    for lp in _lps():
        for ruiz, alpha in ((10, 1.0), (0, 1.0), (3, 0.5)):
            prm = oracle.params(ruiz_iter=ruiz, chambolle_pock_alpha=alpha)
            _, P = _native_problem(handle, lp, prm)
            d1, d2 = P.scaling()
            S = oracle.OracleState(lp, prm)
            sc = S.scaled()
            if alpha == 1.0:
                assert np.array_equal(d1, sc["D1"]) and np.array_equal(d2, sc["D2"]), lp.name
            else:  # generic p-norm uses pow(): libm and CUDA may differ in the last bit
                np.testing.assert_allclose(d1, sc["D1"], rtol=1e-13)
                np.testing.assert_allclose(d2, sc["D2"], rtol=1e-13)
            S.close()
            P.close()


def test_step_size_and_primal_weight(handle, oracle):
    from coolpdlp import native
    for lp in _lps():
        prm = oracle.params()
        _, P = _native_problem(handle, lp, prm)
        st = native.State(P, prm).stats()
        S = oracle.OracleState(lp, prm)
        so = S.stats()
        assert math.isclose(st.eta, so["eta"], rel_tol=1e-10), (st.eta, so["eta"])
        assert math.isclose(st.omega, so["omega"], rel_tol=1e-12)
        assert abs(st.power_iterations - so["power_iterations"]) <= 2


@pytest.mark.parametrize("algorithm", [0, 1])
def test_steps_match_oracle(handle, oracle, algorithm):
    from coolpdlp import native
    for lp in (_lps()[0], _lps()[1], _lps()[3]):
        prm = oracle.params(algorithm)
        _, P = _native_problem(handle, lp, prm)
        st = native.State(P, prm)
        S = oracle.OracleState(lp, prm)
        # same starting eta (the power method sums in a different order)
        eta_g = st.stats().eta
        done = 0
        for k in (1, 9, 90, 200):
            st.step(k)
            S.step(k)
            done += k
            for which in (0, 1, 2, 3) if algorithm == 0 else (0, 1):
                xg, yg = st.vectors(which)
                xo, yo = S.vectors(which)
                sx = max(1.0, np.max(np.abs(xo)))
                sy = max(1.0, np.max(np.abs(yo)))
                # eta agrees to ~1e-13; the drift stays far below this bound
                assert np.max(np.abs(xg - xo)) <= 1e-9 * sx * max(1, done / 10), (lp.name, k, which)
                assert np.max(np.abs(yg - yo)) <= 1e-9 * sy * max(1, done / 10), (lp.name, k, which)
        ek = st.kkt(0)
        eo = S.kkt(0)
        for f in ("primal", "dual", "gap", "primal_scale", "dual_scale", "gap_scale"):
            assert math.isclose(getattr(ek, f), eo[f], rel_tol=1e-7, abs_tol=1e-12), f
        assert st.stats().kkt_passes == S.stats()["kkt_passes"] == done
        del eta_g


@pytest.mark.parametrize("algorithm", [0, 1])
def test_solve_matches_oracle_f64(handle, oracle, algorithm):
    import coolpdlp as cp
    for lp in _lps(solvable_only=True):
        kw = {} if algorithm == 0 else {"termination_reltol": 1e-3, "max_kkt_passes": 200000}
        prm = oracle.params(algorithm, **kw)
        xo, yo, so = oracle.solve(lp, prm)
        milp = cp.MILP.from_lpdata(lp)
        algo = (cp.PDLP if algorithm == 0 else cp.PDHG)(np.float64, **kw)
        sol, stats = cp.solve(milp, algo)
        assert int(stats.termination_status) == so["termination_status"], lp.name
        assert stats.kkt_passes == so["kkt_passes"], (lp.name, stats.kkt_passes, so["kkt_passes"])
        assert len(stats.error_history) == so["history_length"]
        og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
        assert abs(og - oo) <= 1e-6 * max(1.0, abs(oo)), (lp.name, og, oo)
        for f in ("primal", "dual", "gap"):
            assert math.isclose(getattr(stats.err, f), so["err"][f], rel_tol=1e-6,
                                abs_tol=1e-10), (lp.name, f)
        if algorithm == 0:
            assert stats.outer == so["outer"] and stats.inner == so["inner"]
            assert math.isclose(stats.omega, so["omega"], rel_tol=1e-8)


def test_solve_f32_reaches_oracle_objective(handle, oracle):
    import coolpdlp as cp
    for lp in _lps()[:2]:
        xo, yo, so = oracle.solve(lp, oracle.params())
        sol, stats = cp.solve(cp.MILP.from_lpdata(lp), cp.PDLP(np.float32))
        assert stats.termination_status == cp.OPTIMAL
        assert cp.relative(stats.err) <= 1e-4
        og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
        assert abs(og - oo) <= 1e-3 * max(1.0, abs(oo)), (og, oo)


def test_two_variable_lp_known_answer(handle):
    """test/moi.jl:38-53: objective 205 (atol 1e-2), in Float64 and Float32."""
    import coolpdlp as cp
    from coolpdlp import generators as G
    milp = cp.MILP.from_lpdata(G.two_variable_lp())
    for T in (np.float64, np.float32):
        sol, stats = cp.solve(milp, cp.PDLP(T))
        assert stats.termination_status == cp.OPTIMAL
        assert abs(cp.objective_value(sol.x, milp) - 205.0) <= 1e-2


def test_termination_check_not_skipped(handle):
    """test/algorithms/all.jl 'Termination check not skipped'."""
    import coolpdlp as cp
    from coolpdlp import generators as G
    sol, stats = cp.solve(cp.MILP.from_lpdata(G.termination_check_lp()), cp.PDLP())
    assert stats.termination_status == cp.OPTIMAL


def test_limits_and_early_exit(handle):
    import coolpdlp as cp
    from coolpdlp import generators as G
    milp = cp.MILP.from_lpdata(G.random_sparse_lp(200, 400, 5, seed=3))
    _, st = cp.solve(milp, cp.PDLP(max_kkt_passes=300, termination_reltol=1e-12))
    assert st.termination_status == cp.ITERATION_LIMIT and st.kkt_passes == 300
    _, st = cp.solve(milp, cp.PDLP(time_limit=0.0, termination_reltol=1e-12))
    assert st.termination_status == cp.TIME_LIMIT and st.kkt_passes == 100
    # no constraints, zero cost: x = proj_box(0, lv, uv) (common.jl:194-198)
    e = cp.MILP(c=np.zeros(3), lv=np.array([1.0, -2.0, -np.inf]), uv=np.array([2.0, -1.0, 5.0]),
                A=np.zeros((0, 3)), lc=np.zeros(0), uc=np.zeros(0))
    sol, st = cp.solve(e, cp.PDLP())
    assert st.termination_status == cp.OPTIMAL
    assert np.array_equal(sol.x, [1.0, -1.0, 0.0])


def test_warm_start_matches_oracle(handle, oracle):
    import coolpdlp as cp
    from coolpdlp import generators as G
    lp, x0, y0 = G.random_milp_and_sol(50, 100, 0.2, seed=8)
    prm = oracle.params(max_kkt_passes=2000)
    xo, yo, so = oracle.solve(lp, prm, x0, y0)
    sol, st = cp.solve(cp.MILP.from_lpdata(lp), cp.PrimalDualSolution(x0, y0),
                       cp.PDLP(max_kkt_passes=2000))
    assert int(st.termination_status) == so["termination_status"]
    assert st.kkt_passes == so["kkt_passes"]
    np.testing.assert_allclose(sol.x, xo, rtol=1e-6, atol=1e-8)


def test_fp32_with_fp64_refinement_reaches_1e8(handle, oracle):
    """FP32 iterates to 1e-4, then FP64 refinement to 1e-8 relative KKT; the
    objective must agree with the Float64 oracle solved to 1e-8."""
    import coolpdlp as cp
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(300, 600, 5, seed=7)
    xo, yo, so = oracle.solve(lp, oracle.params(termination_reltol=1e-8, max_kkt_passes=200000))
    assert so["termination_status"] == 0
    milp = cp.MILP.from_lpdata(lp)
    sol, st = cp.solve(milp, cp.PDLP(np.float32, refine_reltol=1e-8, max_kkt_passes=200000))
    assert st.termination_status == cp.OPTIMAL
    assert cp.relative(st.err) <= 1e-8
    assert st.refine_kkt_passes > 0 and st.kkt_passes > st.refine_kkt_passes
    og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
    assert abs(og - oo) <= 1e-6 * max(1.0, abs(oo)), (og, oo)
    # error_history covers every phase (common.jl:226-228): FP32 checks at
    # multiples of check_every, then the refinement checks; passes never
    # decrease, the last entry is the final error
    hist = st.error_history
    assert len(hist) >= 2
    passes = [p for p, _ in hist]
    assert passes == sorted(passes) and passes[-1] == st.kkt_passes
    assert passes[0] % 100 == 0 and passes[0] > 0
    assert cp.relative(hist[-1][1]) == cp.relative(st.err)
    assert any(p > st.kkt_passes - st.refine_kkt_passes for p in passes)
    _, st_nohist = cp.solve(milp, cp.PDLP(np.float32, refine_reltol=1e-8, max_kkt_passes=200000,
                                          record_error_history=0))
    assert st_nohist.error_history == []
    # the same through the C ABI (cpdlp_solve)
    from coolpdlp import native, _abi as A
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc, lp.uc)
    p = A.default_params_py(); p.float_type = A.VAL_F32; p.refine_reltol = 1e-8
    p.max_kkt_passes = 200000
    x, y, s = native.solve_lp(handle, L, p)
    assert s.termination_status == 0 and s.refine_kkt_passes > 0
    assert abs(float(lp.c @ x) - oo) <= 1e-6 * max(1.0, abs(oo))


def test_pdhg_fp32_refinement_runs(handle):
    """PDHG (no restarts, no averages) through the mixed-precision path: FP32
    phase, refinement rounds on the residual LP, FP64 continuation if needed.
    PDHG converges sublinearly, so the check is the plumbing: a consistent
    status, and at OPTIMAL the tolerance met and the Float64 path's objective."""
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(120, 240, 5, seed=21)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    p = A.default_params_py(A.ALGO_PDHG)
    p.float_type = A.VAL_F32
    p.refine_reltol = 1e-5
    p.max_kkt_passes = 100000
    x, y, st = native.solve_lp(handle, L, p)
    e = st.err
    rel = max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)
    assert st.termination_status in (A.OPTIMAL, A.ITERATION_LIMIT)
    if st.termination_status == A.ITERATION_LIMIT:
        assert st.kkt_passes >= p.max_kkt_passes
        return
    assert rel <= 1e-5
    p64 = A.default_params_py(A.ALGO_PDHG)
    p64.termination_reltol = 1e-5
    x64, _, st64 = native.solve_lp(handle, L, p64)
    if st64.termination_status == A.OPTIMAL:
        o, o64 = float(lp.c @ x), float(lp.c @ x64)
        assert abs(o - o64) <= 1e-3 * max(1.0, abs(o64))
