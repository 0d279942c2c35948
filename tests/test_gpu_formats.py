"""The matrix_type of the solve (Algorithm{A}(T, Ti, M), conversion.jl:37-55):
M = "ELL" runs every product of the solve (steps, KKT checks, power method)
on the ELL engine, whose rows are summed in column order like the reference's
spmv_ell! loop; M = "COO" solves on the CSR engine; M = None lets the
autotuner choose.  Checked against the Float64 oracle: same termination
status, KKT passes and objective (1e-6 relative), as the CSR solves in
test_gpu_solver.py; an ELL solve also matches the CSR solve of the same LP."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lps():
    from coolpdlp import generators as G
    return [G.random_sparse_lp(200, 400, 5, seed=3), G.random_sparse_lp(1000, 2000, 5, seed=0),
            G.multicommodity_flow_lp(side=8, K=3, seed=2),
            G.powerlaw_lp(2000, 4000, 24000, seed=3, cap=20000)]


@pytest.mark.parametrize("M", ["ELL", "COO"])
def test_matrix_type_solves_match_oracle(handle, oracle, M):
    import coolpdlp as cp
    for lp in _lps():
        xo, yo, so = oracle.solve(lp, oracle.params(max_kkt_passes=400000))
        milp = cp.MILP.from_lpdata(lp)
        algo = cp.PDLP(np.float64, M=M, max_kkt_passes=400000)
        dm, sol0 = cp.preprocess(milp, cp.PrimalDualSolution(np.zeros(lp.n), np.zeros(lp.m)), algo)
        lay = dm.problem.layout()
        want = "ELL" if M == "ELL" else "CSR"
        assert lay["A"]["format"] == lay["At"]["format"] == want, lay
        if M == "ELL":
            widths = np.diff(lp.to_scipy().tocsr().indptr).max(), np.diff(lp.colptr).max()
            assert (lay["A"]["ell_width"], lay["At"]["ell_width"]) == tuple(int(w) for w in widths)
        sol, st = cp.solve(milp, algo)
        assert int(st.termination_status) == so["termination_status"], lp.name
        assert st.kkt_passes == so["kkt_passes"], (lp.name, M, st.kkt_passes, so["kkt_passes"])
        og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
        assert abs(og - oo) <= 1e-6 * max(1.0, abs(oo)), (lp.name, og, oo)


def test_ell_fp32_and_narrow_solves(handle, oracle):
    """FP32 iterates on the ELL engine, with valued and with narrow +-1 storage
    (the flow LP), reach OPTIMAL with the oracle's objective within 1e-3."""
    import coolpdlp as cp
    from coolpdlp import generators as G
    for lp in (_lps()[0], G.multicommodity_flow_lp(side=10, K=3, seed=4)):
        xo, _, so = oracle.solve(lp, oracle.params())
        sol, st = cp.solve(cp.MILP.from_lpdata(lp), cp.PDLP(np.float32, M="ELL"))
        assert st.termination_status == cp.OPTIMAL and cp.relative(st.err) <= 1e-4
        og, oo = float(lp.c @ sol.x), float(lp.c @ xo)
        assert abs(og - oo) <= 1e-3 * max(1.0, abs(oo)), (lp.name, og, oo)


def test_ell_steps_match_oracle_on_long_rows(handle, oracle):
    """The ELL engine sums every row sequentially in column order, the
    oracle's order, also on rows longer than 64 nonzeros (the power-law LP):
    FP64 iterates stay within 1e-9 relative of the oracle's after 50 steps."""
    from coolpdlp import native
    lp = _lps()[3]
    prm = oracle.params()
    prm.matrix_type = 1  # CPDLP_FMT_ELL
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    P = native.Problem(handle, L, prm)
    st = native.State(P, prm)
    S = oracle.OracleState(lp, prm)
    st.step(50)
    S.step(50)
    xg, yg = st.vectors(0)
    xo, yo = S.vectors(0)
    assert np.max(np.abs(xg - xo)) <= 1e-9 * max(1.0, np.max(np.abs(xo)))
    assert np.max(np.abs(yg - yo)) <= 1e-9 * max(1.0, np.max(np.abs(yo)))
    S.close()
