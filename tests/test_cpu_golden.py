"""CPU: the oracle against the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py): the reference suite's known answers, HiGHS
objectives (an independent solver) and the oracle's own recorded outputs
(bit-exact regression pins).  No GPU needed."""
import json
import math
import os
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden.npz")))
    return meta, arrays


@pytest.fixture(scope="module")
def lp_sets():
    sys.path.insert(0, GOLDEN)
    import make_golden
    return make_golden.lp_sets()


def test_known_answers(oracle, golden):
    """test/utils/linalg.jl:37-43 (combine) and test/moi.jl:38-53 (205)."""
    meta, _ = golden
    for l, u, want in meta["known"]["combine"]:
        assert oracle.scalar("combine", l, u) == want
    from coolpdlp import generators as G
    lp = G.two_variable_lp()
    x, _, st = oracle.solve(lp)
    assert st["termination_status"] == 0
    assert abs(float(lp.c @ x) - meta["known"]["two_variable_lp_objective"]) <= 1e-2


def test_conversions_pinned(oracle, golden):
    meta, a = golden
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(40, 60, 3, seed=5)
    assert np.array_equal(lp.colptr, a["conv_colptr"]) and np.array_equal(lp.rowval, a["conv_rowval"])
    ptr, idx, val = oracle.csr_from_csc(lp)
    assert np.array_equal(ptr, a["csr_ptr"]) and np.array_equal(idx, a["csr_idx"])
    assert np.array_equal(val, a["csr_val"])
    d, col, v = oracle.ell_from_csc(lp)
    assert d == meta["conv"]["ell_width"]
    assert np.array_equal(col, a["ell_col"]) and np.array_equal(v, a["ell_val"])
    r, c, v = oracle.coo_from_csc(lp)
    assert np.array_equal(r, a["coo_row"]) and np.array_equal(c, a["coo_col"])
    assert np.array_equal(v, a["coo_val"])


def test_preconditioner_pinned(oracle, golden):
    _, a = golden
    from coolpdlp import generators as G
    lp = G.random_sparse_lp(200, 400, 5, seed=11)
    D1, D2 = oracle.preconditioner(lp, 10, 1.0, True)
    assert np.array_equal(D1, a["prec_D1"]) and np.array_equal(D2, a["prec_D2"])


def test_kkt_pinned(oracle, golden):
    meta, _ = golden
    from coolpdlp import generators as G
    lp, x, y = G.random_milp_and_sol(60, 120, 0.2, seed=4)
    S = oracle.OracleState(lp, oracle.params())
    sc = S.scaled()
    e = S.kkt_of(x / sc["D2"], y / sc["D1"])
    S.close()
    for k, v in meta["kkt"]["errors"].items():
        assert e[k] == v, k


def test_solve_trajectories_pinned(oracle, golden):
    meta, _ = golden
    from coolpdlp import generators as G
    cases = [(G.random_sparse_lp(150, 300, 5, seed=2), 0),
             (G.random_sparse_lp(300, 600, 4, seed=8), 0),
             (G.random_sparse_lp(150, 300, 5, seed=2), 1),
             (G.multicommodity_flow_lp(side=6, K=2, seed=26), 0)]
    for (lp, algo), want in zip(cases, meta["solves"]):
        assert lp.name == want["name"]
        prm = oracle.params(algo)
        if algo == 1:
            prm.max_kkt_passes = 3000
        x, _, st = oracle.solve(lp, prm)
        assert st["termination_status"] == want["termination_status"]
        assert st["kkt_passes"] == want["kkt_passes"]
        assert st["power_iterations"] == want["power_iterations"]
        assert float(lp.c @ x) == want["objective"]


@pytest.mark.parametrize("kind", ["single", "batch", "flow"])
def test_oracle_matches_highs(oracle, golden, lp_sets, kind):
    """The oracle solved to 1e-8 relative KKT reaches HiGHS's optimal
    objective within 1e-6 relative (the bar stated for every solve)."""
    meta, _ = golden
    lps = lp_sets[kind]
    want = meta["highs"][kind]
    for lp, w in zip(lps, want):
        assert lp.name == w["name"]
        x, _, st = oracle.solve(lp, oracle.params(termination_reltol=1e-8, max_kkt_passes=400000,
                                                  time_limit=300.0))
        assert st["termination_status"] == 0, lp.name
        obj = float(lp.c @ x)
        assert abs(obj - w["objective"]) <= 1e-6 * max(1.0, abs(w["objective"])), (lp.name, obj, w)
