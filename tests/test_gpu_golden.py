"""GPU: the device path against the committed golden fixtures (tests/golden/):
bit-exact matrix conversions and scaling diagonals, the oracle's recorded FP64
solve trajectories (same KKT passes and status, objective within 1e-6), and
HiGHS objectives (1e-6 relative at a 1e-8 relative KKT tolerance) for the
single-LP path in FP64 and FP32 + FP64 refinement and for the batched path.
No oracle is run here: the fixtures carry the answers."""
import json
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(GOLDEN, "golden.npz")))


@pytest.fixture(scope="module")
def lp_sets():
    sys.path.insert(0, GOLDEN)
    import make_golden
    return make_golden.lp_sets()


def _struct(lp):
    from coolpdlp import native
    return native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                           lp.lc, lp.uc)


def test_device_conversions_match_golden(handle, golden):
    import coolpdlp as cp
    from coolpdlp import generators as G
    meta, a = golden
    lp = G.random_sparse_lp(40, 60, 3, seed=5)
    A = cp.CSCMatrix(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval)
    csr = cp.GPUSparseMatrixCSR(A, np.float64)
    ptr, idx, val = csr.export()
    assert np.array_equal(ptr, a["csr_ptr"]) and np.array_equal(idx, a["csr_idx"])
    assert np.array_equal(val, a["csr_val"])
    ell = cp.GPUSparseMatrixELL(A, np.float64)
    _, col, v = ell.export()
    assert ell.width == meta["conv"]["ell_width"]
    assert np.array_equal(col.ravel(order="F"), a["ell_col"])
    assert np.array_equal(v.ravel(order="F"), a["ell_val"])
    coo = cp.GPUSparseMatrixCOO(A, np.float64)
    r, c, v = coo.export()
    assert np.array_equal(r, a["coo_row"]) and np.array_equal(c, a["coo_col"])
    assert np.array_equal(v, a["coo_val"])


def test_device_scaling_matches_golden(handle, golden):
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    _, a = golden
    lp = G.random_sparse_lp(200, 400, 5, seed=11)
    P = native.Problem(handle, _struct(lp), A.default_params_py())
    D1, D2 = P.scaling()
    assert np.array_equal(D1, a["prec_D1"]) and np.array_equal(D2, a["prec_D2"])


def test_device_trajectories_match_golden(handle, golden):
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    meta, _ = golden
    cases = [(G.random_sparse_lp(150, 300, 5, seed=2), 0),
             (G.random_sparse_lp(300, 600, 4, seed=8), 0),
             (G.random_sparse_lp(150, 300, 5, seed=2), 1),
             (G.multicommodity_flow_lp(side=6, K=2, seed=26), 0)]
    for (lp, algo), want in zip(cases, meta["solves"]):
        prm = A.default_params_py(algo)
        if algo == 1:
            prm.max_kkt_passes = 3000
        x, _, st = native.solve_lp(handle, _struct(lp), prm)
        assert st.termination_status == want["termination_status"], lp.name
        assert st.kkt_passes == want["kkt_passes"], lp.name
        obj = float(lp.c @ x)
        assert abs(obj - want["objective"]) <= 1e-6 * max(1.0, abs(want["objective"])), lp.name


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_single_lp_path_matches_highs(handle, golden, lp_sets, mode):
    from coolpdlp import native, _abi as A
    meta, _ = golden
    prm = A.default_params_py()
    prm.max_kkt_passes = 400000
    if mode == "fp64":
        prm.termination_reltol = 1e-8
    else:
        prm.float_type = A.VAL_F32
        prm.refine_reltol = 1e-8
    for kind in ("single", "flow"):
        for lp, w in zip(lp_sets[kind], meta["highs"][kind]):
            x, _, st = native.solve_lp(handle, _struct(lp), prm)
            assert st.termination_status == 0, (mode, lp.name)
            obj = float(lp.c @ x)
            assert abs(obj - w["objective"]) <= 1e-6 * max(1.0, abs(w["objective"])), (mode, lp.name)


@pytest.mark.parametrize("float_type", [0, 1])
def test_batched_path_matches_highs(handle, golden, lp_sets, float_type):
    from coolpdlp import native, _abi as A
    meta, _ = golden
    lps = lp_sets["batch"] + lp_sets["flow"]
    want = meta["highs"]["batch"] + meta["highs"]["flow"]
    prm = A.default_params_py()
    prm.max_kkt_passes = 400000
    prm.float_type = float_type
    if float_type == A.VAL_F32:
        prm.refine_reltol = 1e-8
    else:
        prm.termination_reltol = 1e-8
    xs, _, st = native.batch_solve(handle, [_struct(lp) for lp in lps], prm)
    for k, (lp, w) in enumerate(zip(lps, want)):
        assert st[k].termination_status == 0, lp.name
        obj = float(lp.c @ xs[k])
        assert abs(obj - w["objective"]) <= 1e-6 * max(1.0, abs(w["objective"])), (lp.name, obj, w)
