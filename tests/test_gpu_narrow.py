"""Narrow +-1 matrix storage (the signs in the column indices, no value array).

Index arrays and values must read back bit-identical to the Float32 CSR of the
same matrix, and mul! must be bit-identical to it (products with +-1 are
exact and the rows are summed in the same order).  A single-LP solve with
Float32 iterates stores a +-1 matrix narrow by default; it must reach the
same status and objective as the valued storage and as HiGHS (golden
objectives of the multicommodity flow LPs)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.json")


def _sign_mats():
    """+-1 matrices: random patterns (incl. empty rows/columns, long rows
    that take the split path) and the flow LPs' incidence matrices."""
    from coolpdlp import generators as G
    st = G.Stream(11, 0)
    mats = []
    for (m, n, dens) in ((1, 1, 1.0), (10, 20, 0.2), (30, 10, 0.3), (200, 400, 0.02),
                         (40, 3000, 0.4), (3, 30000, 0.9)):
        mask = st.uniform(m * n) < dens
        flat = np.nonzero(mask)[0]
        cols, rows = flat // m, flat % m
        vals = np.where(st.uniform(flat.size) < 0.5, -1.0, 1.0)
        mats.append(G.csc_from_triplets(m, n, rows, cols, vals) + (m, n))
    lp = G.multicommodity_flow_lp(side=8, K=3, seed=2)
    mats.append((lp.colptr, lp.rowval, lp.nzval, lp.m, lp.n))
    return mats


def test_pm1_csr_export_and_mul_bit_exact(handle):
    import torch
    import coolpdlp as cp
    from coolpdlp import generators as G
    st = G.Stream(5, 3)
    for k, (colptr, rowval, nzval, m, n) in enumerate(_sign_mats()):
        C = cp.CSCMatrix(m, n, colptr, rowval, nzval)
        N = cp.GPUSparseMatrixCSR(C, dtype=np.float32, narrow=True, handle=handle)
        V = cp.GPUSparseMatrixCSR(C, dtype=np.float32, handle=handle)
        assert N.shape == (m, n) and N.nnz() == V.nnz() == nzval.size
        for a, b in zip(N.export(), V.export()):
            assert np.array_equal(a, b), k
        b = torch.tensor(st.normal(n).astype(np.float32), device="cuda")
        c0 = st.normal(m).astype(np.float32)
        for (al, be) in ((1.0, 0.0), (0.7310585786300049, 0.2689414213699951)):
            cn = torch.tensor(c0, device="cuda")
            cv = torch.tensor(c0, device="cuda")
            N.mul(cn, b, al, be)
            V.mul(cv, b, al, be)
            assert torch.equal(cn, cv), (k, al, be)
        N.close()
        V.close()


def test_pm1_argument_checks(handle):
    import coolpdlp as cp
    from coolpdlp import _abi as A
    C = cp.CSCMatrix(2, 2, np.array([1, 2, 3]), np.array([1, 2]), np.array([1.0, 0.5]))
    with pytest.raises(A.ArgumentError):
        cp.GPUSparseMatrixCSR(C, dtype=np.float32, narrow=True, handle=handle)
    with pytest.raises(A.ArgumentError):
        cp.GPUSparseMatrixCSR(C, dtype=np.float64, narrow=True, handle=handle)
    C1 = cp.CSCMatrix(2, 2, np.array([1, 2, 3]), np.array([1, 2]), np.array([1.0, -1.0]))
    with pytest.raises(A.CpdlpError) as e:
        cp.GPUSparseMatrixELL(C1, dtype=np.float32, narrow=True, handle=handle)
    assert e.value.code == A.ERR_UNSUPPORTED


def _flow_golden():
    from coolpdlp import generators as G
    with open(GOLDEN) as f:
        g = json.load(f)
    out = []
    for rec in g["highs"]["flow"]:
        args = rec["name"][rec["name"].index("(") + 1:-1]
        kw = {k: int(v) for k, v in (a.split("=") for a in args.split(","))}
        out.append((G.multicommodity_flow_lp(**kw), rec["objective"]))
    return out


def _params(narrow: bool, **kw):
    from coolpdlp import _abi as A
    p = A.default_params_py()
    p.float_type = A.VAL_F32
    p.tile_flags = 0 if narrow else A.TILE_NO_NARROW
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_narrow_storage_is_used_and_steps_agree(handle):
    """The narrow problem reads 4 bytes per nonzero (kernel_bytes) and its
    iterates follow the valued storage's to FP32 rounding."""
    from coolpdlp import native
    from coolpdlp import generators as G
    lp = G.multicommodity_flow_lp(side=8, K=3, seed=2)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    res = {}
    for narrow in (True, False):
        prm = _params(narrow)
        P = native.Problem(handle, L, prm)
        S = native.State(P, prm)
        res[narrow] = (S.kernel_bytes(), S)
        S.step(100)
        res[narrow] = res[narrow] + (S.vectors(),)
    bn, bv = res[True][0], res[False][0]
    assert bv[0] - bn[0] == pytest.approx(4.0 * lp.nnz - 4.0 * lp.n)
    assert bv[1] - bn[1] == pytest.approx(4.0 * lp.nnz - 8.0 * lp.m)
    (xn, yn), (xv, yv) = res[True][2], res[False][2]
    for a, b in ((xn, xv), (yn, yv)):
        assert np.max(np.abs(a - b)) <= 1e-4 * max(1.0, np.max(np.abs(b)))


def test_narrow_power_method_matches_valued(handle):
    from coolpdlp import native
    from coolpdlp import generators as G
    lp = G.multicommodity_flow_lp(side=10, K=2, seed=30)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    out = {}
    for narrow in (True, False):
        prm = _params(narrow, power_maxiter_override=30)
        P = native.Problem(handle, L, prm)
        out[narrow] = P.spectral_norm(prm)
    (sn, itn), (sv, itv) = out[True], out[False]
    assert abs(sn - sv) <= 1e-5 * sv, (sn, sv)
    assert abs(itn - itv) <= 2


@pytest.mark.parametrize("refine", [False, True])
def test_narrow_flow_solves_match_highs(handle, refine):
    """FP32 iterates on the narrow matrix to 1e-4 (objective within the
    reference's rtol 1e-2 of HiGHS, and of the valued storage's), and with
    FP64 refinement to 1e-8 (objective within 1e-6 relative of HiGHS)."""
    from coolpdlp import native
    for lp, obj in _flow_golden():
        L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                            lp.lc, lp.uc)
        got = {}
        for narrow in ((True, False) if not refine else (True,)):
            prm = _params(narrow, max_kkt_passes=400000,
                          refine_reltol=1e-8 if refine else 0.0)
            x, y, s = native.solve_lp(handle, L, prm)
            assert s.termination_status == 0, (lp.m, narrow, s.termination_status)
            got[narrow] = float(lp.c @ x)
        tol = 1e-6 if refine else 1e-2
        for narrow, o in got.items():
            assert abs(o - obj) <= tol * max(1.0, abs(obj)), (narrow, o, obj)
        if not refine:
            assert abs(got[True] - got[False]) <= 1e-2 * max(1.0, abs(obj))


def test_unknown_tile_flags_rejected(handle):
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    lp = G.two_variable_lp()
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    p = _params(True)
    p.tile_flags = 8
    with pytest.raises(A.ArgumentError):
        native.solve_lp(handle, L, p)
    # the density order forced both on and off
    p.tile_flags = A.TILE_DENSITY_ORDER | A.TILE_NO_DENSITY_ORDER
    with pytest.raises(A.ArgumentError):
        native.solve_lp(handle, L, p)
