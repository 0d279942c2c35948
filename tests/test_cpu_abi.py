"""CPU tests of the C ABI boundary: the library builds and loads without a
GPU, exports every function include/coolpdlp_cuda.h declares, the ctypes
structs match the header's layout, and the host-side API mirrors the
reference's constructors and checks (no GPU computation here)."""
import ctypes
import os
import re

import numpy as np
import pytest


def _header_functions():
    from coolpdlp import _abi
    text = open(_abi.HEADER_PATH).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(cpdlp_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_function(cuda_lib):
    from coolpdlp import _abi
    declared = _header_functions()
    assert len(declared) >= 30, declared
    for name in declared:
        assert hasattr(cuda_lib, name), name
    assert set(declared) == set(_abi.EXPORTED_SYMBOLS), set(declared) ^ set(_abi.EXPORTED_SYMBOLS)
    assert cuda_lib.cpdlp_abi_version() == 1


def test_params_default_matches_reference_defaults(cuda_lib):
    """Algorithm{A} defaults (common.jl:53-116) and PDHG overrides (pdhg.jl:6-16)."""
    from coolpdlp import _abi as A
    for algo in (A.ALGO_PDLP, A.ALGO_PDHG):
        p = A.ParamsC()
        cuda_lib.cpdlp_params_default(ctypes.byref(p), algo)
        q = A.default_params_py(algo)
        for f, _ in A.ParamsC._fields_:
            a, b = getattr(p, f), getattr(q, f)
            assert (a == b) or (isinstance(a, float) and np.isnan(a) and np.isnan(b)), f
    p = A.default_params_py(A.ALGO_PDLP)
    assert (p.ruiz_iter, p.check_every, p.max_kkt_passes) == (10, 100, 100000)
    assert (p.termination_reltol, p.time_limit, p.invnorm_scaling) == (1e-4, 100.0, 0.9)


def test_struct_sizes_match_header():
    """Field-by-field sizes of the structs (8-byte aligned layout)."""
    from coolpdlp import _abi as A
    assert ctypes.sizeof(A.KKTErrorsC) == 48
    assert ctypes.sizeof(A.LPC) == 11 * 8
    assert ctypes.sizeof(A.ParamsC) % 8 == 0 and ctypes.sizeof(A.StatsC) % 8 == 0


def test_create_without_gpu_fails_cleanly(cuda_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = cuda_lib.cpdlp_create(0, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_milp_checks_mirror_reference():
    """test/problems/milp.jl 'Checks': DimensionMismatch / ArgumentError."""
    import coolpdlp as cp
    from coolpdlp import generators as G
    lp, _, _ = G.random_milp_and_sol(20, 40, 0.3, seed=1)
    kw = dict(c=lp.c, lv=lp.lv, uv=lp.uv, A=lp.to_scipy(), lc=lp.lc, uc=lp.uc)
    cp.MILP(**kw)
    with pytest.raises(cp.ArgumentError):
        cp.MILP(**{**kw, "c": np.array(list(lp.c), dtype=object)})
    for bad in ({"c": lp.lc}, {"lv": lp.lc}, {"lc": lp.lv}, {"D1": np.ones(lp.n)},
                {"int_var": np.zeros(lp.n + 1, dtype=bool)}):
        with pytest.raises(cp.DimensionMismatch):
            cp.MILP(**{**kw, **bad})
    with pytest.raises(cp.DimensionMismatch):
        cp.MILP(**{**kw, "A": lp.to_scipy().T})
    m = cp.MILP(**kw)
    assert cp.nbvar(m) == 40 and cp.nbcons(m) == 20
    assert cp.nbcons_eq(m) + cp.nbcons_ineq(m) == 20


def test_is_feasible_and_objective_known_answers():
    """test/problems/solution.jl 'Cube MILP'."""
    import warnings
    import coolpdlp as cp
    milp = cp.MILP(c=[1.0, 2.0], lv=np.zeros(2), uv=2 * np.ones(2), A=np.array([[1.0, 1.0]]),
                   lc=[1.0], uc=[1.0], int_var=[True, False])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert cp.is_feasible([1.0, 0.0], milp)
        assert not cp.is_feasible([0.5, 0.5], milp)
        assert not cp.is_feasible([0.0, 0.0], milp)
        assert not cp.is_feasible([2.0, -1.0], milp)
    assert cp.objective_value([1.0, 1.0], milp) == 3


def test_algorithm_keywords():
    import coolpdlp as cp
    a = cp.PDLP(np.float32, termination_reltol=1e-6, time_limit=10.0)
    assert a.params.float_type == 1 and a.params.termination_reltol == 1e-6
    b = cp.PDHG()
    assert b.params.ruiz_iter == 0 and np.isnan(b.params.sufficient_decay)
    with pytest.raises(TypeError):
        cp.PDLP(not_a_keyword=1)
