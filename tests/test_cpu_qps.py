"""MPS reading for MILP(qps) (src/problems/milp.jl:117-136).  The LPs here are
written for these tests; the rules checked are the MPS format's (ROWS types,
RHS on the objective row, RANGES, BOUNDS types, MARKER blocks, free and fixed
columns)."""
import math

import numpy as np
import pytest

FREE = """\
* a small LP exercising every section
NAME          TESTLP
OBJSENSE
    MAX
ROWS
 N  COST
 E  R1
 L  R2
 G  R3
 E  R4
 N  FREEROW
 G  R5
COLUMNS
    X1        COST      1.5        R1        2.0
    X1        R2        -1.0       FREEROW   9.0
    MARKER    'MARKER'  'INTORG'
    X2        COST      -3.0       R2        1.0
    X2        R3        4.0
    MARKER    'MARKER'  'INTEND'
    X3        R1        1.0        R4        -2.5
    X3        R5        1.0
    X4        COST      2.0        R3        1.0
    X5        R4        1.0
    X6        R5        3.0
    X7        COST      1.0
RHS
    RHS       COST      -7.25      R1        3.0
    RHS       R2        4.0        R3        1.0
    RHS       R4        2.0        R5        -1.0
RANGES
    RNG       R1        2.0        R2        1.5
    RNG       R3        0.5        R4        -1.0
BOUNDS
 UP BND       X1        4.0
 LO BND       X2        -1.0
 UI BND       X2        8
 FX BND       X3        1.25
 FR BND       X4
 MI BND       X5
 BV BND       X6
 UP BND       X7        -2.0
ENDATA
"""


def _expect():
    inf = math.inf
    return dict(
        c=np.array([1.5, -3.0, 0.0, 2.0, 0.0, 0.0, 1.0]),
        c0=7.25,
        lcon=np.array([3.0, 2.5, 1.0, 1.0, -1.0]),
        ucon=np.array([5.0, 4.0, 1.5, 2.0, inf]),
        lvar=np.array([0.0, -1.0, 1.25, -inf, -inf, 0.0, -inf]),
        uvar=np.array([4.0, 8.0, 1.25, inf, inf, 1.0, -2.0]),
        vartypes=[0, 1, 0, 0, 0, 2, 0],
        A=np.array([[2.0, 0, 1.0, 0, 0, 0, 0],
                    [-1.0, 1.0, 0, 0, 0, 0, 0],
                    [0, 4.0, 0, 1.0, 0, 0, 0],
                    [0, 0, -2.5, 0, 1.0, 0, 0],
                    [0, 0, 1.0, 0, 0, 3.0, 0]]))


def _check(q):
    import coolpdlp as cp
    from coolpdlp.qps import VTYPE_Binary, VTYPE_Integer
    e = _expect()
    assert q.name == "TESTLP" and q.objname == "COST" and q.objsense == "MAX"
    assert q.c0 == e["c0"]
    for k in ("c", "lcon", "ucon", "lvar", "uvar"):
        assert np.array_equal(getattr(q, k), e[k]), k
    assert list(q.vartypes) == e["vartypes"]
    assert q.varnames == [f"X{i}" for i in range(1, 8)]
    assert q.connames == ["R1", "R2", "R3", "R4", "R5"]
    milp = cp.MILP.from_qps(q)
    assert np.array_equal(milp.A.to_scipy().toarray(), e["A"])
    assert np.array_equal(milp.int_var, [False, True, False, False, False, True, False])
    assert milp.var_names == q.varnames and milp.name == "TESTLP"
    assert np.array_equal(milp.At.to_scipy().toarray(), e["A"].T)


def test_readqps_free():
    from coolpdlp.qps import readqps
    _check(readqps(FREE, mpsformat="free"))


def _to_fixed(text):
    """The same file in fixed columns (fields at 2-3, 5-12, 15-22, 25-36, 40-47, 50-61)."""
    out = []
    section = None
    for line in text.splitlines():
        if not line.strip() or line.startswith("*"):
            out.append(line)
            continue
        if not line[0].isspace():
            section = line.split()[0]
            out.append(line)
            continue
        f = line.split()
        if section == "COLUMNS" and "'MARKER'" in line:
            out.append(line)
            continue
        if section in ("ROWS", "BOUNDS"):
            fl = f if section == "BOUNDS" else [f[0], f[1]]
            if section == "BOUNDS" and len(f) == 3 and f[0] in ("FR", "MI", "PL", "BV"):
                fl = f
        else:
            fl = [""] + f
        cols = [(1, 3), (4, 12), (14, 22), (24, 36), (39, 47), (49, 61)]
        buf = [" "] * 61
        for (a, b), v in zip(cols, fl):
            for i, ch in enumerate(v):
                buf[a + i] = ch
        out.append("".join(buf).rstrip())
    return "\n".join(out) + "\n"


def test_readqps_fixed_matches_free():
    from coolpdlp.qps import readqps
    fixed = _to_fixed(FREE)
    _check(readqps(fixed, mpsformat="fixed"))


def _write_mps(lp, name="RT"):
    def r(v):
        return repr(float(v))

    lines = [f"NAME {name}", "ROWS", " N OBJ"]
    for i in range(lp.m):
        t = "E" if lp.lc[i] == lp.uc[i] else ("L" if math.isinf(lp.lc[i]) else "G")
        lines.append(f" {t} C{i + 1}")
    lines.append("COLUMNS")
    for j in range(lp.n):
        lines.append(f" V{j + 1} OBJ {r(lp.c[j])}")
        for k in range(lp.colptr[j] - 1, lp.colptr[j + 1] - 1):
            lines.append(f" V{j + 1} C{lp.rowval[k]} {r(lp.nzval[k])}")
    lines.append("RHS")
    for i in range(lp.m):
        b = lp.lc[i] if not math.isinf(lp.lc[i]) else lp.uc[i]
        lines.append(f" RHS C{i + 1} {r(b)}")
    lines.append("RANGES")
    for i in range(lp.m):
        if not math.isinf(lp.lc[i]) and not math.isinf(lp.uc[i]) and lp.lc[i] != lp.uc[i]:
            lines.append(f" RNG C{i + 1} {r(lp.uc[i] - lp.lc[i])}")
    lines.append("BOUNDS")
    for j in range(lp.n):
        lo, up = lp.lv[j], lp.uv[j]
        if math.isinf(lo) and math.isinf(up):
            lines.append(f" FR BND V{j + 1}")
            continue
        if math.isinf(lo):
            lines.append(f" MI BND V{j + 1}")
        elif lo != 0.0:
            lines.append(f" LO BND V{j + 1} {r(lo)}")
        if not math.isinf(up):
            lines.append(f" UP BND V{j + 1} {r(up)}")
    lines.append("ENDATA")
    return "\n".join(lines) + "\n"


def test_mps_round_trip_bit_exact():
    import coolpdlp as cp
    from coolpdlp import generators as G
    from coolpdlp.qps import readqps
    for lp in (G.random_sparse_lp(40, 80, 5, seed=11), G.multicommodity_flow_lp(side=4, K=2, seed=5)):
        milp = cp.MILP.from_qps(readqps(_write_mps(lp), mpsformat="free"))
        assert np.array_equal(milp.A.colptr, lp.colptr)
        assert np.array_equal(milp.A.rowval, lp.rowval)
        assert np.array_equal(milp.A.nzval, lp.nzval)
        for k in ("c", "lv", "uv", "lc", "uc"):
            assert np.array_equal(getattr(milp, k), getattr(lp, k)), k


def test_readqps_errors():
    from coolpdlp import _abi as A
    from coolpdlp.qps import readqps
    with pytest.raises(A.ArgumentError):
        readqps("ROWS\n N OBJ\nCOLUMNS\n X1 NOPE 1.0\nENDATA\n", mpsformat="free")
    with pytest.raises(A.ArgumentError):
        readqps("ROWS\n Q R1\nENDATA\n", mpsformat="free")
    with pytest.raises(A.ArgumentError):
        readqps("ROWS\n N OBJ\nCOLUMNS\n X1 OBJ abc\nENDATA\n", mpsformat="free")
