"""MPS / QPS reading for MILP(qps) (src/problems/milp.jl:117-136).

The reference reads files with QPSReader.jl 0.2.1 (``readqps``) and builds a
MILP from the QPSData fields c, lvar, uvar, (arows, acols, avals), lcon, ucon,
vartypes and varnames.  That package is not part of this tree; this module
restates the MPS rules those fields follow:

* ROWS: the first N row is the objective (later N rows are free rows and are
  dropped); E rows get lcon = ucon = rhs, L rows (-Inf, rhs], G rows
  [rhs, +Inf); the right-hand side defaults to 0.
* COLUMNS: ``col row value [row value]``; MARKER lines with 'INTORG' /
  'INTEND' bracket integer columns.  An entry on the objective row is c[col].
* RHS: an entry on the objective row sets the constant c0 = -value.
* RANGES (R on row r with rhs b): E rows become [b, b+|R|] for R > 0 and
  [b-|R|, b] for R < 0; L rows [b-|R|, b]; G rows [b, b+|R|].
* BOUNDS (default [0, +Inf]): UP, LO, FX, FR, MI, PL, BV ([0, 1], binary),
  LI / UI (integer lower / upper).  An UP bound below 0 on a column whose
  lower bound is still 0 moves the lower bound to -Inf.
* QUADOBJ / QMATRIX entries are read into (qrows, qcols, qvals) and are not
  used by MILP(qps), which is an LP.
* OBJSENSE is read (``objsense``); MILP(qps) ignores it, as the reference does.

``mpsformat="free"`` splits lines on whitespace; ``"fixed"`` reads the classic
columns (fields at 2-3, 5-12, 15-22, 25-36, 40-47, 50-61), which allows
spaces inside names.
"""
from __future__ import annotations

import dataclasses
import io
import math
import os

import numpy as np

from ._abi import ArgumentError
from . import _abi as A

VTYPE_Continuous, VTYPE_Integer, VTYPE_Binary = 0, 1, 2


@dataclasses.dataclass
class QPSData:
    name: str = ""
    objname: str = ""
    objsense: str = "MIN"
    c0: float = 0.0
    c: np.ndarray = None
    qrows: np.ndarray = None
    qcols: np.ndarray = None
    qvals: np.ndarray = None
    arows: np.ndarray = None   # 1-based
    acols: np.ndarray = None   # 1-based
    avals: np.ndarray = None
    lcon: np.ndarray = None
    ucon: np.ndarray = None
    lvar: np.ndarray = None
    uvar: np.ndarray = None
    vartypes: list = None
    varnames: list = None
    connames: list = None

    @property
    def nvar(self) -> int:
        return len(self.varnames)

    @property
    def ncon(self) -> int:
        return len(self.connames)


_FIXED = ((1, 3), (4, 12), (14, 22), (24, 36), (39, 47), (49, 61))


def _fields(line: str, fmt: str):
    if fmt == "free":
        return line.split()
    out = []
    for a, b in _FIXED:
        if a >= len(line):
            break
        f = line[a:b].strip()
        out.append(f)
    while out and out[-1] == "":
        out.pop()
    return out


def _num(s: str, where: str) -> float:
    try:
        return float(s.replace("D", "E").replace("d", "e"))
    except ValueError:
        raise ArgumentError(A.ERR_ARGUMENT, f"MPS: bad number {s!r} in {where}") from None


def readqps(source, mpsformat: str = "fixed") -> QPSData:
    """Reads an MPS/QPS file (path, text or file object) into QPSData."""
    if mpsformat not in ("fixed", "free"):
        raise ArgumentError(A.ERR_ARGUMENT, "mpsformat must be 'fixed' or 'free'")
    if hasattr(source, "read"):
        text = source.read()
    elif isinstance(source, str) and "\n" not in source and os.path.exists(source):
        with open(source) as f:
            text = f.read()
    else:
        text = str(source)
    q = QPSData()
    objrow = None
    rowtype, rowidx, connames = {}, {}, []
    colidx, varnames, vartypes = {}, [], []
    cvals, ents, qents = {}, [], []
    rhs, rng = {}, {}
    bounds = []
    integer_block = False
    section = None
    for raw in io.StringIO(text):
        line = raw.rstrip("\n").rstrip("\r")
        if not line.strip() or line.lstrip().startswith("*"):
            continue
        if not line[0].isspace():
            head = line.split()
            section = head[0].upper()
            if section == "NAME":
                q.name = line[4:].strip() if mpsformat == "fixed" else " ".join(head[1:])
            elif section == "OBJSENSE" and len(head) > 1:
                q.objsense = "MAX" if head[1].upper().startswith("MAX") else "MIN"
            elif section == "ENDATA":
                break
            elif section not in ("ROWS", "COLUMNS", "RHS", "RANGES", "BOUNDS", "QUADOBJ",
                                 "QMATRIX", "OBJSENSE"):
                raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown section {section}")
            continue
        if section == "COLUMNS" and "'MARKER'" in line.upper():
            tok = [t.strip("'\"").upper() for t in line.split()]
            if "INTORG" in tok:
                integer_block = True
            elif "INTEND" in tok:
                integer_block = False
            continue
        f = _fields(line, mpsformat)
        if mpsformat == "fixed" and section in ("COLUMNS", "RHS", "RANGES", "QUADOBJ",
                                                "QMATRIX") and f and f[0] == "":
            f = f[1:]  # field 1 is blank in these sections
        if not f:
            continue
        if section == "OBJSENSE":
            q.objsense = "MAX" if line.split()[0].upper().startswith("MAX") else "MIN"
        elif section == "ROWS":
            t, nm = f[0].upper(), f[1]
            if t == "N":
                if objrow is None:
                    objrow = nm
                    q.objname = nm
                rowtype[nm] = "N"
                continue
            if t not in ("E", "L", "G"):
                raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown row type {t}")
            rowtype[nm] = t
            rowidx[nm] = len(connames)
            connames.append(nm)
        elif section == "COLUMNS":
            col = f[0]
            if col not in colidx:
                colidx[col] = len(varnames)
                varnames.append(col)
                vartypes.append(VTYPE_Integer if integer_block else VTYPE_Continuous)
            j = colidx[col]
            for k in range(1, len(f) - 1, 2):
                rn, v = f[k], _num(f[k + 1], f"COLUMNS {col}")
                if rn == objrow:
                    cvals[j] = cvals.get(j, 0.0) + v
                elif rn in rowidx:
                    ents.append((rowidx[rn] + 1, j + 1, v))
                elif rowtype.get(rn) == "N":
                    continue  # a free row beyond the objective
                else:
                    raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown row {rn} in COLUMNS")
        elif section in ("RHS", "RANGES"):
            # the set name may be absent in free format (odd number of fields)
            items = f[1:] if len(f) % 2 == 1 else f
            for k in range(0, len(items) - 1, 2):
                rn, v = items[k], _num(items[k + 1], section)
                if section == "RHS" and rn == objrow:
                    q.c0 = -v
                elif rn in rowidx:
                    (rhs if section == "RHS" else rng)[rn] = v
                elif rowtype.get(rn) == "N":
                    continue
                else:
                    raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown row {rn} in {section}")
        elif section == "BOUNDS":
            t = f[0].upper()
            if t in ("FR", "MI", "PL", "BV"):
                col = f[2] if len(f) >= 3 else f[1]
                val = _num(f[3], "BOUNDS") if len(f) >= 4 else None
            else:
                if len(f) >= 4:
                    col, val = f[2], _num(f[3], "BOUNDS")
                elif len(f) == 3:
                    col, val = f[1], _num(f[2], "BOUNDS")
                else:
                    raise ArgumentError(A.ERR_ARGUMENT, f"MPS: short BOUNDS line {line!r}")
            bounds.append((t, col, val))
        elif section in ("QUADOBJ", "QMATRIX"):
            qents.append((f[0], f[1], _num(f[2], section)))
    n, m = len(varnames), len(connames)
    q.varnames, q.connames, q.vartypes = varnames, connames, vartypes
    q.c = np.zeros(n)
    for j, v in cvals.items():
        q.c[j] = v
    q.lvar = np.zeros(n)
    q.uvar = np.full(n, math.inf)
    for t, col, val in bounds:
        if col not in colidx:
            raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown column {col} in BOUNDS")
        j = colidx[col]
        if t == "UP" or t == "UI":
            q.uvar[j] = val
            if val < 0 and q.lvar[j] == 0.0:
                q.lvar[j] = -math.inf
            if t == "UI":
                q.vartypes[j] = VTYPE_Integer
        elif t == "LO" or t == "LI":
            q.lvar[j] = val
            if t == "LI":
                q.vartypes[j] = VTYPE_Integer
        elif t == "FX":
            q.lvar[j] = q.uvar[j] = val
        elif t == "FR":
            q.lvar[j], q.uvar[j] = -math.inf, math.inf
        elif t == "MI":
            q.lvar[j] = -math.inf
        elif t == "PL":
            q.uvar[j] = math.inf
        elif t == "BV":
            q.lvar[j], q.uvar[j] = 0.0, 1.0
            q.vartypes[j] = VTYPE_Binary
        else:
            raise ArgumentError(A.ERR_ARGUMENT, f"MPS: unknown bound type {t}")
    q.lcon = np.zeros(m)
    q.ucon = np.zeros(m)
    for nm, i in rowidx.items():
        b = rhs.get(nm, 0.0)
        t = rowtype[nm]
        lo, up = {"E": (b, b), "L": (-math.inf, b), "G": (b, math.inf)}[t]
        if nm in rng:
            r = rng[nm]
            if t == "E":
                lo, up = (b, b + abs(r)) if r > 0 else (b - abs(r), b)
            elif t == "L":
                lo = b - abs(r)
            else:
                up = b + abs(r)
        q.lcon[i], q.ucon[i] = lo, up
    if ents:
        e = np.array(ents, dtype=np.float64)
        q.arows, q.acols, q.avals = e[:, 0].astype(np.int64), e[:, 1].astype(np.int64), e[:, 2]
    else:
        q.arows = np.zeros(0, dtype=np.int64)
        q.acols = np.zeros(0, dtype=np.int64)
        q.avals = np.zeros(0)
    if qents:
        q.qrows = np.array([colidx[a] + 1 for a, _, _ in qents], dtype=np.int64)
        q.qcols = np.array([colidx[b] + 1 for _, b, _ in qents], dtype=np.int64)
        q.qvals = np.array([v for _, _, v in qents])
    else:
        q.qrows = np.zeros(0, dtype=np.int64)
        q.qcols = np.zeros(0, dtype=np.int64)
        q.qvals = np.zeros(0)
    return q
