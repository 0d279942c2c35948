#!/usr/bin/env python3
"""Generates the golden fixtures of tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).  Three kinds, each with its source:

* known answers restated from the reference's own test suite
  (test/utils/linalg.jl:27-43 for proj_multiplier and combine;
  test/moi.jl:38-53 for the two-variable LP, optimal objective 205);
* optimal objectives from an independent solver (HiGHS through scipy's
  linprog) for seeded LPs of the single-LP, batched and multicommodity-flow
  workloads, the requests of the serving test's stream and a scaled-down
  power-law LP of the large single-LP workload: these pin the oracle and the
  device path to an answer that does not come from this repository's code;
* outputs of the CPU oracle (oracle/) on small seeded inputs: the CSR / ELL /
  COO fields of matrix conversions, the Ruiz + Pock-Chambolle diagonals, KKT
  errors at fixed points, whole solve trajectories (KKT passes, status,
  objective) and the scaled-down power-law LP solved to 1e-4 and 1e-8.  The oracle is a restatement of the reference's algorithm, not
  the reference itself (Julia is not available), so these fixtures pin
  regressions of the oracle and give the device tests bit-exact targets; they
  are not an independent check.

Everything is seeded; the fixtures are small (golden.npz + golden.json).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "coolpdlp.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def highs_objective(lp) -> float:
    from scipy.optimize import linprog
    A = lp.to_scipy().tocsr()
    eq = lp.lc == lp.uc
    le = np.isfinite(lp.uc) & ~eq
    ge = np.isfinite(lp.lc) & ~eq
    import scipy.sparse as sp
    A_ub = sp.vstack([A[le], -A[ge]]).tocsr()
    b_ub = np.concatenate([lp.uc[le], -lp.lc[ge]])
    r = linprog(lp.c, A_ub=A_ub if A_ub.shape[0] else None, b_ub=b_ub if b_ub.size else None,
                A_eq=A[eq] if eq.any() else None, b_eq=lp.uc[eq] if eq.any() else None,
                bounds=list(zip(np.where(np.isfinite(lp.lv), lp.lv, None),
                                np.where(np.isfinite(lp.uv), lp.uv, None))),
                method="highs", options={"primal_feasibility_tolerance": 1e-9,
                                         "dual_feasibility_tolerance": 1e-9})
    if r.status != 0:
        raise RuntimeError(f"HiGHS failed on {lp.name}: {r.message}")
    return float(r.fun)


def lp_sets():
    from coolpdlp import generators as G
    single = [G.random_sparse_lp(1000, 2000, 5, seed=s) for s in range(3)]
    batch = G.batch_lps(12, m_lo=50, m_hi=400, seed0=1000)
    # above the batched solver's cluster threshold (24,000 nonzeros)
    batch += [G.random_sparse_lp(2600, 5200, 5, seed=1077), G.random_sparse_lp(4000, 8000, 4, seed=1078)]
    flows = [G.multicommodity_flow_lp(side=s, K=k, seed=20 + s) for s, k in ((6, 2), (8, 3), (10, 2))]
    return {"single": single, "batch": batch, "flow": flows}


def served_requests():
    """The small served stream of tests/test_gpu_serving.py (36 requests,
    seed 11: random sparse LPs m in [60, 1500], grid flows side 6..14, K 2..4,
    tolerance 1e-4 or 1e-8)."""
    from coolpdlp import generators as G
    reqs = G.served_stream(36, 400.0, seed=11, m_lo=60, m_hi=1500, side_lo=6, side_hi=14,
                           k_lo=2, k_hi=4)
    return reqs, [G.request_lp(r) for r in reqs]


def powerlaw_small():
    """The large single LP's generator scaled down to m = 5,000, n = 10,000,
    60,000 nonzeros (power-law rows with tail 1.5 and the cap at 20,000, so
    76 rows exceed 64 nonzeros and 4 exceed 512; row factors log-U[1e-3,
    1e3]; seed 1)."""
    from coolpdlp import generators as G
    return G.powerlaw_lp(5000, 10000, 60000, seed=1, cap=20000)


def main():
    import oracle as O
    from coolpdlp import generators as G
    O.build()
    arrays = {}
    meta = {"sources": __doc__.strip().splitlines()[0]}

    # ---- known answers (reference test suite)
    meta["known"] = {
        "combine": [[1.0, 2.0, 2.0], [3.0, 3.0, 3.0], [-np.inf, 2.0, 2.0], [3.0, np.inf, 3.0],
                    [-np.inf, np.inf, 0.0]],
        "two_variable_lp_objective": 205.0,
    }

    # ---- HiGHS objectives
    sets = lp_sets()
    meta["highs"] = {}
    for kind, lps in sets.items():
        meta["highs"][kind] = [{"name": lp.name, "objective": highs_objective(lp)} for lp in lps]

    # ---- HiGHS objectives of the served requests of the serving test
    reqs, rlps = served_requests()
    meta["served"] = [{"rid": r.rid, "name": lp.name, "reltol": r.reltol,
                       "objective": highs_objective(lp)} for r, lp in zip(reqs, rlps)]

    # ---- the scaled-down large single LP: HiGHS, and the oracle (FP64 PDLP)
    # to 1e-4 and to 1e-8 relative KKT
    lpp = powerlaw_small()
    meta["powerlaw"] = {"name": lpp.name, "m": lpp.m, "n": lpp.n, "nnz": lpp.nnz,
                        "highs_objective": highs_objective(lpp)}
    for tol in (1e-4, 1e-8):
        x, y, st = O.solve(lpp, O.params(termination_reltol=tol, max_kkt_passes=2_000_000,
                                         time_limit=3600.0))
        meta["powerlaw"][f"oracle_{tol:.0e}"] = {
            "termination_status": st["termination_status"], "kkt_passes": st["kkt_passes"],
            "objective": float(np.dot(lpp.c, x)), "err": st["err"]}

    # ---- oracle: conversions of a small matrix with an empty row and column
    lp = G.random_sparse_lp(40, 60, 3, seed=5)
    ptr, idx, val = O.csr_from_csc(lp)
    d, ecol, eval_ = O.ell_from_csc(lp)
    crow, ccol, cval = O.coo_from_csc(lp)
    arrays.update({"conv_colptr": lp.colptr, "conv_rowval": lp.rowval, "conv_nzval": lp.nzval,
                   "csr_ptr": ptr, "csr_idx": idx, "csr_val": val, "ell_col": ecol,
                   "ell_val": eval_, "coo_row": crow, "coo_col": ccol, "coo_val": cval})
    meta["conv"] = {"m": lp.m, "n": lp.n, "ell_width": int(d), "name": lp.name}

    # ---- oracle: preconditioner diagonals (Ruiz 10 + Pock-Chambolle alpha 1)
    lp = G.random_sparse_lp(200, 400, 5, seed=11)
    D1, D2 = O.preconditioner(lp, 10, 1.0, True)
    arrays.update({"prec_D1": D1, "prec_D2": D2})
    meta["prec"] = {"name": lp.name, "m": 200, "n": 400, "nnz_per_col": 5, "seed": 11}

    # ---- oracle: KKT errors at a fixed point (original units)
    lpk, xk, yk = G.random_milp_and_sol(60, 120, 0.2, seed=4)
    S = O.OracleState(lpk, O.params())
    sc = S.scaled()
    e = S.kkt_of(xk / sc["D2"], yk / sc["D1"])
    S.close()
    meta["kkt"] = {"name": lpk.name, "m": 60, "n": 120, "p": 0.2, "seed": 4, "errors": e}

    # ---- oracle: solve trajectories (FP64, default PDLP and PDHG)
    meta["solves"] = []
    for lp, algo in ((G.random_sparse_lp(150, 300, 5, seed=2), "PDLP"),
                     (G.random_sparse_lp(300, 600, 4, seed=8), "PDLP"),
                     (G.random_sparse_lp(150, 300, 5, seed=2), "PDHG"),
                     (G.multicommodity_flow_lp(side=6, K=2, seed=26), "PDLP")):
        prm = O.params(1 if algo == "PDHG" else 0)
        if algo == "PDHG":
            prm.max_kkt_passes = 3000
        x, y, st = O.solve(lp, prm)
        meta["solves"].append({"name": lp.name, "algorithm": algo,
                               "termination_status": st["termination_status"],
                               "kkt_passes": st["kkt_passes"],
                               "power_iterations": st["power_iterations"],
                               "objective": float(np.dot(lp.c, x)),
                               "err": st["err"]})

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True,
                  default=lambda v: float(v) if isinstance(v, np.floating) else int(v))
    print("wrote", os.path.join(HERE, "golden.npz"), "and golden.json")


if __name__ == "__main__":
    main()
