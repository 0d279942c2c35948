#!/usr/bin/env python3
"""PDLP throughput on one GB300 (libcoolpdlp_cuda).

Workload: the large single LP -- m = 2,000,000 rows, n = 4,000,000 columns,
~24M nonzeros with power-law row lengths (tail 1.5, capped at 20,000), row
factors log-uniform in [1e-3, 1e3], seed 1 -- solved by PDLP with FP32
iterates and FP64 KKT reductions.  Seeded synthetic input (the reference
publishes no benchmark data).

A "step" is one block of solve!: check_every = 100 PDLP iterations plus one
termination/restart check (four-iterate KKT pass).  `value` = iterations/s
with the LP resident in HBM, timed with CUDA events on the library's stream;
`e2e` = iterations/s through cpdlp_solve with the LP in pinned host memory
(upload, scaling, power method, 1,000 iterations, download all inside the
timed region).  The working set (~0.6 GB per iteration) is larger than L2,
so no flush is needed between steps.

The same JSON line also carries `flow` (the 256x256 grid multicommodity flow
LP with K=16: FP32 iterations/s with the narrow +-1 storage and with scaled
values, and solves to 1e-4 and, with refinement rounds, to 1e-8), `batch`
(4,096 random LPs in persistent launches against the one-at-a-time FP64
path) and `serving` (a Poisson stream through the continuous-batching
server, p50/p99, then the same requests arriving at once for throughput).

--impl reference times the CPU restatement of the reference algorithm
(oracle/, Float64, all host threads) on the same LP.
Under torchrun with N ranks every rank solves its own copy (one LP does not
shard): value = all ranks' iterations / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "coolpdlp.jl_gb300"))

METRIC = "PDHG iters/s (HBM GB/s) and LPs/s to 1e-4 rel KKT; p50/p99 solve latency"
UNIT = "iters/s"
CHECK_EVERY = 100
E2E_ITERS = 1000


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink the workload (testing only; 1.0 = the named workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--batch-lps", type=int, default=4096,
                    help="LPs of the batched workload (0 skips the batch measurement)")
    ap.add_argument("--sequential-sample", type=int, default=32,
                    help="LPs of the batch solved one at a time by the FP64 path")
    ap.add_argument("--serve-requests", type=int, default=160,
                    help="requests of the served stream (0 skips the serving measurement)")
    ap.add_argument("--serve-rates", type=str, default="8,16,32",
                    help="Poisson arrival rates per second, comma separated")
    ap.add_argument("--c1-solves", type=int, default=1,
                    help="1: solve the large LP to 1e-4 and (refined) to 1e-8 in the line")
    ap.add_argument("--c1-time-limit", type=float, default=120.0,
                    help="time limit in seconds of the large-LP solve to 1e-4")
    ap.add_argument("--c1-refine-time-limit", type=float, default=90.0,
                    help="time limit in seconds of the large-LP solve to 1e-8")
    ap.add_argument("--batch-m-hi", type=int, default=5000,
                    help="largest m of the batched LPs (5000 = the named workload)")
    ap.add_argument("--flow-side", type=int, default=256,
                    help="grid side of the multicommodity flow LP (0 skips the flow section)")
    ap.add_argument("--flow-k", type=int, default=16, help="commodities of the flow LP")
    ap.add_argument("--flow-no-solve", action="store_true",
                    help="flow section without the solves to 1e-4 / 1e-8")
    ap.add_argument("--only-flow", action="store_true",
                    help="run only the flow measurement (profiling); no headline value")
    ap.add_argument("--matrix-type", choices=["auto", "csr", "ell"], default="auto",
                    help="product format of the large LP and the flow LP (profiling; auto = the autotuner)")
    ap.add_argument("--tile-nnz", type=int, default=0,
                    help="CSR tile size of the large LP and the flow LP (profiling; 0 = autotuned)")
    ap.add_argument("--density-order", choices=["auto", "on", "off"], default="auto",
                    help="density order of the large LP and the flow LP (profiling; auto = the autotuner)")
    ap.add_argument("--only-serving-stream", type=int, default=0,
                    help="run only a long served stream of this many requests at the first "
                         "rate of --serve-rates (FP32+FP64-refined); no headline value")
    ap.add_argument("--only-batch", action="store_true",
                    help="run only the batched measurement (profiling small cases)")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(scale: float):
    from coolpdlp import generators as G
    m = int(2_000_000 * scale)
    n = 2 * m
    nnz = int(24_000_000 * scale)
    return G.powerlaw_lp(m, n, nnz, seed=1, cap=min(20000, n))


def workload_config(lp, scale):
    return {
        "workload": (f"power-law single LP m={lp.m:,} n={lp.n:,} nnz={lp.nnz:,} "
                     "(row lengths tail 1.5 capped at 20,000; row factors log-U[1e-3,1e3]; seed 1)"),
        "algorithm": "PDLP", "iterates": "FP32", "kkt_reductions": "FP64",
        "step": f"{CHECK_EVERY} PDLP iterations + one termination/restart check",
        "l2": "inputs larger than L2 (~0.6 GB moved per iteration), no flush",
        "scale": scale,
    }


def load_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def rel_kkt(st) -> float:
    e = st.err
    return max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)


def fp64_reference(h, lp, reltol: float = 1e-8, time_limit: float = 60.0):
    """The plain FP64 path (cpdlp_solve, Float64 iterates) to `reltol`: the
    FP64 reference objective that every reported result is compared with."""
    from coolpdlp import native
    p = native.default_params()
    p.termination_reltol = reltol
    p.max_kkt_passes = 1 << 40
    p.time_limit = time_limit
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    x, _, st = native.solve_lp(h, L, p)
    return float(lp.c @ x), st


def obj_err(obj: float, ref: float) -> float:
    return abs(obj - ref) / max(1.0, abs(ref))


def err_summary(errs) -> dict:
    import numpy as np
    a = np.asarray(errs, dtype=float)
    return {"max": float(a.max()), "median": float(np.median(a)), "count": int(a.size)}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(lp, budget_s: float = 16.0, single_core_s: float = 6.0, c0=None) -> dict:
    """The oracle (CPU restatement, FP64) on the same LP: preprocessing
    untimed, then 10-iteration steps until ~budget_s on all host threads
    (OpenMP row loops), and a sample on 1 thread (the reference's CPU path is
    single-threaded).  With `c0` (the GPU's FP64 C0 result), the C0 LP is also
    solved by the oracle on 1 thread: iterations/s and parity (status, KKT
    passes, objective)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    cores = int(O.lib().orc_num_threads())
    prm = O.params(termination_reltol=0.0, max_kkt_passes=1 << 60, time_limit=1e30)
    t0 = time.perf_counter()
    S = O.OracleState(lp, prm)
    t_setup = time.perf_counter() - t0

    def sample(limit_s, max_iters):
        iters, t = 0, 0.0
        while t < limit_s and iters < max_iters:
            a = time.perf_counter()
            S.step(10)
            t += time.perf_counter() - a
            iters += 10
        return iters, t

    iters, t = sample(budget_s, 100 * 50)
    O.lib().orc_set_num_threads(1)
    it1, t1 = sample(single_core_s, 100 * 50)
    O.lib().orc_set_num_threads(cores)
    S.close()
    out = {"value": iters / t, "unit": UNIT, "cores": cores, "kind": "port",
           "precision": "FP64",
           "sample": (f"{iters} PDLP iterations (FP64) of the same LP after "
                      f"{t_setup:.1f} s of untimed preprocessing"), "seconds": t,
           "single_core": {"value": it1 / t1, "unit": UNIT, "cores": 1,
                           "sample": f"{it1} PDLP iterations (FP64) of the same LP"}}
    if c0 is not None:
        from coolpdlp import generators as G
        lp0 = G.random_sparse_lp(1000, 2000, 5, seed=0)
        O.lib().orc_set_num_threads(1)
        a = time.perf_counter()
        xo, _, so = O.solve(lp0, O.params())
        dt = time.perf_counter() - a
        O.lib().orc_set_num_threads(cores)
        obj = float(lp0.c @ xo)
        out["c0"] = {"iters_per_s": so["kkt_passes"] / dt, "cores": 1,
                     "termination_status": so["termination_status"],
                     "kkt_passes": so["kkt_passes"], "objective": obj,
                     "parity_vs_gpu_fp64": {
                         "same_status": so["termination_status"] == c0["status"],
                         "same_kkt_passes": so["kkt_passes"] == c0["iterations"],
                         "objective_rel_diff": obj_err(c0["objective"], obj)}}
    return out


def measure_batch(h, count: int, sample: int, m_hi: int = 5000, rank: int = 0, world: int = 1,
                  device=None) -> dict:
    """LPs/s to 1e-4 relative KKT on `count` random sparse LPs (m log-U[50,5000],
    n = 2m, 3-8 nonzeros per column, seed 1000 + i): the batched solver with
    FP32 iterates (stalled FP32 LPs finish in its FP64 phase) and with FP64
    iterates, against the plain FP64 one-LP-at-a-time path (cpdlp_solve) on an
    evenly spaced sample of the same LPs.  Every result's relative KKT error
    is read back and checked; objectives are compared with the FP64 batch.
    Under torchrun every rank solves its shard (index = rank mod world) and the
    LPs/s figures use the slowest rank's time; the sample runs on rank 0."""
    import numpy as np
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    from coolpdlp import native
    from coolpdlp.distributed import reduce_over_ranks, shard_indices
    all_lps = G.batch_lps(count, m_hi=m_hi)
    lps = [all_lps[k] for k in shard_indices(count, rank, world)]
    S = [native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                         lp.uc) for lp in lps]
    warm = native.default_params()
    native.batch_solve(h, S[:4], warm)          # loads the kernels
    out = {"lps": count, "nnz_total": int(sum(lp.nnz for lp in all_lps)), "ranks": world}
    res = {}
    for name, ft in (("fp32_refined", A.VAL_F32), ("fp64_batched", A.VAL_F64)):
        p = native.default_params()
        p.float_type = ft
        t0 = time.perf_counter()
        xs, ys, st = native.batch_solve(h, S, p)
        dt = reduce_over_ranks(time.perf_counter() - t0, "max", device)
        rel = np.array([max(s.err.primal / s.err.primal_scale, s.err.dual / s.err.dual_scale,
                            s.err.gap / s.err.gap_scale) for s in st])
        res[name] = xs
        te = np.array([s.time_elapsed for s in st])
        out[name] = {"lps_per_s": count / dt, "seconds": dt,
                     "lp_seconds_sum": reduce_over_ranks(float(te.sum()), "sum", device),
                     "lp_seconds_max": reduce_over_ranks(float(te.max()), "max", device),
                     "setup_seconds": float(st[0].setup_seconds),
                     "optimal": int(reduce_over_ranks(
                         sum(s.termination_status == 0 for s in st), "sum", device)),
                     "max_rel_kkt": reduce_over_ranks(float(np.nanmax(rel)), "max", device),
                     "fp64_phase_lps": int(reduce_over_ranks(
                         sum(s.refine_kkt_passes > 0 for s in st), "sum", device)),
                     "mean_passes": reduce_over_ranks(
                         float(np.sum([s.kkt_passes for s in st])), "sum", device) / count}
    obj = lambda k, x: float(np.dot(lps[k].c, x))
    out["max_obj_rel_diff_fp32_vs_fp64"] = reduce_over_ranks(float(max(
        abs(obj(k, res["fp32_refined"][k]) - obj(k, res["fp64_batched"][k]))
        / max(1.0, abs(obj(k, res["fp64_batched"][k]))) for k in range(len(lps)))), "max", device)
    out["workload"] = (f"{count} random sparse LPs, m log-U[50,{m_hi}], n=2m, 3-8 nnz/column, "
                       "seed 1000+i, 1e-4 relative KKT")
    if sample <= 0 or rank != 0:
        return out
    idx = list(range(0, count, max(1, count // max(sample, 1))))[:sample]
    p = native.default_params()
    t0 = time.perf_counter()
    passes = 0
    for k in idx:
        lp = all_lps[k]
        _, _, s1 = native.solve_lp(h, native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval,
                                                      lp.c, lp.lv, lp.uv, lp.lc, lp.uc), p)
        passes += s1.kkt_passes
    dt = time.perf_counter() - t0
    seq = len(idx) / dt
    out["fp64_sequential"] = {"lps_per_s": seq, "sample": len(idx), "seconds": dt,
                              "mean_passes": passes / len(idx)}
    out["speedup_fp32_refined_vs_sequential"] = out["fp32_refined"]["lps_per_s"] / seq
    out["speedup_fp64_batched_vs_sequential"] = out["fp64_batched"]["lps_per_s"] / seq
    if world > 1:  # the sample's indices are global, the results are this rank's shard
        return out
    # every batched result of the sample against the FP64 path solved to 1e-8
    errs = {"fp32_refined": [], "fp64_batched": []}
    for k in idx:
        ref, st = fp64_reference(h, all_lps[k])
        for name in errs:
            errs[name].append(obj_err(obj(k, res[name][k]), ref))
    out["err_vs_fp64"] = {"reference": ("plain FP64 path (cpdlp_solve) to 1e-8 relative KKT on "
                                        f"the same {len(idx)}-LP sample; relative objective error"),
                          **{name: err_summary(v) for name, v in errs.items()}}
    return out


def layout_params(prm, args):
    """--matrix-type, --tile-nnz and --density-order (profiling: a pinned
    layout, no autotuner launches) on a problem's parameters."""
    from coolpdlp import _abi as A
    if args is None:
        return
    prm.matrix_type = {"auto": A.FMT_AUTO, "csr": A.FMT_CSR, "ell": A.FMT_ELL}[args.matrix_type]
    prm.tile_nnz = args.tile_nnz
    prm.tile_flags |= {"auto": 0, "on": A.TILE_DENSITY_ORDER,
                       "off": A.TILE_NO_DENSITY_ORDER}[args.density_order]


def measure_flow(h, side: int, K: int, blocks: int = 10, solves: bool = True,
                 args=None) -> dict:
    """The structured multicommodity min-cost flow LP (side x side grid, K
    commodities, matrix values exactly +-1): FP32 PDLP iterations per second
    with the narrow +-1 storage (the default) and with the scaled values
    (CPDLP_TILE_NO_NARROW), per-kernel GB/s from CUDA events, and cpdlp_solve to
    1e-4 (FP32) and to 1e-8 (FP32 + refinement rounds with FP64 residuals)."""
    import ctypes
    import numpy as np
    import torch
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    from coolpdlp import native
    lp = G.multicommodity_flow_lp(side=side, K=K, seed=2)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    peak, peak_kind = load_peak()
    out = {"workload": (f"multicommodity flow LP, {side}x{side} grid, K={K}, seed 2: "
                        f"m={lp.m:,} n={lp.n:,} nnz={lp.nnz:,}, values exactly +-1"),
           "peak_gbs": peak, "peak_source": peak_kind}
    ext = torch.cuda.ExternalStream(h.stream)
    for name, flags in (("narrow", 0), ("valued", A.TILE_NO_NARROW)):
        prm = A.default_params_py(A.ALGO_PDLP)
        prm.float_type = A.VAL_F32
        prm.tile_flags = flags
        prm.termination_reltol = 0.0
        prm.max_kkt_passes = 1 << 60
        prm.time_limit = 1e30
        layout_params(prm, args)
        P = native.Problem(h, L, prm)
        S = native.State(P, prm)
        for _ in range(3):
            S.solve_blocks(1)
        h.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(blocks):
            S.solve_blocks(1)
        e1.record(ext)
        h.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        prof = S.profile(20)
        kb = S.kernel_bytes()
        out[name] = {
            "iters_per_s": blocks * CHECK_EVERY / (ms * 1e-3), "layout": P.layout(),
            "kernels": {nm: {"ms": float(prof[i]), "bytes": float(kb[i]),
                             "gbs": float(kb[i] / (prof[i] * 1e-3) / 1e9),
                             "frac": float(kb[i] / (prof[i] * 1e-3) / 1e9 / peak)}
                        for i, nm in enumerate(("primal_step", "dual_step", "kkt4"))}}
        del S, P
    out["narrow_speedup"] = out["narrow"]["iters_per_s"] / out["valued"]["iters_per_s"]
    for tag, tol, refine in ((("solve_1e-4", 1e-4, 0.0), ("solve_1e-8", 1e-4, 1e-8))
                             if solves else ()):
        prm = A.default_params_py(A.ALGO_PDLP)
        prm.float_type = A.VAL_F32
        prm.termination_reltol = tol
        prm.refine_reltol = refine
        prm.max_kkt_passes = 1 << 40
        prm.time_limit = 300.0
        t0 = time.perf_counter()
        x, y, st = native.solve_lp(h, L, prm)
        dt = time.perf_counter() - t0
        e = st.err
        rel = max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)
        out[tag] = {"status": int(st.termination_status), "iterations": int(st.kkt_passes),
                    "refine_iterations": int(st.refine_kkt_passes), "rel_kkt": rel,
                    "seconds": dt, "objective": float(np.dot(lp.c, x))}
    if solves:
        out["err_vs_fp64"] = fp64_verified_errors(out)
    return out


def fp64_verified_errors(sec: dict) -> dict:
    """Objective error of the 1e-4 result against the 1e-8 result, whose KKT
    error is evaluated in FP64 on the FP64 copy of the LP (the refinement's
    FP64 residuals): the FP64 reference at sizes where the plain FP64 path
    cannot reach 1e-8 within the bench."""
    ref = sec["solve_1e-8"]
    return {"reference": ("solve_1e-8 result (FP32 corrections accumulated in FP64, KKT "
                          f"evaluated in FP64: relative KKT {ref['rel_kkt']:.2e}, status "
                          f"{ref['status']})"),
            "solve_1e-4": obj_err(sec["solve_1e-4"]["objective"], ref["objective"]),
            "solve_1e-8": 0.0}


def measure_c1_solves(h, lp, tl_1e4: float, tl_1e8: float) -> dict:
    """cpdlp_solve of the large single LP from host memory: to 1e-4 relative
    KKT with FP32 iterates, and to 1e-8 with FP32 iterates plus refinement
    rounds (FP64 residuals and KKT errors); iterations, seconds, final relative
    KKT error and objective, each within the stated time limit."""
    import numpy as np
    from coolpdlp import _abi as A
    from coolpdlp import native
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    out = {}
    for tag, tol, refine, tl in (("solve_1e-4", 1e-4, 0.0, tl_1e4),
                                 ("solve_1e-8", 1e-4, 1e-8, tl_1e8)):
        prm = A.default_params_py(A.ALGO_PDLP)
        prm.float_type = A.VAL_F32
        prm.termination_reltol = tol
        prm.refine_reltol = refine
        prm.max_kkt_passes = 1 << 40
        prm.time_limit = tl
        t0 = time.perf_counter()
        x, y, st = native.solve_lp(h, L, prm)
        dt = time.perf_counter() - t0
        e = st.err
        out[tag] = {"status": int(st.termination_status), "iterations": int(st.kkt_passes),
                    "refine_iterations": int(st.refine_kkt_passes), "rel_kkt": rel_kkt(st),
                    "rel_primal": e.primal / e.primal_scale, "rel_dual": e.dual / e.dual_scale,
                    "rel_gap": e.gap / e.gap_scale, "seconds": dt,
                    "iters_per_s": st.kkt_passes / dt, "time_limit_s": tl,
                    "objective": float(np.dot(lp.c, x))}
    out["err_vs_fp64"] = fp64_verified_errors(out)
    return out


def measure_c0(h, reps: int = 5) -> dict:
    """The 1,000 x 2,000 random sparse LP (5 nonzeros per column, seed 0) with
    plain FP64 PDLP to 1e-4 through cpdlp_solve: iterations/s, kernel launches
    per iteration and the result (its oracle parity is in cpu_baseline.c0)."""
    import numpy as np
    from coolpdlp import generators as G
    from coolpdlp import native
    lp = G.random_sparse_lp(1000, 2000, 5, seed=0)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    p = native.default_params()
    native.solve_lp(h, L, p)  # warm-up (module load, allocator pools)
    ts = []
    for _ in range(reps):
        a = time.perf_counter()
        x, y, st = native.solve_lp(h, L, p)
        ts.append(time.perf_counter() - a)
    t = statistics.median(ts)
    return {"workload": "random sparse LP m=1,000 n=2,000 5 nnz/column seed 0, FP64, 1e-4",
            "status": int(st.termination_status), "iterations": int(st.kkt_passes),
            "seconds": t, "iters_per_s": st.kkt_passes / t,
            "launches_per_iter": st.kernel_launches / max(1, st.kkt_passes),
            "objective": float(np.dot(lp.c, x)), "rel_kkt": rel_kkt(st)}


def measure_serving(requests: int, rates, err_sample: int = 12) -> dict:
    """The served stream: Poisson arrivals, 80% random sparse LPs (m log-U[100,
    20000]) and 20% grid multicommodity flows (side U{32..128}, K U{2..8}),
    tolerance 1e-4 or 1e-8; replayed in real time through the continuous-
    batching server with FP32+FP64-refined iterates at each arrival rate of
    `rates` (the first also with plain FP64 iterates), then all requests
    arriving at once (throughput when the GPU is the bottleneck).  A sample of
    the served results is checked against the plain FP64 path to 1e-8."""
    import numpy as np
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    from coolpdlp import native
    from coolpdlp import serving
    out = {"requests": requests, "rates_per_s": list(rates),
           "workload": (f"{requests} Poisson arrivals per rate: 80% random sparse LPs "
                        "m log-U[100,20000] n=2m 5 nnz/col, 20% grid multicommodity flows "
                        "side U{32..128} K U{2..8}; tolerance 1e-4 or 1e-8; "
                        "150 GB admission budget")}
    t0 = time.perf_counter()
    reqs = G.served_stream(requests, 1.0, seed=7)
    lps = [G.request_lp(r) for r in reqs]
    out["generation_s"] = time.perf_counter() - t0
    base = np.array([q.arrival for q in reqs])   # arrival times at 1 request/s
    tols = [q.reltol for q in reqs]
    sweep = {}
    kept = {}
    for i, rate in enumerate(rates):
        modes = (("fp32_refined", A.VAL_F32), ("fp64", A.VAL_F64)) if i == 0 else \
            (("fp32_refined", A.VAL_F32),)
        row = {}
        for name, ft in modes:
            srv = serving.Server(float_type=ft, hbm_budget=150e9)
            row[name] = serving.replay(srv, list(base / rate), lps, tols)
            if i == 0:
                kept[name] = dict(srv.results)
            srv.close()
        sweep[f"{rate:g}/s"] = row
    out["sweep"] = sweep
    # the plain FP64 path one request at a time (cpdlp_solve), evenly spaced sample
    h = native.Handle(0)
    idx = list(range(0, requests, max(1, requests // 40)))[:40]
    t0 = time.perf_counter()
    for i in idx:
        lp = lps[i]
        p = native.default_params()
        p.termination_reltol = reqs[i].reltol
        native.solve_lp(h, native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c,
                                           lp.lv, lp.uv, lp.lc, lp.uc), p)
    seq = len(idx) / (time.perf_counter() - t0)
    out["fp64_sequential"] = {"lps_per_s": seq, "sample": len(idx)}
    for row in sweep.values():
        for r in row.values():
            r["throughput_vs_sequential"] = r["throughput_lps_per_s"] / seq
    srv = serving.Server(float_type=A.VAL_F32, hbm_budget=150e9)
    r = serving.replay(srv, [0.0] * len(reqs), lps, tols)
    srv.close()
    r["throughput_vs_sequential"] = r["throughput_lps_per_s"] / seq
    out["fp32_refined_saturated"] = r
    # served results (first rate) against the FP64 path to 1e-8, on the
    # requests of the batched route (up to 40,000 nonzeros), evenly spaced
    small = [i for i in range(requests) if lps[i].nnz <= 40_000]
    pick = small[::max(1, len(small) // err_sample)][:err_sample]
    errs = {name: {"1e-4": [], "1e-8": []} for name in kept}
    for i in pick:
        ref, _ = fp64_reference(h, lps[i])
        key = "1e-8" if tols[i] < 1e-6 else "1e-4"
        for name, res in kept.items():
            errs[name][key].append(obj_err(float(lps[i].c @ res[i].x), ref))
    out["err_vs_fp64"] = {
        "reference": ("plain FP64 path (cpdlp_solve) to 1e-8 relative KKT; relative objective "
                      f"error of {len(pick)} served results of the first rate, by requested "
                      "tolerance"),
        **{name: {k: err_summary(v) for k, v in d.items() if v} for name, d in errs.items()}}
    return out


def measure_serving_stream(requests: int, rate: float, err_sample: int = 24,
                           seq_sample: int = 40) -> dict:
    """One long served stream (the full request count of the served workload)
    at one Poisson rate, FP32+FP64-refined iterates, each LP built on arrival.
    The x and y of an evenly spaced sample of requests are kept and checked
    against the plain FP64 path to 1e-8; the plain FP64 path's one-at-a-time
    throughput is timed on another evenly spaced sample."""
    import numpy as np
    from coolpdlp import _abi as A
    from coolpdlp import generators as G
    from coolpdlp import native
    from coolpdlp import serving
    reqs = G.served_stream(requests, 1.0, seed=7)
    arrivals = [q.arrival / rate for q in reqs]
    tols = [q.reltol for q in reqs]
    pick = list(range(0, requests, max(1, requests // err_sample)))[:err_sample]
    srv = serving.Server(float_type=A.VAL_F32, hbm_budget=150e9, keep=set(pick))
    out = {"requests": requests, "rate_per_s": rate,
           "workload": (f"{requests} Poisson arrivals at {rate:g}/s: 80% random sparse LPs "
                        "m log-U[100,20000] n=2m 5 nnz/col, 20% grid multicommodity flows "
                        "side U{32..128} K U{2..8}; tolerance 1e-4 or 1e-8; "
                        "150 GB admission budget; LPs built on arrival")}
    out["fp32_refined"] = serving.replay(srv, arrivals, lambda i: G.request_lp(reqs[i]), tols,
                                         timeout=4 * 3600.0)
    results = srv.results
    srv.close()
    notopt = [i for i in range(requests) if int(results[i].stats.termination_status) != 0]
    out["not_optimal"] = {
        "count": len(notopt),
        "by_route": {rt: sum(1 for i in notopt if results[i].route == rt)
                     for rt in ("batch", "single")},
        "first": [[i, reqs[i].kind, reqs[i].m, tols[i], results[i].route,
                   int(results[i].stats.termination_status), int(results[i].stats.kkt_passes)]
                  for i in notopt[:20]]}
    h = native.Handle(0)
    # the plain FP64 path (same pass limit) on the first few of them
    same = []
    for i in notopt[:6]:
        lp = G.request_lp(reqs[i])
        p = native.default_params()
        p.termination_reltol = tols[i]
        _, _, st = native.solve_lp(h, native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval,
                                                      lp.c, lp.lv, lp.uv, lp.lc, lp.uc), p)
        same.append([i, int(st.termination_status), int(st.kkt_passes)])
    out["not_optimal"]["plain_fp64_path"] = same
    seq_idx = list(range(0, requests, max(1, requests // seq_sample)))[:seq_sample]
    t0 = time.perf_counter()
    for i in seq_idx:
        lp = G.request_lp(reqs[i])
        p = native.default_params()
        p.termination_reltol = tols[i]
        native.solve_lp(h, native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c,
                                           lp.lv, lp.uv, lp.lc, lp.uc), p)
    seq = len(seq_idx) / (time.perf_counter() - t0)
    out["fp64_sequential"] = {"lps_per_s": seq, "sample": len(seq_idx),
                              "what": "cpdlp_solve one request at a time, LP building excluded"}
    out["fp32_refined"]["throughput_vs_sequential"] = \
        out["fp32_refined"]["throughput_lps_per_s"] / seq
    errs = {"1e-4": [], "1e-8": []}
    for i in pick:
        lp = G.request_lp(reqs[i])
        ref, _ = fp64_reference(h, lp)
        errs["1e-8" if tols[i] < 1e-6 else "1e-4"].append(obj_err(float(lp.c @ results[i].x), ref))
    out["err_vs_fp64"] = {
        "reference": ("plain FP64 path (cpdlp_solve) to 1e-8 relative KKT; relative objective "
                      f"error of {len(pick)} evenly spaced served results, by requested tolerance"),
        **{k: err_summary(v) for k, v in errs.items() if v}}
    return out


def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    lp = workload(args.scale)
    prm = O.params(termination_reltol=0.0, max_kkt_passes=1 << 60, time_limit=1e30)
    S = O.OracleState(lp, prm)
    # a step is the GPU arm's: one solve! block of CHECK_EVERY PDLP iterations
    # plus its termination/restart check (about 1.3 s on 16 Grace cores)
    for _ in range(args.warmup):
        S.solve_blocks(1)
    p0 = S.stats()["kkt_passes"]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        S.solve_blocks(1)
    dt = time.perf_counter() - t0
    iters = S.stats()["kkt_passes"] - p0
    S.close()
    v = iters / dt
    cores = int(O.lib().orc_num_threads())
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(lp, args.scale),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": (f"{args.steps} solve! blocks of {CHECK_EVERY} PDLP iterations "
                                    "+ one termination/restart check each (FP64)")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "precision": "FP64 iterates and sums (the oracle restates the reference's Float64 path)",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from coolpdlp import build as B
    B.build_library()
    from coolpdlp import _abi as A
    from coolpdlp import native

    if args.only_flow:
        if rank == 0:
            h = native.Handle(local)
            print(json.dumps({"metric": METRIC, "impl": "ours", "value": None,
                              "flow": measure_flow(h, args.flow_side, args.flow_k,
                                                   solves=not args.flow_no_solve, args=args)}),
                  flush=True)
        return
    if args.only_serving_stream > 0:
        if rank == 0:
            rate = [float(r) for r in args.serve_rates.split(",") if r][0]
            print(json.dumps({"metric": METRIC, "impl": "ours", "value": None,
                              "serving_stream": measure_serving_stream(
                                  args.only_serving_stream, rate)}), flush=True)
        return
    if args.only_batch:
        # the batched workload alone (small cases for profilers); no headline value
        h = native.Handle(local)
        b = measure_batch(h, args.batch_lps, args.sequential_sample, args.batch_m_hi, rank, ws,
                          torch.device("cuda", local))
        if rank == 0:
            print(json.dumps({"metric": METRIC, "impl": "ours", "value": None, "batch": b}),
                  flush=True)
        return
    lp = workload(args.scale)
    h = native.Handle(local)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.float_type = A.VAL_F32
    prm.termination_reltol = 0.0
    prm.max_kkt_passes = 1 << 60
    prm.time_limit = 1e30
    layout_params(prm, args)
    L = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv, lp.lc,
                        lp.uc)
    t0 = time.perf_counter()
    P = native.Problem(h, L, prm)
    S = native.State(P, prm)
    setup_s = time.perf_counter() - t0
    layout = P.layout()   # the autotuner's product format per matrix
    layout["density_order"] = P.order() is not None
    ext = torch.cuda.ExternalStream(h.stream, device=torch.device("cuda", local))

    for _ in range(args.warmup):
        S.solve_blocks(1)
    launches0 = S.stats().kernel_launches
    clk = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    h.synchronize()
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    w0 = time.perf_counter()
    for _ in range(args.steps):
        S.solve_blocks(1)
    e1.record(ext)
    h.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    launches = S.stats().kernel_launches - launches0
    ms_max = ms
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
        torch.distributed.barrier()
    iters = args.steps * CHECK_EVERY
    value = ws * iters / (ms_max * 1e-3)

    # roofline of the dominant kernel: live CUDA-event timing per kernel
    prof = S.profile(20)
    kb = S.kernel_bytes()
    names = ["primal_step", "dual_step", "kkt4"]
    per_step_ms = [prof[0] * CHECK_EVERY, prof[1] * CHECK_EVERY, prof[2]]
    dom = int(np.argmax(per_step_ms))
    peak, peak_kind = load_peak()
    kernels = {}
    for i, nm in enumerate(names):
        gbs = kb[i] / (prof[i] * 1e-3) / 1e9
        kernels[nm] = {"ms": prof[i], "bytes": kb[i], "gbs": gbs, "frac": gbs / peak,
                       "share_of_step": per_step_ms[i] / sum(per_step_ms)}
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic_powerlaw_fp32.json")
    if os.path.exists(tp) and args.scale == 1.0:
        try:
            with open(tp) as f:
                traffic = json.load(f).get(names[dom])
        except Exception:
            traffic = None
    ach = kernels[names[dom]]["gbs"]
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": ach, "peak": peak,
                "peak_source": peak_kind, "unit": "GB/s", "frac": ach / peak, "traffic": traffic}
    step_bytes = kb[0] * CHECK_EVERY + kb[1] * CHECK_EVERY + kb[2]
    hbm_gbs_whole = step_bytes * args.steps / (ms * 1e-3) / 1e9

    # e2e through cpdlp_solve with pinned host buffers
    def pinned(a, dt):
        t = torch.empty(a.shape, dtype=dt, pin_memory=True)
        t.numpy()[...] = a
        return t
    pins = [pinned(lp.colptr, torch.int64), pinned(lp.rowval, torch.int64),
            pinned(lp.nzval, torch.float64), pinned(lp.c, torch.float64),
            pinned(lp.lv, torch.float64), pinned(lp.uv, torch.float64),
            pinned(lp.lc, torch.float64), pinned(lp.uc, torch.float64)]
    Lp = native.LPStruct(lp.m, lp.n, *[p.numpy() for p in pins])
    xo = torch.empty(lp.n, dtype=torch.float64, pin_memory=True)
    yo = torch.empty(lp.m, dtype=torch.float64, pin_memory=True)
    prm_e = A.ParamsC.from_buffer_copy(prm)
    prm_e.max_kkt_passes = E2E_ITERS
    import ctypes
    def e2e_once():
        st = A.StatsC()
        h.check(h.lib.cpdlp_solve(h.h, ctypes.byref(Lp.s), ctypes.byref(prm_e), None, None,
                                  native._pd(xo.numpy()), native._pd(yo.numpy()),
                                  ctypes.byref(st)), "cpdlp_solve")
        return st
    e2e_val = None
    if args.e2e_steps > 0:
        del S, P
        e2e_once()  # warm-up
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.e2e_steps):
            a = time.perf_counter()
            st = e2e_once()
            ts.append(time.perf_counter() - a)
        t_e2e = statistics.mean(ts)
        if ws > 1:
            t = torch.tensor([t_e2e], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            t_e2e = float(t.item())
        e2e_val = ws * st.kkt_passes / t_e2e
    h2d = (lp.n + 1) * 8 + lp.nnz * 16 + (3 * lp.n + 2 * lp.m) * 8
    d2h = (lp.n + lp.m) * 8 + ctypes.sizeof(A.StatsC)

    # the batched LPs shard over the ranks (every rank takes part)
    batch = None
    if args.batch_lps > 0:
        batch = measure_batch(h, args.batch_lps, args.sequential_sample, args.batch_m_hi, rank,
                              ws, torch.device("cuda", local))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(lp, args.scale),
            "hbm_gbs": hbm_gbs_whole, "layout": layout,
            "roofline": roofline, "kernels": kernels,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "what": f"cpdlp_solve of the LP from pinned host buffers, {E2E_ITERS} iterations"},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "wall_s_timed": wall, "setup_s": setup_s,
        }
        line["precision"] = {"value": "FP32 iterates and SpMVs, FP64 KKT/restart sums",
                             "e2e": "FP32 iterates and SpMVs, FP64 KKT/restart sums",
                             "cpu_baseline": "FP64 (CPU restatement of the reference)"}
        c0 = measure_c0(h)
        line["c0"] = c0
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(lp, c0=c0)
        if args.c1_solves:
            line["c1"] = measure_c1_solves(h, lp, args.c1_time_limit, args.c1_refine_time_limit)
        if args.flow_side > 0:
            line["flow"] = measure_flow(h, args.flow_side, args.flow_k,
                                        solves=not args.flow_no_solve, args=args)
        if batch is not None:
            line["batch"] = batch
        if args.serve_requests > 0:
            rates = [float(r) for r in args.serve_rates.split(",") if r]
            line["serving"] = measure_serving(args.serve_requests, rates)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
