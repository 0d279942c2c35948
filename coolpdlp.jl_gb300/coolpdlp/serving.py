"""Continuous-batching LP server on one GPU.

Requests (an LP and its target relative KKT tolerance) arrive over time.  The
server keeps a FIFO of arrived requests and, on every ``pump()``:

* admits as many waiting requests as the in-flight slot count and the HBM
  budget allow (each request's device footprint comes from
  ``cpdlp_batch_footprint``) and submits them together as one asynchronous
  job (``cpdlp_submit``): the job preprocesses its LPs on its own CUDA stream
  and a persistent kernel solves them, one LP per CTA.  Jobs admitted while
  others run execute at the same time; each job is capped at ``max_ctas``
  CTAs so that later jobs find SMs (the CTAs of a job hand their SMs over as
  its queue drains);
* routes LPs above ``big_nnz`` nonzeros (``big_nnz_refined`` for requests that
  need FP64 refinement) to the single-LP path (the whole GPU,
  graph-captured step kernels) on worker threads with their own handles, so
  that one large LP does not occupy a single CTA for seconds;
* polls every job (``cpdlp_poll`` never blocks), retires finished ones and
  releases their slots and bytes, which the next admission backfills.

Latency is measured from a request's arrival to the pump that sees it done.
With FP32 iterates the batched path stops each LP at the FP32 tolerance and
finishes LPs with tighter targets in an FP64 phase warm-started from the FP32
solution (LPs whose FP32 iterates stall restart cold in FP64); the single-LP
path refines tighter targets through refine_reltol (FP32 rounds on the FP64
residual), except that such requests under ``fp64_refined_below`` nonzeros run
FP64 iterates from the start.  There is no counterpart in the reference, which
solves one LP per call.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import threading
import time

import numpy as np

from . import _abi as A
from . import native


@dataclasses.dataclass
class Result:
    rid: int
    x: np.ndarray
    y: np.ndarray
    stats: object
    arrival: float
    admitted: float
    finished: float
    route: str               # "batch" or "single"

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclasses.dataclass
class _Waiting:
    rid: int
    lp: native.LPStruct
    reltol: float
    arrival: float
    nbytes: int
    nnz: int


class Server:
    def __init__(self, device: int = 0, float_type: int = A.VAL_F32, params: A.ParamsC = None,
                 hbm_budget: float = 150e9, max_inflight_lps: int | None = None,
                 max_job_lps: int = 1024, big_nnz: int = 40_000, max_ctas: int | None = None,
                 single_workers: int = 32, fp32_reltol: float = 1e-4, keep=None,
                 big_nnz_refined: int = 20_000, fp64_refined_below: int = 60_000):
        """keep: None keeps every result's x and y; otherwise a container of
        the request ids whose x and y are kept (the others keep their
        statistics only, which bounds host memory on long streams).
        big_nnz_refined: with FP32 iterates, requests tighter than
        fp32_reltol take the single-LP path above this many nonzeros (instead
        of big_nnz): it has the refinement rounds, a job's FP64 phase has not
        (saturated 160-request stream: 41.7 LPs/s against 36.8-40.3 with
        40,000 for every request).
        fp64_refined_below: such requests on the single-LP path with fewer
        nonzeros run FP64 iterates from the start: their kernels are
        latency-bound, so FP32 gains little, and the FP32 phase's stall rule
        and the rounds can cost passes (one 22,760-nonzero 1e-8 request ran
        into the 100,000-pass limit that plain FP64 stays under; the
        saturated stream went from 42.4 to 43.0 LPs/s with 60,000, and to
        35.6 with 150,000)."""
        self.keep = keep
        self.big_nnz_refined = int(big_nnz_refined)
        self.fp64_refined_below = int(fp64_refined_below)
        self.handle = native.Handle(device)
        self.params = params if params is not None else native.default_params()
        self.params.float_type = float_type
        self.float_type = float_type
        self.fp32_reltol = fp32_reltol
        if float_type == A.VAL_F32:
            self.params.termination_reltol = fp32_reltol
        self.hbm_budget = float(hbm_budget)
        sms = self._num_sms(device)
        self.max_ctas = int(max_ctas) if max_ctas is not None else sms
        self.max_inflight = int(max_inflight_lps) if max_inflight_lps else 4 * sms
        self.max_job_lps = int(max_job_lps)
        self.big_nnz = int(big_nnz)
        self.waiting: collections.deque[_Waiting] = collections.deque()
        self.jobs = []      # (Job, [_Waiting], admitted time)
        self.singles = []   # (Future, _Waiting, admitted time)
        self.inflight_bytes = 0
        self.inflight_lps = 0
        self.results: dict[int, Result] = {}
        self.t0 = time.perf_counter()
        self._pool = cf.ThreadPoolExecutor(max_workers=max(1, single_workers))
        self._tls = threading.local()
        self.device = device
        self.jobs_submitted = 0
        self.peak_bytes = 0

    @staticmethod
    def _num_sms(device: int) -> int:
        try:
            import torch
            return int(torch.cuda.get_device_properties(device).multi_processor_count)
        except Exception:
            return 152

    def now(self) -> float:
        return time.perf_counter() - self.t0

    # ---- requests -------------------------------------------------------------
    def offer(self, rid: int, lp, reltol: float, arrival: float | None = None):
        """Queues a request (LPData-like: m, n, colptr, rowval, nzval, c, lv, uv,
        lc, uc; 1-based CSC).  arrival defaults to now on the server clock."""
        S = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                            lp.lc, lp.uc)
        nbytes = native.batch_footprint([S], self.params)
        if nbytes > self.hbm_budget:
            raise A.ArgumentError(A.ERR_ARGUMENT, f"request {rid} needs {nbytes} device bytes, "
                                                  f"above the {self.hbm_budget:.0f}-byte budget")
        self.waiting.append(_Waiting(rid, S, float(reltol),
                                     self.now() if arrival is None else float(arrival),
                                     nbytes, int(S.s.nnz)))

    # ---- the loop -------------------------------------------------------------
    def pump(self) -> int:
        """Retires finished work, then admits waiting requests; never blocks on
        the GPU.  Returns the number of requests finished in this call."""
        done = self._retire()
        self._admit()
        return done

    def idle(self) -> bool:
        return not self.waiting and not self.jobs and not self.singles

    def _retire(self) -> int:
        finished = 0
        still = []
        for job, reqs, t_adm in self.jobs:
            all_done = job.poll()
            t = self.now()
            ready = job.ready()
            for k, w in enumerate(reqs):
                if ready[k] and w.rid not in self.results:
                    x, y, st = job.collect_lp(k)
                    if not self._kept(w.rid):
                        x = y = None
                    self.results[w.rid] = Result(w.rid, x, y, st, w.arrival, t_adm, t, "batch")
                    self.inflight_bytes -= w.nbytes
                    self.inflight_lps -= 1
                    finished += 1
            if all_done:
                job.close()
            else:
                still.append((job, reqs, t_adm))
        self.jobs = still
        still = []
        for fut, w, t_adm in self.singles:
            if not fut.done():
                still.append((fut, w, t_adm))
                continue
            x, y, st = fut.result()
            if not self._kept(w.rid):
                x = y = None
            self.results[w.rid] = Result(w.rid, x, y, st, w.arrival, t_adm, self.now(), "single")
            self.inflight_bytes -= w.nbytes
            self.inflight_lps -= 1
            finished += 1
        self.singles = still
        return finished

    def _threshold(self, w: _Waiting) -> int:
        refined = self.float_type == A.VAL_F32 and w.reltol < self.fp32_reltol
        return min(self.big_nnz, self.big_nnz_refined) if refined else self.big_nnz

    def _kept(self, rid: int) -> bool:
        return self.keep is None or rid in self.keep

    def _fits(self, w: _Waiting) -> bool:
        return (self.inflight_lps < self.max_inflight
                and self.inflight_bytes + w.nbytes <= self.hbm_budget)

    def _admit(self):
        batch, tols = [], []
        while self.waiting and len(batch) < self.max_job_lps:
            w = self.waiting[0]
            if not self._fits(w):
                break
            self.waiting.popleft()
            self.inflight_bytes += w.nbytes
            self.inflight_lps += 1
            self.peak_bytes = max(self.peak_bytes, self.inflight_bytes)
            if w.nnz > self._threshold(w):
                self.singles.append((self._pool.submit(self._solve_single, w), w, self.now()))
            else:
                batch.append(w)
                tols.append(w.reltol)
        if batch:
            job = native.Job(self.handle, [w.lp for w in batch], self.params, reltol=tols,
                             max_ctas=self.max_ctas)
            self.jobs.append((job, batch, self.now()))
            self.jobs_submitted += 1

    def _solve_single(self, w: _Waiting):
        h = getattr(self._tls, "handle", None)
        if h is None:
            h = self._tls.handle = native.Handle(self.device)
        p = native.copy_params(self.params)
        if self.float_type == A.VAL_F32 and not (w.reltol < self.fp32_reltol
                                                 and w.nnz < self.fp64_refined_below):
            # FP32 to the FP32 tolerance; FP64 for tighter targets and stalls
            p.termination_reltol = max(self.fp32_reltol, w.reltol)
            p.refine_reltol = w.reltol
        else:
            p.float_type = A.VAL_F64
            p.termination_reltol = w.reltol
        return native.solve_lp(h, w.lp, p)

    def close(self):
        self._pool.shutdown(wait=True)
        for job, _, _ in self.jobs:
            job.close()
        self.jobs = []


def replay(server: Server, arrivals, lps, reltols, poll_sleep: float = 2e-4,
           timeout: float = 3600.0) -> dict:
    """Replays a request stream in real time: request i is offered once the
    server clock reaches arrivals[i] (seconds); returns latency and
    throughput figures, overall and by requested tolerance.  lps[i] is the LP
    of request i, or lps is a callable that builds it on arrival (long
    streams: the LPs are not all held in host memory; see Server.keep for
    the solutions)."""
    get = lps if callable(lps) else (lambda i: lps[i])
    order = np.argsort(np.asarray(arrivals), kind="stable")
    server.t0 = time.perf_counter()
    nxt = 0
    n = len(order)
    while True:
        now = server.now()
        while nxt < n and arrivals[order[nxt]] <= now:
            i = int(order[nxt])
            server.offer(i, get(i), reltols[i], arrival=float(arrivals[i]))
            nxt += 1
        server.pump()
        if nxt == n and server.idle():
            break
        if now > timeout:
            raise TimeoutError("served stream did not finish")
        time.sleep(poll_sleep)
    lat = np.array([server.results[i].latency for i in range(n)])
    finish = max(r.finished for r in server.results.values())
    status = np.bincount([int(server.results[i].stats.termination_status) for i in range(n)],
                         minlength=4)
    tol = np.asarray(reltols, dtype=np.float64)[:n]
    by_tol = {}
    for t in sorted(set(tol.tolist())):
        sel = tol == t
        by_tol[f"{t:g}"] = {"requests": int(sel.sum()),
                            "p50_ms": float(np.percentile(lat[sel], 50) * 1e3),
                            "p99_ms": float(np.percentile(lat[sel], 99) * 1e3)}
    return {
        "requests": n,
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_ms": float(lat.mean() * 1e3),
        "throughput_lps_per_s": float(n / finish) if finish > 0 else None,
        "makespan_s": float(finish),
        "status_counts": [int(v) for v in status],
        "jobs": server.jobs_submitted,
        "single_route": int(sum(1 for r in server.results.values() if r.route == "single")),
        "peak_admitted_bytes": int(server.peak_bytes),
        "by_tolerance": by_tol,
    }
