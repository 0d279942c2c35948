"""The served-stream replay loop (coolpdlp.serving.replay) on the CPU, against a
stub server that finishes each request a fixed time after it is offered:
arrival order, lazily built LPs (a callable), latency percentiles overall and
by requested tolerance, status counts and throughput are the loop's own host
logic and need no GPU."""
import time
import types

import numpy as np


class _StubServer:
    def __init__(self, service_s):
        self.service_s = service_s
        self.t0 = time.perf_counter()
        self.pending = []
        self.results = {}
        self.jobs_submitted = 0
        self.peak_bytes = 123
        self.offered = []

    def now(self):
        return time.perf_counter() - self.t0

    def offer(self, rid, lp, reltol, arrival=None):
        self.offered.append((rid, lp, reltol))
        self.pending.append((rid, arrival, self.now()))

    def pump(self):
        from coolpdlp import serving
        t = self.now()
        still = []
        for rid, arrival, admitted in self.pending:
            if t - admitted >= self.service_s:
                st = types.SimpleNamespace(termination_status=0 if rid % 5 else 2)
                self.results[rid] = serving.Result(rid, None, None, st, arrival, admitted, t,
                                                   "batch" if rid % 2 else "single")
                self.jobs_submitted += 1
            else:
                still.append((rid, arrival, admitted))
        self.pending = still
        return 0

    def idle(self):
        return not self.pending


def test_replay_accounting_with_lazy_lps():
    from coolpdlp import serving
    n = 20
    arrivals = list(np.linspace(0.0, 0.05, n)[::-1])     # offered in arrival order
    tols = [1e-8 if i % 2 else 1e-4 for i in range(n)]
    built = []

    def make(i):
        built.append(i)
        return ("lp", i)

    srv = _StubServer(service_s=0.01)
    out = serving.replay(srv, arrivals, make, tols, poll_sleep=1e-4)
    assert sorted(built) == list(range(n))
    assert [rid for rid, _, _ in srv.offered] == sorted(range(n), key=lambda i: arrivals[i])
    assert all(lp == ("lp", rid) for rid, lp, _ in srv.offered)
    assert out["requests"] == n
    assert out["status_counts"] == [16, 0, 4, 0]          # rid % 5 == 0 stop at the limit
    assert out["single_route"] == 10 and out["jobs"] == n and out["peak_admitted_bytes"] == 123
    assert out["p99_ms"] >= out["p50_ms"] >= 10.0          # at least the service time
    assert set(out["by_tolerance"]) == {"1e-08", "0.0001"}
    assert sum(v["requests"] for v in out["by_tolerance"].values()) == n
    lat = np.array([srv.results[i].latency for i in range(n)]) * 1e3
    assert abs(out["p50_ms"] - np.percentile(lat, 50)) < 1e-9
    assert out["throughput_lps_per_s"] == n / out["makespan_s"]
