"""The continuous-batching server (coolpdlp.serving): requests that arrive
while others run are admitted as slots and HBM budget free up, their work
overlaps on the GPU, and every result equals the result of the same request
solved alone (bit-identical: an LP's arithmetic does not depend on the mix).
Every served result is also checked against HiGHS's optimal objective for its
LP (committed fixture, tests/golden/): within 1e-6 relative for requests at
1e-8 relative KKT, within 1e-2 for requests at 1e-4."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream(count=36, rate=400.0, seed=11):
    from coolpdlp import generators as G
    reqs = G.served_stream(count, rate, seed=seed, m_lo=60, m_hi=1500, side_lo=6, side_hi=14,
                           k_lo=2, k_hi=4)
    lps = [G.request_lp(r) for r in reqs]
    return reqs, lps


def _rel(st):
    e = st.err
    return max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)


@pytest.mark.parametrize("float_type", [1, 0])
def test_served_stream_equals_alone(float_type):
    from coolpdlp import native, serving, _abi as A
    reqs, lps = _stream()
    server = serving.Server(float_type=float_type, big_nnz=4000, max_ctas=16,
                            max_inflight_lps=24)
    out = serving.replay(server, [r.arrival for r in reqs], lps, [r.reltol for r in reqs])
    assert out["requests"] == len(reqs)
    assert out["status_counts"][0] == len(reqs), out
    assert out["jobs"] >= 2 and out["single_route"] >= 1, out
    assert out["p99_ms"] >= out["p50_ms"] > 0
    overlapped = 0
    h = native.Handle(0)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "golden.json")) as f:
        highs = {d["rid"]: d for d in json.load(f)["served"]}
    for r in reqs:
        res = server.results[r.rid]
        assert _rel(res.stats) <= r.reltol, (r.rid, _rel(res.stats), r.reltol)
        want = highs[r.rid]
        assert want["name"] == lps[r.rid].name and want["reltol"] == r.reltol
        obj, ref = float(lps[r.rid].c @ res.x), want["objective"]
        tol = 1e-6 if r.reltol < 1e-6 else 1e-2
        assert abs(obj - ref) <= tol * max(1.0, abs(ref)), (r.rid, r.reltol, obj, ref)
        lp = lps[r.rid]
        S = native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                            lp.lc, lp.uc)
        if res.route == "batch":
            x1, y1, s1 = native.Job(h, [S], server.params, reltol=[r.reltol]).result()
            x1, y1, s1 = x1[0], y1[0], s1[0]
        else:
            x1, y1, s1 = server._solve_single(serving._Waiting(r.rid, S, r.reltol, 0.0, 0,
                                                                int(S.s.nnz)))
        assert np.array_equal(x1, res.x) and np.array_equal(y1, res.y), (r.rid, res.route)
        assert s1.kkt_passes == res.stats.kkt_passes
        overlapped += int(any(o.admitted < res.finished and o.finished > res.admitted
                              for o in server.results.values() if o.rid != r.rid))
    assert overlapped >= len(reqs) // 2   # requests really ran while others were in flight
    server.close()


def test_admission_respects_hbm_budget():
    from coolpdlp import native, serving, _abi as A
    reqs, lps = _stream(count=12, rate=1000.0, seed=5)
    probe = serving.Server(float_type=A.VAL_F32)
    sizes = []
    for i, lp in enumerate(lps):
        probe.offer(i, lp, 1e-4)
        sizes.append(probe.waiting[-1].nbytes)
    probe.close()
    budget = 2.5 * max(sizes)
    server = serving.Server(float_type=A.VAL_F32, hbm_budget=budget, big_nnz=10**9)
    out = serving.replay(server, [r.arrival for r in reqs], lps, [1e-4] * len(reqs))
    assert out["status_counts"][0] == len(reqs)
    assert 0 < out["peak_admitted_bytes"] <= budget
    assert out["jobs"] >= 3
    server.close()


def test_lazy_stream_keeps_only_sampled_solutions():
    """LPs built on arrival (replay with a callable) and Server(keep=...): the
    kept requests' x and y equal those of the same stream replayed with every
    LP built up front; the others keep their statistics only; the per-tolerance
    latency figures cover every request."""
    from coolpdlp import generators as G
    from coolpdlp import serving, _abi as A
    reqs, lps = _stream(count=16, rate=800.0, seed=3)
    keep = {0, 5, 11}
    built = []

    def make(i):
        built.append(i)
        return G.request_lp(reqs[i])

    lazy = serving.Server(float_type=A.VAL_F32, big_nnz=4000, max_ctas=16, keep=keep)
    out = serving.replay(lazy, [r.arrival for r in reqs], make, [r.reltol for r in reqs])
    full = serving.Server(float_type=A.VAL_F32, big_nnz=4000, max_ctas=16)
    serving.replay(full, [r.arrival for r in reqs], lps, [r.reltol for r in reqs])
    assert sorted(built) == list(range(len(reqs)))
    assert out["status_counts"][0] == len(reqs)
    assert sum(v["requests"] for v in out["by_tolerance"].values()) == len(reqs)
    for i in range(len(reqs)):
        got, ref = lazy.results[i], full.results[i]
        assert got.stats.kkt_passes == ref.stats.kkt_passes
        if i in keep:
            assert np.array_equal(got.x, ref.x) and np.array_equal(got.y, ref.y)
        else:
            assert got.x is None and got.y is None
    lazy.close()
    full.close()
