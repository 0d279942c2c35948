"""The batched persistent solver (cpdlp_batch_solve) and asynchronous jobs
(cpdlp_submit / poll / cancel / collect): many LPs of uneven size in one
launch, one LP per CTA.

Tolerances: a batch result and the single-LP device result of the same LP
follow different reduction orders, so their trajectories drift apart in the
last bits; both must reach the stated relative KKT tolerance, and their
objectives must agree within 1e-6 relative when both are solved to 1e-8
(FP64).  FP32 results at 1e-4 are compared with the FP64 oracle's objective
within the reference's own tolerance at 1e-4 (rtol 1e-2, test/algorithms/all.jl:36-38).  The same LP alone and in a mix gives bit-identical
results (its arithmetic does not depend on the other LPs)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _set(count=20, seed0=500):
    """Small random LPs (one CTA each), the reference suite's two tiny LPs, a
    flow LP, and two LPs above 12,000 nonzeros (a thread-block cluster each)."""
    from coolpdlp import generators as G
    lps = G.batch_lps(count, m_lo=40, m_hi=400, seed0=seed0)
    lps.append(G.two_variable_lp())
    lps.append(G.termination_check_lp())
    lps.append(G.multicommodity_flow_lp(side=6, K=2, seed=9))
    lps.append(G.random_sparse_lp(2600, 5200, 5, seed=seed0 + 77))
    lps.append(G.random_sparse_lp(4000, 8000, 4, seed=seed0 + 78))
    return lps


def _structs(lps):
    from coolpdlp import native
    return [native.LPStruct(lp.m, lp.n, lp.colptr, lp.rowval, lp.nzval, lp.c, lp.lv, lp.uv,
                            lp.lc, lp.uc) for lp in lps]


def _rel(st):
    e = st.err
    return max(e.primal / e.primal_scale, e.dual / e.dual_scale, e.gap / e.gap_scale)


def _obj(lp, x):
    return float(np.dot(lp.c, x))


def test_batch_fp64_matches_single_lp_path(handle):
    from coolpdlp import native, _abi as A
    lps = _set(12)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.termination_reltol = 1e-8
    xs, ys, st = native.batch_solve(handle, S, prm)
    for k, lp in enumerate(lps):
        x1, _, s1 = native.solve_lp(handle, S[k], prm)
        assert s1.termination_status == 0 and st[k].termination_status == 0, (k, lp.name)
        assert _rel(st[k]) <= 1e-8, (k, lp.name, _rel(st[k]))
        o_b, o_s = _obj(lp, xs[k]), _obj(lp, x1)
        assert abs(o_b - o_s) <= 1e-6 * max(1.0, abs(o_s)), (k, lp.name, o_b, o_s)
        assert st[k].kkt_passes % prm.check_every == 0


def test_batch_fp32_against_oracle(handle, oracle):
    from coolpdlp import native, _abi as A
    lps = _set(12, seed0=900)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.float_type = A.VAL_F32
    xs, ys, st = native.batch_solve(handle, S, prm)
    for k, lp in enumerate(lps):
        xo, yo, so = oracle.solve(lp, oracle.params())
        assert so["termination_status"] == 0
        assert st[k].termination_status == 0, (k, lp.name, st[k].kkt_passes)
        assert _rel(st[k]) <= 1e-4
        oo = _obj(lp, xo)
        # two 1e-4-accurate solutions: the reference's own objective tolerance at
        # 1e-4 (rtol 1e-2, test/algorithms/all.jl:36-38)
        assert abs(_obj(lp, xs[k]) - oo) <= 1e-2 * max(1.0, abs(oo)), (k, lp.name)


def test_batch_fp32_refined_to_1e8(handle, oracle):
    """FP32 to 1e-4, then the batched FP64 phase warm-started from the FP32
    solution to 1e-8 (the refinement of cpdlp_solve, batched)."""
    from coolpdlp import native, _abi as A
    lps = _set(8, seed0=1300)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.float_type = A.VAL_F32
    prm.refine_reltol = 1e-8
    xs, ys, st = native.batch_solve(handle, S, prm)
    refined = 0
    for k, lp in enumerate(lps):
        assert st[k].termination_status == 0, (k, lp.name)
        assert _rel(st[k]) <= 1e-8, (k, lp.name, _rel(st[k]))
        refined += int(st[k].refine_kkt_passes > 0)
        xo, _, so = oracle.solve(lp, oracle.params(termination_reltol=1e-8))
        oo = _obj(lp, xo)
        assert abs(_obj(lp, xs[k]) - oo) <= 1e-6 * max(1.0, abs(oo)), (k, lp.name)
    assert refined >= len(lps) - 2   # the tiny LPs may already be at 1e-8 after FP32


@pytest.mark.parametrize("float_type", [0, 1])
def test_alone_equals_mix(handle, float_type):
    """Each LP's result (x, y, passes, errors) is bit-identical alone and inside
    a mix of other LPs, including jobs that run at the same time."""
    from coolpdlp import native, _abi as A
    lps = _set(10, seed0=2100)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.float_type = float_type
    mix_x, mix_y, mix_st = native.Job(handle, S, prm).result()
    # the same LPs alone, submitted as concurrent single-LP jobs
    jobs = [native.Job(handle, [S[k]], prm) for k in range(len(S))]
    for k, job in enumerate(jobs):
        x1, y1, s1 = job.result()
        assert np.array_equal(x1[0], mix_x[k]), k
        assert np.array_equal(y1[0], mix_y[k]), k
        assert s1[0].kkt_passes == mix_st[k].kkt_passes
        assert s1[0].termination_status == mix_st[k].termination_status
        assert s1[0].err.primal == mix_st[k].err.primal and s1[0].err.gap == mix_st[k].err.gap
        job.close()
    # and in a different mix (reversed order, two LPs repeated)
    order = list(reversed(range(len(S)))) + [0, 3]
    rx, ry, rst = native.Job(handle, [S[k] for k in order], prm).result()
    for pos, k in enumerate(order):
        assert np.array_equal(rx[pos], mix_x[k]) and np.array_equal(ry[pos], mix_y[k]), (pos, k)


def test_job_per_lp_tolerance_and_overlap(handle):
    from coolpdlp import native, _abi as A
    lps = _set(6, seed0=3100)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.float_type = A.VAL_F32
    tol = np.array([1e-4 if k % 2 == 0 else 1e-8 for k in range(len(S))])
    j1 = native.Job(handle, S, prm, reltol=tol)
    j2 = native.Job(handle, S[::-1], prm)            # submitted while j1 runs
    pending = {1: j1, 2: j2}
    t0 = time.time()
    while pending and time.time() - t0 < 120:
        for key in list(pending):
            if pending[key].poll():
                pending.pop(key)
        time.sleep(0.001)
    assert not pending
    x1, _, s1 = j1.result()
    for k in range(len(S)):
        assert s1[k].termination_status == 0
        assert _rel(s1[k]) <= tol[k]
        if tol[k] < 1e-4:
            assert s1[k].refine_kkt_passes >= 0
    x2, _, s2 = j2.result()
    for k in range(len(S)):
        assert s2[k].termination_status == 0 and _rel(s2[k]) <= 1e-4


def test_job_cancel(handle):
    """A job that cannot converge (a 1e-300 tolerance) stops at its next check
    after cancel(); unfinished LPs report STILL_RUNNING."""
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    lps = G.batch_lps(4, m_lo=200, m_hi=400, seed0=4100)
    lps.append(G.random_sparse_lp(3000, 6000, 5, seed=4177))   # a cluster's LP
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.termination_reltol = 1e-300
    prm.max_kkt_passes = 10_000_000
    prm.time_limit = 60.0
    job = native.Job(handle, S, prm)
    time.sleep(0.5)
    assert not job.poll()
    t0 = time.time()
    job.cancel()
    x, y, st = job.result()
    assert time.time() - t0 < 10.0
    for k in range(len(S)):
        assert st[k].termination_status == A.STILL_RUNNING
        assert st[k].kkt_passes % prm.check_every == 0
        assert np.all(np.isfinite(x[k]))


def test_job_lps_retire_individually(handle):
    """An LP's result is available as soon as its CTA finishes it, while a
    slower LP of the same job is still running."""
    from coolpdlp import native, _abi as A
    from coolpdlp import generators as G
    slow = G.batch_lps(1, m_lo=300, m_hi=300, seed0=6100)
    fast = G.batch_lps(6, m_lo=40, m_hi=80, seed0=6200)
    S = _structs(slow + fast)
    prm = A.default_params_py(A.ALGO_PDLP)
    prm.max_kkt_passes = 10_000_000
    prm.time_limit = 20.0
    tol = [1e-300] + [1e-4] * len(fast)       # the first LP cannot converge
    job = native.Job(handle, S, prm, reltol=tol)
    t0 = time.time()
    seen_early = False
    while time.time() - t0 < 15.0:
        done = job.poll()
        r = job.ready()
        if r[1:].all() and not r[0]:
            seen_early = not done
            break
        time.sleep(0.01)
    assert seen_early
    for k in range(1, len(S)):
        x, y, st = job.collect_lp(k)
        assert st.termination_status == 0 and _rel(st) <= 1e-4
    with pytest.raises(A.ArgumentError):
        job.collect_lp(0)
    job.cancel()
    xs, ys, st = job.result()
    assert st[0].termination_status == A.STILL_RUNNING


def test_batch_pdhg_limits_and_errors(handle):
    from coolpdlp import native, _abi as A
    lps = _set(6, seed0=77)
    S = _structs(lps)
    prm = A.default_params_py(A.ALGO_PDHG)
    prm.termination_reltol = 1e-2
    prm.max_kkt_passes = 300
    xs, ys, st = native.batch_solve(handle, S, prm)
    for k in range(len(lps)):
        assert st[k].termination_status in (0, 2)
        assert st[k].kkt_passes <= 300 and st[k].kkt_passes % 100 == 0
        if st[k].termination_status == 0:
            assert _rel(st[k]) <= 1e-2
    bad = _structs([lps[0]])[0]
    bad.arrays[1][0] = lps[0].m + 1   # a row index outside its LP
    with pytest.raises(A.ArgumentError):
        native.batch_solve(handle, [bad], prm)
    assert native.batch_footprint(S, prm) > sum(lp.nzval.size for lp in lps) * 8
