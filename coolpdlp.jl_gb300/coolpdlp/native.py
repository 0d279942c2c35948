"""Thin object layer over the C ABI: handles, problems, states, matrices."""
from __future__ import annotations

import ctypes
import sys
import threading
from ctypes import POINTER, byref, c_double, c_int32, c_int64, c_void_p

import numpy as np

from . import _abi as A

_PD = POINTER(c_double)
_P64 = POINTER(c_int64)


def _pd(a):
    return None if a is None else a.ctypes.data_as(_PD)


def _p64(a):
    return None if a is None else a.ctypes.data_as(_P64)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


class Handle:
    """cpdlp_handle on one CUDA device (one stream)."""

    def __init__(self, device: int = 0):
        self.lib = A.load_library()
        h = c_void_p()
        rc = self.lib.cpdlp_create(device, byref(h))
        if rc != A.OK:
            A.raise_for(rc, f"cpdlp_create(device={device}) failed")
        self.h = h
        self.device = device

    def check(self, rc: int, what: str = ""):
        if rc != A.OK:
            msg = self.lib.cpdlp_last_error(self.h)
            A.raise_for(rc, (what + ": " if what else "") + (msg.decode() if msg else ""))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpdlp_destroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down:
        # the process releases the device memory itself
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        self.check(self.lib.cpdlp_synchronize(self.h), "cpdlp_synchronize")

    @property
    def stream(self) -> int:
        return int(self.lib.cpdlp_stream(self.h) or 0)


_DEFAULT: dict[int, Handle] = {}
_LOCK = threading.Lock()


def default_handle(device: int = 0) -> Handle:
    """One handle per (thread, device), as the C ABI requires."""
    key = (threading.get_ident(), device)
    with _LOCK:
        h = _DEFAULT.get(key)
        if h is None:
            h = Handle(device)
            _DEFAULT[key] = h
        return h


def default_params(algorithm: int = A.ALGO_PDLP) -> A.ParamsC:
    p = A.ParamsC()
    A.load_library().cpdlp_params_default(byref(p), algorithm)
    return p


def copy_params(p: A.ParamsC) -> A.ParamsC:
    q = A.ParamsC()
    ctypes.memmove(ctypes.addressof(q), ctypes.addressof(p), ctypes.sizeof(A.ParamsC))
    return q


class LPStruct:
    """A cpdlp_lp pointing at numpy arrays that it keeps alive."""

    def __init__(self, m, n, colptr, rowval, nzval, c, lv, uv, lc, uc):
        self.arrays = [i64(colptr), i64(rowval), f64(nzval), f64(c), f64(lv), f64(uv), f64(lc),
                       f64(uc)]
        cp, rv, nz, cc, lvv, uvv, lcc, ucc = self.arrays
        self.s = A.LPC(int(m), int(n), int(nz.size), _p64(cp), _p64(rv), _pd(nz), _pd(cc),
                       _pd(lvv), _pd(uvv), _pd(lcc), _pd(ucc))


class Problem:
    """cpdlp_problem: the preprocessed LP resident on the device."""

    def __init__(self, handle: Handle, lp: LPStruct, params: A.ParamsC):
        self.handle = handle
        self.m, self.n = lp.s.m, lp.s.n
        p = c_void_p()
        handle.check(handle.lib.cpdlp_problem_create(handle.h, byref(lp.s), byref(params),
                                                     byref(p)), "cpdlp_problem_create")
        self.p = p

    def layout(self) -> dict:
        """cpdlp_problem_layout: format, CSR tile size and ELL width of the
        products over the rows of A ("A") and of A' ("At")."""
        fmt = (c_int32 * 2)()
        tile = (c_int32 * 2)()
        width = (c_int64 * 2)()
        self.handle.check(self.handle.lib.cpdlp_problem_layout(self.p, fmt, tile, width))
        names = {A.FMT_CSR: "CSR", A.FMT_ELL: "ELL"}
        return {side: {"format": names.get(fmt[k], str(fmt[k])), "tile_nnz": int(tile[k]),
                       "ell_width": int(width[k])} for k, side in enumerate(("A", "At"))}

    def order(self):
        """cpdlp_problem_order: None when the solve runs in the caller's order,
        else the 0-based (order_row, order_col) of the density order
        (internal row i is the caller's row order_row[i])."""
        flag = c_int32(0)
        orow = np.empty(max(self.m, 1), dtype=np.int64)
        ocol = np.empty(max(self.n, 1), dtype=np.int64)
        self.handle.check(self.handle.lib.cpdlp_problem_order(self.handle.h, self.p, byref(flag),
                                                              _p64(orow), _p64(ocol)),
                          "cpdlp_problem_order")
        if not flag.value:
            return None
        return orow[:self.m] - 1, ocol[:self.n] - 1

    def scaling(self):
        d1 = np.empty(self.m)
        d2 = np.empty(self.n)
        self.handle.check(self.handle.lib.cpdlp_problem_scaling(self.handle.h, self.p, _pd(d1),
                                                                _pd(d2)))
        return d1, d2

    def spectral_norm(self, params: A.ParamsC):
        v = c_double()
        it = c_int64()
        self.handle.check(self.handle.lib.cpdlp_problem_spectral_norm(
            self.handle.h, self.p, byref(params), byref(v), byref(it)))
        return v.value, it.value

    def close(self):
        if getattr(self, "p", None):
            self.handle.lib.cpdlp_problem_destroy(self.p)
            self.p = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down:
        # the process releases the device memory itself
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class State:
    """cpdlp_state: iterates, step sizes and counters of one solve."""

    def __init__(self, problem: Problem, params: A.ParamsC, x0=None, y0=None):
        self.problem = problem
        self.handle = problem.handle
        self.m, self.n = problem.m, problem.n
        s = c_void_p()
        x0 = None if x0 is None else f64(x0)
        y0 = None if y0 is None else f64(y0)
        self.handle.check(self.handle.lib.cpdlp_state_create(
            self.handle.h, problem.p, byref(params), _pd(x0), _pd(y0), byref(s)),
            "cpdlp_state_create")
        self.s = s

    def solve(self) -> A.StatsC:
        st = A.StatsC()
        self.handle.check(self.handle.lib.cpdlp_state_solve(self.handle.h, self.s, byref(st)),
                          "cpdlp_state_solve")
        return st

    def solve_blocks(self, max_blocks: int) -> A.StatsC:
        st = A.StatsC()
        self.handle.check(self.handle.lib.cpdlp_state_solve_blocks(
            self.handle.h, self.s, int(max_blocks), byref(st)), "cpdlp_state_solve_blocks")
        return st

    def profile(self, reps: int = 20):
        ms = np.zeros(3)
        self.handle.check(self.handle.lib.cpdlp_state_profile(self.handle.h, self.s, int(reps),
                                                              _pd(ms)), "cpdlp_state_profile")
        return ms

    def kernel_bytes(self):
        b = np.zeros(3)
        self.handle.lib.cpdlp_state_kernel_bytes(self.s, _pd(b))
        return b

    def step(self, count: int):
        self.handle.check(self.handle.lib.cpdlp_state_step(self.handle.h, self.s, int(count)),
                          "cpdlp_state_step")

    def kkt(self, which: int = A.VEC_SOL) -> A.KKTErrorsC:
        e = A.KKTErrorsC()
        self.handle.check(self.handle.lib.cpdlp_state_kkt(self.handle.h, self.s, which, byref(e)))
        return e

    def vectors(self, which: int = A.VEC_SOL):
        x = np.empty(self.n)
        y = np.empty(self.m)
        self.handle.check(self.handle.lib.cpdlp_state_vectors(self.handle.h, self.s, which,
                                                              _pd(x), _pd(y)))
        return x, y

    def solution(self):
        x = np.empty(self.n)
        y = np.empty(self.m)
        self.handle.check(self.handle.lib.cpdlp_state_solution(self.handle.h, self.s, _pd(x),
                                                               _pd(y)))
        return x, y

    def stats(self) -> A.StatsC:
        st = A.StatsC()
        self.handle.check(self.handle.lib.cpdlp_state_stats(self.handle.h, self.s, byref(st)))
        return st

    def history(self):
        cnt = c_int64()
        self.handle.lib.cpdlp_state_history(self.s, None, None, 0, byref(cnt))
        k = cnt.value
        passes = np.empty(max(k, 1), dtype=np.int64)
        errs = (A.KKTErrorsC * max(k, 1))()
        self.handle.lib.cpdlp_state_history(self.s, _p64(passes), errs, k, byref(cnt))
        return [(int(passes[i]), errs[i]) for i in range(k)]

    def close(self):
        if getattr(self, "s", None):
            self.handle.lib.cpdlp_state_destroy(self.s)
            self.s = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down:
        # the process releases the device memory itself
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def solve_lp(handle: Handle, lp: LPStruct, params: A.ParamsC, x0=None, y0=None):
    """cpdlp_solve: returns (x, y, StatsC) in the original units."""
    m, n = lp.s.m, lp.s.n
    x = np.empty(n)
    y = np.empty(m)
    st = A.StatsC()
    x0 = None if x0 is None else f64(x0)
    y0 = None if y0 is None else f64(y0)
    handle.check(handle.lib.cpdlp_solve(handle.h, byref(lp.s), byref(params), _pd(x0), _pd(y0),
                                        _pd(x), _pd(y), byref(st)), "cpdlp_solve")
    return x, y, st


def solve_history(handle: Handle):
    """cpdlp_solve_history: the error history of the last cpdlp_solve on the
    handle, as [(kkt_passes, KKTErrorsC)]."""
    cnt = c_int64()
    handle.check(handle.lib.cpdlp_solve_history(handle.h, None, None, 0, byref(cnt)))
    k = cnt.value
    passes = np.empty(max(k, 1), dtype=np.int64)
    errs = (A.KKTErrorsC * max(k, 1))()
    handle.check(handle.lib.cpdlp_solve_history(handle.h, _p64(passes), errs, k, byref(cnt)))
    return [(int(passes[i]), errs[i]) for i in range(k)]


def reduced_costs(handle: Handle, lp: LPStruct, y):
    """cpdlp_reduced_costs: (z, dual objective) of the solution y of the LP, on
    the device (moi.jl:215-227)."""
    z = np.empty(lp.s.n)
    obj = c_double()
    yy = f64(y)
    handle.check(handle.lib.cpdlp_reduced_costs(handle.h, byref(lp.s), _pd(yy), _pd(z),
                                                byref(obj)), "cpdlp_reduced_costs")
    return z, obj.value


def batch_solve(handle: Handle, lps: list, params: A.ParamsC):
    """cpdlp_batch_solve over LPStructs; returns lists of x, y and StatsC."""
    k = len(lps)
    arr = (A.LPC * max(k, 1))(*[lp.s for lp in lps])
    xs = [np.empty(lp.s.n) for lp in lps]
    ys = [np.empty(lp.s.m) for lp in lps]
    xp = (_PD * max(k, 1))(*[_pd(x) for x in xs])
    yp = (_PD * max(k, 1))(*[_pd(y) for y in ys])
    st = (A.StatsC * max(k, 1))()
    handle.check(handle.lib.cpdlp_batch_solve(handle.h, k, arr, byref(params), xp, yp, st),
                 "cpdlp_batch_solve")
    return xs, ys, [st[i] for i in range(k)]


class Job:
    """An asynchronous batch (cpdlp_submit): the LPs are copied, preprocessed
    on the job's own stream and solved by a persistent kernel while the
    caller continues.  poll() never blocks; result() waits and collects."""

    def __init__(self, handle: Handle, lps: list, params: A.ParamsC, reltol=None,
                 x0=None, y0=None, max_ctas: int = 0):
        self.handle = handle
        self.j = None
        self.k = len(lps)
        self.shapes = [(lp.s.m, lp.s.n) for lp in lps]
        arr = (A.LPC * max(self.k, 1))(*[lp.s for lp in lps])
        rt = None if reltol is None else f64(np.broadcast_to(np.asarray(reltol, dtype=np.float64),
                                                             (self.k,)).copy())
        self._keep = [rt]
        x0p = y0p = None
        if x0 is not None:
            xs = [None if v is None else f64(v) for v in x0]
            self._keep.append(xs)
            x0p = (_PD * max(self.k, 1))(*[_pd(v) for v in xs])
        if y0 is not None:
            ys = [None if v is None else f64(v) for v in y0]
            self._keep.append(ys)
            y0p = (_PD * max(self.k, 1))(*[_pd(v) for v in ys])
        out = c_void_p()
        handle.check(handle.lib.cpdlp_submit(handle.h, self.k, arr, byref(params), _pd(rt),
                                             x0p, y0p, int(max_ctas), byref(out)),
                     "cpdlp_submit")
        self.j = out.value
        self._keep = None

    def poll(self) -> bool:
        done = c_int32()
        self.handle.check(self.handle.lib.cpdlp_poll(self.handle.h, self.j, byref(done)),
                          "cpdlp_poll")
        return bool(done.value)

    def wait(self):
        self.handle.check(self.handle.lib.cpdlp_wait(self.handle.h, self.j), "cpdlp_wait")

    def cancel(self):
        self.handle.check(self.handle.lib.cpdlp_cancel(self.handle.h, self.j), "cpdlp_cancel")

    def result(self):
        """waits, then returns lists of x, y and StatsC (original units)"""
        self.wait()
        xs = [np.empty(n) for (_, n) in self.shapes]
        ys = [np.empty(m) for (m, _) in self.shapes]
        xp = (_PD * max(self.k, 1))(*[_pd(x) for x in xs])
        yp = (_PD * max(self.k, 1))(*[_pd(y) for y in ys])
        st = (A.StatsC * max(self.k, 1))()
        self.handle.check(self.handle.lib.cpdlp_collect(self.handle.h, self.j, xp, yp, st),
                          "cpdlp_collect")
        return xs, ys, [st[i] for i in range(self.k)]

    def ready(self) -> np.ndarray:
        """per LP: finished as of the last poll()"""
        r = np.zeros(max(self.k, 1), dtype=np.int32)
        self.handle.check(self.handle.lib.cpdlp_job_ready(
            self.handle.h, self.j, r.ctypes.data_as(POINTER(c_int32))), "cpdlp_job_ready")
        return r[:self.k].astype(bool)

    def collect_lp(self, k: int):
        """x, y, StatsC of finished LP k"""
        m, n = self.shapes[k]
        x, y, st = np.empty(n), np.empty(m), A.StatsC()
        self.handle.check(self.handle.lib.cpdlp_collect_lp(self.handle.h, self.j, int(k), _pd(x),
                                                           _pd(y), byref(st)), "cpdlp_collect_lp")
        return x, y, st

    def close(self):
        if getattr(self, "j", None):
            self.handle.lib.cpdlp_job_destroy(self.j)
            self.j = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down:
        # the process releases the device memory itself
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def batch_footprint(lps: list, params: A.ParamsC) -> int:
    """Upper bound of the device bytes a job over these LPs holds."""
    lib = A.load_library()
    k = len(lps)
    arr = (A.LPC * max(k, 1))(*[lp.s for lp in lps])
    return int(lib.cpdlp_batch_footprint(k, arr, byref(params)))
