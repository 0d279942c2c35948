"""Seeded synthetic LP generators (numpy).

The reference's own benchmark instances (Netlib via a download) are not
available, so every workload here is a seeded synthetic LP with the shapes,
sizes and value distributions of the named workload:

* ``random_sparse_lp``     -- 1,000 x 2,000, 5 nonzeros per column, N(0,1)
  values, half equality / half <= rows, x in [0,10]; feasible and bounded by
  construction (single-LP Float64 workload).
* ``powerlaw_lp``          -- 2,000,000 x 4,000,000, power-law row lengths
  (tail exponent 1.5, capped at 20,000, ~24M nonzeros), row factors
  log-uniform in [1e-3, 1e3]; the large single-LP workload.
* ``multicommodity_flow_lp`` -- K-commodity min-cost flow on a directed grid,
  +-1 incidence entries, shared arc capacities.
* ``batch_lps``            -- many random sparse LPs of uneven size.

All randomness comes from a counter-based SplitMix64 stream (Steele, Lea &
Flood 2014), so a (seed, stream, index) triple always gives the same number.
Matrices are returned in Julia's SparseMatrixCSC layout (1-based int64).
"""
from __future__ import annotations

import dataclasses

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, counters: np.ndarray) -> np.ndarray:
    """SplitMix64 output for each counter (vectorised, wraps modulo 2^64)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (counters.astype(np.uint64) + np.uint64(1)) * _GOLD
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _substream(seed: int, stream: int) -> int:
    return int(splitmix64(seed, np.array([stream], dtype=np.uint64))[0])


class Stream:
    """A named sub-stream of a seed; successive draws use fresh counters."""

    def __init__(self, seed: int, stream: int):
        self.key = _substream(seed, stream)
        self.pos = 0

    def bits(self, count: int) -> np.ndarray:
        c = np.arange(self.pos, self.pos + count, dtype=np.uint64)
        self.pos += count
        return splitmix64(self.key, c)

    def uniform(self, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """U[lo, hi) with 53 random bits."""
        u = (self.bits(count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def uniform_open0(self, count: int) -> np.ndarray:
        """U(0, 1]."""
        return ((self.bits(count) >> np.uint64(11)).astype(np.float64) + 1.0) * (
            1.0 / 9007199254740992.0)

    def normal(self, count: int) -> np.ndarray:
        """N(0,1) by Box-Muller (one output per pair of uniforms)."""
        u1 = self.uniform_open0(count)
        u2 = self.uniform_open0(count)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)

    def integers(self, count: int, lo: int, hi: int) -> np.ndarray:
        """Integers in [lo, hi) (multiply-shift, negligible bias for small ranges)."""
        span = np.uint64(hi - lo)
        b = self.bits(count) >> np.uint64(32)
        return (lo + ((b * span) >> np.uint64(32)).astype(np.int64)).astype(np.int64)


@dataclasses.dataclass
class LPData:
    """An LP in cuPDLPx form (milp.jl:1-20) with a 1-based CSC matrix."""
    m: int
    n: int
    colptr: np.ndarray   # int64, n+1, 1-based
    rowval: np.ndarray   # int64, nnz, 1-based
    nzval: np.ndarray    # float64, nnz
    c: np.ndarray
    lv: np.ndarray
    uv: np.ndarray
    lc: np.ndarray
    uc: np.ndarray
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.nzval.shape[0])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.nzval, self.rowval - 1, self.colptr - 1),
                             shape=(self.m, self.n))

    def dense(self) -> np.ndarray:
        return self.to_scipy().toarray()


def csc_from_triplets(m: int, n: int, rows: np.ndarray, cols: np.ndarray,
                      vals: np.ndarray, sum_duplicates: bool = False):
    """1-based CSC arrays from 0-based triplets (rows ascending per column)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    key = cols * np.int64(max(m, 1)) + rows
    order = np.argsort(key, kind="stable")
    key = key[order]
    rows, cols, vals = rows[order], cols[order], vals[order]
    if sum_duplicates and key.size:
        uniq, start = np.unique(key, return_index=True)
        vals = np.add.reduceat(vals, start)
        rows, cols = rows[start], cols[start]
    elif key.size and np.any(key[1:] == key[:-1]):
        raise ValueError("duplicate entries")
    counts = np.bincount(cols, minlength=n).astype(np.int64)
    colptr = np.empty(n + 1, dtype=np.int64)
    colptr[0] = 1
    np.cumsum(counts, out=colptr[1:])
    colptr[1:] += 1
    return colptr, rows + 1, vals


def _distinct_per_group(st: Stream, group_sizes: np.ndarray, universe: int) -> np.ndarray:
    """For each group g, group_sizes[g] distinct integers in [0, universe),
    concatenated.  Collisions are redrawn until none are left."""
    total = int(group_sizes.sum())
    group = np.repeat(np.arange(group_sizes.size, dtype=np.int64), group_sizes)
    vals = st.integers(total, 0, universe)
    for _ in range(64):
        key = group * np.int64(universe) + vals
        order = np.argsort(key, kind="stable")
        ks = key[order]
        dup_sorted = np.zeros(total, dtype=bool)
        dup_sorted[1:] = ks[1:] == ks[:-1]
        if not dup_sorted.any():
            return vals
        dup = np.zeros(total, dtype=bool)
        dup[order[dup_sorted]] = True
        vals[dup] = st.integers(int(dup.sum()), 0, universe)
    raise RuntimeError("could not draw distinct indices")


def _feasible_rhs(st: Stream, rows, cols, vals, m, n, n_eq, x_hi=10.0, zero_frac=0.3):
    """x* ~ U[0, x_hi] (zeros on a random subset with reduced costs s >= 0);
    b_eq = A_eq x*, b_le = A_le x* + U[0,1]; y*_eq ~ N(0,1), y*_le = -|N(0,1)|;
    c = A'y* + s."""
    xs = st.uniform(n, 0.0, x_hi)
    at_lower = st.uniform(n) < zero_frac
    xs[at_lower] = 0.0
    s = np.where(at_lower, st.uniform(n), 0.0)
    Ax = np.bincount(rows, weights=vals * xs[cols], minlength=m)
    slack = st.uniform(m)
    lc = np.full(m, -np.inf)
    uc = Ax + slack
    lc[:n_eq] = Ax[:n_eq]
    uc[:n_eq] = Ax[:n_eq]
    ys = st.normal(m)
    ys[n_eq:] = -np.abs(ys[n_eq:])
    c = np.bincount(cols, weights=vals * ys[rows], minlength=n) + s
    return c, lc, uc


def random_sparse_lp(m: int = 1000, n: int = 2000, nnz_per_col: int = 5, seed: int = 0,
                     eq_frac: float = 0.5, x_hi: float = 10.0,
                     nnz_per_col_range: tuple[int, int] | None = None) -> LPData:
    """Random sparse LP: each column holds `nnz_per_col` distinct uniform rows
    (or a per-LP count drawn from `nnz_per_col_range`), values N(0,1); the
    first eq_frac*m rows are equalities, the rest <= rows; x in [0, x_hi]."""
    st = Stream(seed, 1)
    if nnz_per_col_range is not None:
        lo, hi = nnz_per_col_range
        nnz_per_col = int(st.integers(1, lo, hi + 1)[0])
    k = min(nnz_per_col, m)
    sizes = np.full(n, k, dtype=np.int64)
    rows = _distinct_per_group(st, sizes, m)
    cols = np.repeat(np.arange(n, dtype=np.int64), k)
    vals = st.normal(rows.size)
    n_eq = int(round(eq_frac * m))
    c, lc, uc = _feasible_rhs(st, rows, cols, vals, m, n, n_eq, x_hi)
    colptr, rowval, nzval = csc_from_triplets(m, n, rows, cols, vals)
    return LPData(m, n, colptr, rowval, nzval, c, np.zeros(n), np.full(n, x_hi), lc, uc,
                  name=f"random_sparse_lp(m={m},n={n},k={k},seed={seed})")


def powerlaw_row_lengths(st: Stream, m: int, tail: float = 1.5, cap: int = 20000,
                         target_nnz: int | None = None) -> np.ndarray:
    """L_i = min(cap, ceil(X_i)), X_i ~ Pareto(tail, x_min) with x_min tuned
    (bisection on the same draws) so that sum(L) ~ target_nnz."""
    u = st.uniform_open0(m)
    base = u ** (-1.0 / tail)   # Pareto with x_min = 1
    if target_nnz is None:
        return np.minimum(cap, np.ceil(base)).astype(np.int64)
    lo, hi = 0.5, 100.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        tot = np.minimum(cap, np.ceil(mid * base)).sum()
        if tot < target_nnz:
            lo = mid
        else:
            hi = mid
    return np.minimum(cap, np.ceil(hi * base)).astype(np.int64)


def powerlaw_lp(m: int = 2_000_000, n: int = 4_000_000, target_nnz: int = 24_000_000,
                seed: int = 1, cap: int = 20000, tail: float = 1.5) -> LPData:
    """Large LP with power-law row lengths; columns uniform without replacement
    inside each row; values N(0,1) times a row factor log-uniform in
    [1e-3, 1e3]; first half of the rows are equalities."""
    st = Stream(seed, 2)
    cap = min(cap, n)
    L = powerlaw_row_lengths(st, m, tail, cap, target_nnz)
    cols = _distinct_per_group(st, L, n)
    rows = np.repeat(np.arange(m, dtype=np.int64), L)
    factor = np.exp(st.uniform(m, np.log(1e-3), np.log(1e3)))
    vals = st.normal(rows.size) * factor[rows]
    n_eq = m // 2
    c, lc, uc = _feasible_rhs(st, rows, cols, vals, m, n, n_eq, 10.0)
    colptr, rowval, nzval = csc_from_triplets(m, n, rows, cols, vals)
    return LPData(m, n, colptr, rowval, nzval, c, np.zeros(n), np.full(n, 10.0), lc, uc,
                  name=f"powerlaw_lp(m={m},n={n},nnz={rows.size},seed={seed})")


def multicommodity_flow_lp(side: int = 256, K: int = 16, seed: int = 2) -> LPData:
    """K-commodity min-cost flow on a directed side x side grid (right/down
    arcs plus their reverses).  Rows: flow conservation per node per commodity
    (equalities), then one capacity row per arc (sum_k x_ak <= u_a).  Columns:
    x_{a,k} >= 0, ordered arc-major.  Entries are exactly +-1.  Capacities
    u_a ~ U[5,40], raised where needed so that routing each commodity along an
    L-shaped path is feasible (feasible by construction)."""
    st = Stream(seed, 3)
    nodes = side * side
    idx = np.arange(nodes, dtype=np.int64).reshape(side, side)
    right_t = idx[:, :-1].ravel(); right_h = idx[:, 1:].ravel()
    down_t = idx[:-1, :].ravel(); down_h = idx[1:, :].ravel()
    tail = np.concatenate([right_t, right_h, down_t, down_h])
    head = np.concatenate([right_h, right_t, down_h, down_t])
    n_arcs = tail.size
    src = st.integers(K, 0, nodes)
    dst = st.integers(K, 0, nodes)
    for _ in range(64):
        same = src == dst
        if not same.any():
            break
        dst[same] = st.integers(int(same.sum()), 0, nodes)
    demand = st.uniform(K, 1.0, 10.0)
    cost_arc = st.uniform(n_arcs, 1.0, 10.0)
    cap = st.uniform(n_arcs, 5.0, 40.0)
    # arc lookup (tail, head) -> arc id for the L-path load
    arc_of = {}
    for a in range(n_arcs):
        arc_of[(int(tail[a]), int(head[a]))] = a
    load = np.zeros(n_arcs)
    for k in range(K):
        r0, c0 = divmod(int(src[k]), side)
        r1, c1 = divmod(int(dst[k]), side)
        r, cc = r0, c0
        while cc != c1:
            step = 1 if c1 > cc else -1
            load[arc_of[(r * side + cc, r * side + cc + step)]] += demand[k]
            cc += step
        while r != r1:
            step = 1 if r1 > r else -1
            load[arc_of[(r * side + cc, (r + step) * side + cc)]] += demand[k]
            r += step
    cap = np.maximum(cap, load)
    n = n_arcs * K
    var = np.arange(n, dtype=np.int64)
    a_of = var // K
    k_of = var % K
    # conservation rows: node*K + k ; +1 at tail (outflow), -1 at head (inflow)
    rows = np.concatenate([tail[a_of] * K + k_of, head[a_of] * K + k_of,
                           nodes * K + a_of])
    cols = np.concatenate([var, var, var])
    vals = np.concatenate([np.ones(n), -np.ones(n), np.ones(n)])
    m = nodes * K + n_arcs
    b = np.zeros(nodes * K)
    b[src * K + np.arange(K)] += demand
    b[dst * K + np.arange(K)] -= demand
    lc = np.concatenate([b, np.full(n_arcs, -np.inf)])
    uc = np.concatenate([b, cap])
    c = cost_arc[a_of]
    colptr, rowval, nzval = csc_from_triplets(m, n, rows, cols, vals)
    return LPData(m, n, colptr, rowval, nzval, c, np.zeros(n), np.full(n, np.inf), lc, uc,
                  name=f"multicommodity_flow_lp(side={side},K={K},seed={seed})")


def batch_lps(count: int = 4096, m_lo: int = 50, m_hi: int = 5000, seed0: int = 1000,
              nnz_range: tuple[int, int] = (3, 8)) -> list[LPData]:
    """`count` random sparse LPs: m log-uniform in [m_lo, m_hi], n = 2m,
    3-8 nonzeros per column, seed = seed0 + i."""
    out = []
    for i in range(count):
        st = Stream(seed0 + i, 7)
        m = int(round(np.exp(st.uniform(1, np.log(m_lo), np.log(m_hi))[0])))
        out.append(random_sparse_lp(m, 2 * m, seed=seed0 + i, nnz_per_col_range=nnz_range))
    return out


def two_variable_lp() -> LPData:
    """min 12x + 20y  s.t. 6x + 8y >= 100, 7x + 12y >= 120, x >= 0, 0 <= y <= 3
    (test/moi.jl:38-53; optimal objective 205)."""
    colptr = np.array([1, 3, 5], dtype=np.int64)
    rowval = np.array([1, 2, 1, 2], dtype=np.int64)
    nzval = np.array([6.0, 7.0, 8.0, 12.0])
    return LPData(2, 2, colptr, rowval, nzval, np.array([12.0, 20.0]), np.array([0.0, 0.0]),
                  np.array([np.inf, 3.0]), np.array([100.0, 120.0]),
                  np.array([np.inf, np.inf]), name="two_variable_lp")


def termination_check_lp() -> LPData:
    """min x1 + x2  s.t. x1 + x2 >= 1, x >= 0 (test/algorithms/all.jl, the
    'Termination check not skipped' LP; OPTIMAL)."""
    return LPData(1, 2, np.array([1, 2, 3], dtype=np.int64), np.array([1, 1], dtype=np.int64),
                  np.array([1.0, 1.0]), np.array([1.0, 1.0]), np.zeros(2),
                  np.full(2, np.inf), np.array([1.0]), np.array([np.inf]),
                  name="termination_check_lp")


def random_milp_and_sol(m: int, n: int, p: float, seed: int = 0):
    """Seeded counterpart of random_milp_and_sol (src/utils/test.jl:1-50):
    c ~ U[0,1); A = sprandn(m, n, p); bounds are, per entry, equal to a
    N(0,1) draw (25%), infinite (25%) or the draw -/+ U[0,1) (50%); x and y
    are projected N(0,1) draws."""
    st = Stream(seed, 11)
    c = st.uniform(n)
    mask = st.uniform(m * n) < p
    flat = np.nonzero(mask)[0]
    cols = flat // m
    rows = flat % m
    vals = st.normal(flat.size)
    colptr, rowval, nzval = csc_from_triplets(m, n, rows, cols, vals)

    def bounds(count):
        z = st.normal(count)
        r1 = st.uniform(count)
        r2 = st.uniform(count)
        lo = np.where(r1 < 0.25, z, np.where(r1 < 0.5, -np.inf, z - st.uniform(count)))
        hi = np.where(r2 < 0.25, z, np.where(r2 < 0.5, np.inf, z + st.uniform(count)))
        return lo, hi

    lv, uv = bounds(n)
    lc, uc = bounds(m)
    x = np.minimum(uv, np.maximum(lv, st.normal(n)))
    yraw = st.normal(m)
    y = np.where(np.isneginf(lc), np.where(np.isposinf(uc), 0.0, np.minimum(yraw, 0.0)),
                 np.where(np.isposinf(uc), np.maximum(yraw, 0.0), yraw))
    lp = LPData(m, n, colptr, rowval, nzval, c, lv, uv, lc, uc,
                name=f"random_milp(m={m},n={n},p={p},seed={seed})")
    return lp, x, y


@dataclasses.dataclass
class ServedRequest:
    rid: int
    arrival: float          # seconds from the start of the stream
    reltol: float
    kind: str               # "sparse" (m) or "flow" (side, K)
    seed: int
    m: int = 0
    side: int = 0
    K: int = 0


def served_stream(count: int, rate: float, seed: int = 7, m_lo: int = 100, m_hi: int = 20000,
                  side_lo: int = 32, side_hi: int = 128, k_lo: int = 2, k_hi: int = 8,
                  flow_frac: float = 0.2, tols=(1e-4, 1e-8)) -> list[ServedRequest]:
    """A served stream of LPs: Poisson arrivals at `rate` per second; each
    request is, with probability 1 - flow_frac, a random sparse LP (m
    log-uniform in [m_lo, m_hi], n = 2m, 5 nonzeros per column) and otherwise
    a grid multicommodity flow LP (side uniform in {side_lo..side_hi}, K uniform
    in {k_lo..k_hi}); its tolerance is drawn uniformly from `tols`.  LPs are
    built lazily by the caller through ``request_lp`` to bound memory."""
    st = Stream(seed, 21)
    gaps = -np.log(st.uniform_open0(count)) / rate
    arrivals = np.cumsum(gaps) - gaps[0]
    kind = st.uniform(count) < flow_frac
    out = []
    for i in range(count):
        s = seed * 1_000_003 + i
        tol = tols[int(st.integers(1, 0, len(tols))[0])]
        if kind[i]:
            side = int(st.integers(1, side_lo, side_hi + 1)[0])
            K = int(st.integers(1, k_lo, k_hi + 1)[0])
            out.append(ServedRequest(i, float(arrivals[i]), tol, "flow", s, side=side, K=K))
        else:
            m = int(round(np.exp(st.uniform(1, np.log(m_lo), np.log(m_hi))[0])))
            out.append(ServedRequest(i, float(arrivals[i]), tol, "sparse", s, m=m))
    return out


def request_lp(req: ServedRequest) -> LPData:
    """Builds the LP a served request names (see ``served_stream``)."""
    if req.kind == "flow":
        return multicommodity_flow_lp(side=req.side, K=req.K, seed=req.seed)
    return random_sparse_lp(req.m, 2 * req.m, 5, seed=req.seed)
