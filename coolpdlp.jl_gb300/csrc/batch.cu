// batch.cu -- many independent LPs in one persistent launch.
//
// The LPs of a job are concatenated block-diagonally on the host and
// preprocessed once by the single-LP device pipeline: Ruiz and Pock-Chambolle
// scaling work on rows and columns, so the scaling of the concatenation equals
// the scaling of each LP.  The tile partitions are rebuilt so that no tile
// crosses an LP boundary.  One CTA solves one LP at a time and takes the next
// LP from an atomic counter over a largest-first order when it finishes: power
// method (linalg.jl:86-96), primal weight (step_size.jl:29-40), then blocks of
// check_every fused PDHG steps (pdlp.jl:96-136) with the four-iterate KKT
// check, restart and termination logic (pdlp.jl:138-196, restart.jl:40-57,
// termination.jl:89-101) run by the CTA itself, thread 0 taking the FP64
// decisions.  Every loop is bounded by the LP's pass limit and time limit; no
// CTA waits on another.
//
// An LP's arithmetic depends only on the LP and the tile size (its tiles, the
// thread that owns each row, the order of every sum), never on the other LPs
// of the job or on which CTA runs it, so an LP gives the same result alone and
// in any mix.
//
// The per-LP semantics are those of solve(milp, algo) (common.jl:186-209)
// except that no error history is recorded.  With FP32 iterates, LPs whose
// target tolerance is below the FP32 phase's tolerance continue in a second,
// FP64 job phase warm-started from the FP32 solution (the refinement of
// cpdlp_solve, batched).
#include <algorithm>
#include <memory>
#include <numeric>
#include <thread>
#include <type_traits>

#include <cooperative_groups.h>

#include "batch.cuh"
#include "epilogues.cuh"
#include "solver.cuh"

namespace cpdlp {

namespace {

namespace cg = cooperative_groups;

constexpr int BW = TILE_WARPS;  // warps per CTA
constexpr int BT = BW * 32;
constexpr int BATCH_ITEMS = 4;  // default nonzeros per lane of a short tile (128-nonzero tiles)
constexpr int BATCH_RPL = 1;    // rows per lane: short tiles of at most 32 rows
// LPs with at least CLUSTER_MIN_NNZ nonzeros are solved by a thread-block
// cluster of CLUSTER_CTAS CTAs instead of one CTA
constexpr int CLUSTER_CTAS = 8;
// (build-time knob; 12,000 measured best on the 4,096-LP batch: 2.16 s against
// 2.38 s with 24,000)
#ifndef CPDLP_CLUSTER_MIN_NNZ
#define CPDLP_CLUSTER_MIN_NNZ 12000
#endif
constexpr int64_t CLUSTER_MIN_NNZ = CPDLP_CLUSTER_MIN_NNZ;
// In the FP64 phase (few LPs, the tail of a job) the threshold is lower: a
// single CTA takes seconds on the slowest stalled LPs while most SMs are idle
// (a 3,792-nonzero LP needing 30,000 FP64 passes set the 4,096-LP batch's
// makespan at 4,000)
#ifndef CPDLP_PHASE_CLUSTER_MIN_NNZ
#define CPDLP_PHASE_CLUSTER_MIN_NNZ 1000
#endif
constexpr int64_t PHASE_CLUSTER_MIN_NNZ = CPDLP_PHASE_CLUSTER_MIN_NNZ;
// an LP's FP32 run stalls when its relative KKT error has not halved over this
// many checks; it then continues in FP64
#ifndef CPDLP_BATCH_STALL_CHECKS
#define CPDLP_BATCH_STALL_CHECKS 30
#endif
constexpr int64_t BATCH_STALL_CHECKS = CPDLP_BATCH_STALL_CHECKS;

// resident CTAs per SM the solve kernel is compiled for (registers = 65536 /
// (256 threads x this)).  Each CTA's solve is a latency-bound chain of
// dependent half-steps, so more resident CTAs beat fewer spills: with 4
// (64 registers, some spilled to L1) the 4,096-LP FP32 batch takes 2.3 s
// against 3.0 s with 2 (128 registers, no spills).
#ifndef CPDLP_BATCH_MINB_F32
#define CPDLP_BATCH_MINB_F32 4
#endif
#ifndef CPDLP_BATCH_MINB_F64
#define CPDLP_BATCH_MINB_F64 4
#endif
template <class T>
constexpr int batch_min_blocks() {
    return std::is_same<T, float>::value ? CPDLP_BATCH_MINB_F32 : CPDLP_BATCH_MINB_F64;
}

struct BatchLP {
    int32_t m, n, row_off, col_off;
    int32_t a_t0, a_t1, a_l0, a_l1;
    int32_t at_t0, at_t1, at_l0, at_l1;
    int32_t a_lid0, a_lid1, at_lid0, at_lid1;
    int32_t zero_cost, warm;
    double power_tol, power_rtol, reltol, time_limit;
    int64_t power_maxiter, max_passes;
    int64_t stall_passes;  // > 0: stop when the error has not halved for this many passes
    double theta0;         // >= 0: |A|^2 estimate carried over (the power method is skipped)
    double omega0;         // > 0: primal weight carried over
};

struct BatchResult {
    cpdlp_kkt_errors err;
    int64_t kkt_passes, outer, inner, total, power_iterations;
    double eta, omega, eta_sum, time_elapsed;
    int32_t status, restart_from_avg, stalled, pad;
    double theta;
};

struct BatchParams {
    int32_t algorithm, check_every;
    double invnorm_scaling, primal_weight_damping, zero_tol;
    double sufficient_decay, necessary_decay, artificial_decay;
};

template <class T>
struct BatchArgs {
    CsrView<T, T> A, At;
    const T *c, *lv, *uv, *lc, *uc;
    const double *invD1, *invD2, *D1, *D2;
    const T *invD1t, *invD2t;   // 1 ./ D1, 1 ./ D2 in T (the KKT terms)
    T *x[2], *y[2], *xa[2], *ya[2], *xr, *yr, *xbar;
    const double* theta;     // per LP: the power method's estimate of |A|^2
    const int64_t* power_iters;
    const double* x_init;    // warm starts (original units) or null
    const double* y_init;
    const BatchLP* lps;
    const int32_t* order;    // queue order of the LPs
    // results, in mapped host memory: each LP's result and solution are
    // visible to the host once its done flag is set
    BatchResult* res;
    double* out_x;
    double* out_y;
    int* done;
    double* longA;    // row-side long-row terms (2 per long row of A)
    double* longAt;   // column-side long-row terms (3 per long row of A')
    int* next;
    const int* cancel;
    int32_t count;
    BatchParams prm;
};

// The power method of every LP, in FP64 arithmetic over the matrix values as
// stored (V = float or double: the product of the stored values and FP64
// vectors is exact before rounding), so that FP32 iterates step with an
// estimate of |A|^2 as accurate as the FP64 path's.
template <class V>
struct PowerArgs {
    CsrView<V, double> A, At;
    double *x, *Atx, *s;     // x (n), A'Ax (n), Ax (m)
    const double* x_start;   // power-method start vectors
    const BatchLP* lps;
    const int32_t* order;
    double* theta;
    int64_t* iters;
    double* longAt;
    int* next;
    int32_t count;
};

// per-CTA control state of the LP in progress (shared memory; thread 0 writes
// the decisions, every thread reads them after a barrier)
struct BatchCtl {
    BatchLP L;
    cpdlp_kkt_errors e[4], e_cand, e_restart, e_sol;
    double omega, pscale, dscale;
    uint64_t t_start;
    int64_t passes, outer, inner, total, power_it;
    double best_rel;       // smallest relative error at a halving mark
    int64_t mark;          // passes at that mark
    double eta_sum;        // the averaging weight sum (thread 0)
    double kd[2][5];       // step coefficients of this step and the next, rounded to T
    int32_t lp, status, flag, from_avg, restart_valid, cancelled, stop, stalled, tl_hit;
};

// -- the CTA group that solves one LP ------------------------------------------
// One CTA (CS = 1) or a thread-block cluster of CS CTAs on as many SMs, joined
// by the hardware cluster barrier and distributed shared memory.  Every branch
// that encloses a group barrier depends only on values that are identical in
// all CTAs of the group: the LP's descriptor, group sums (computed in the same
// order by every CTA), and the few clock- or flag-derived values that rank 0
// reads and the other CTAs copy from it.
template <int CS>
struct Grp {
    static __device__ __forceinline__ void sync() {
        if constexpr (CS == 1) __syncthreads();
        else cg::this_cluster().sync();
    }
    static __device__ __forceinline__ int rank() {
        if constexpr (CS == 1) return 0;
        else return (int)cg::this_cluster().block_rank();
    }
    // the copy of the shared variable *p held by CTA r of the group
    template <class P>
    static __device__ __forceinline__ P* at(P* p, int r) {
        if constexpr (CS == 1) return p;
        else return cg::this_cluster().map_shared_rank(p, r);
    }
};

// Sums Q per-thread values over the group in a fixed order (warp trees, the
// warps of each CTA in order, then the CTAs in rank order); every thread of
// every CTA receives the same sums.  sh: BW*Q + Q doubles of shared memory.
template <int Q, int CS>
__device__ __forceinline__ void grp_sum(double (&v)[Q], double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[w * Q + q] = x;
    }
    __syncthreads();
    if (threadIdx.x < Q) {
        double s = 0.0;
        for (int ww = 0; ww < BW; ww++) s += sh[ww * Q + threadIdx.x];
        sh[BW * Q + threadIdx.x] = s;
    }
    Grp<CS>::sync();
#pragma unroll
    for (int q = 0; q < Q; q++) {
        double s = Grp<CS>::at(sh, 0)[BW * Q + q];
        for (int r = 1; r < CS; r++) s += Grp<CS>::at(sh, r)[BW * Q + q];
        v[q] = s;
    }
    Grp<CS>::sync();
}

// the LP's tiles of one matrix, the group's warps striding over its tasks; the
// vectors are gathered with coherent loads (this kernel rewrites them between
// products)
template <int ITEMS, int CS, class V, class T, class Epi>
__device__ __forceinline__ void lp_tiles(const CsrView<V, T>& A, int t0, int t1, int l0, int l1,
                                         const T* xin, Epi& epi, typename Epi::Acc& acc,
                                         T* prod) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = Grp<CS>::rank() * BW + w;
    const VecSet<T, 1, true> xs{{xin}};
    for (int t = l0 + gw; t < l1; t += BW * CS) long_piece<ITEMS, 1>(A, xs, epi, acc, A.ltasks[t], lane);
    for (int t = t0 + gw; t < t1; t += BW * CS) {
        const int4 tk = A.tasks[t];
        short_tile<ITEMS, 1, V, T, Epi, true, BATCH_RPL, true>(A, xs, epi, acc, tk.x, tk.y, tk.z, tk.w,
                                                       lane, prod + w * tile_buf<ITEMS>());
    }
}

__device__ __forceinline__ double rel_err(const cpdlp_kkt_errors& e) {
    return jl_max(jl_max(e.primal / e.primal_scale, e.dual / e.dual_scale), e.gap / e.gap_scale);
}
__device__ __forceinline__ double abs_err(const cpdlp_kkt_errors& e, double w) {
    return sqrt((w * w) * (e.primal * e.primal) + (1.0 / (w * w)) * (e.dual * e.dual) +
                e.gap * e.gap);
}
__device__ __forceinline__ bool should_restart(const BatchParams& p, double ac, double ar,
                                               double acl, int64_t inner, int64_t total) {
    return (ac <= p.sufficient_decay * ar) || ((ac <= p.necessary_decay * ar) && (ac > acl)) ||
           ((double)inner >= p.artificial_decay * (double)total);
}

// step coefficients (pdlp.jl:108-117, averaging :126-136): tau = eta/omega,
// sigma = eta*omega, 1/sigma, and the averaging weights eta/(eta+S), S/(eta+S)
template <class T>
__device__ __forceinline__ void fill_coef(BatchCtl& C, int slot, double eta, double omega,
                                          double es) {
    const double sigma = eta * omega;
    C.kd[slot][0] = (double)(T)(eta / omega);
    C.kd[slot][1] = (double)(T)sigma;
    C.kd[slot][2] = (double)(T)(1.0 / sigma);
    C.kd[slot][3] = (double)(T)(eta / (eta + es));
    C.kd[slot][4] = (double)(T)(es / (eta + es));
}

// KKT errors of (xv, yv) (errors.jl:65-109) into *out (thread 0 of every CTA,
// identical values); the whole group takes part; ends with a group barrier
template <int ITEMS, int CS, class T>
__device__ __forceinline__ void lp_kkt(const BatchArgs<T>& g, const BatchCtl& C, const T* xv,
                                       const T* yv, cpdlp_kkt_errors* out, T* prod, double* sh) {
    const BatchLP& L = C.L;
    double rs[2], cs[3];
    {
        KktRowEpi<T, 1> re;
        re.lc = g.lc; re.uc = g.uc; re.invD1 = g.invD1t; re.y[0] = yv;
        re.block_out = nullptr; re.long_out = g.longA;
        typename KktRowEpi<T, 1>::Acc a;
        re.init(a);
        lp_tiles<ITEMS, CS>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, xv, re, a, prod);
        grp_sum<2, CS>(a.v, sh);
        rs[0] = a.v[0]; rs[1] = a.v[1];
    }
    {
        KktColEpi<T, 1> ce;
        ce.c = g.c; ce.lv = g.lv; ce.uv = g.uv; ce.invD2 = g.invD2t; ce.x[0] = xv;
        ce.block_out = nullptr; ce.long_out = g.longAt;
        typename KktColEpi<T, 1>::Acc a;
        ce.init(a);
        lp_tiles<ITEMS, CS>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, yv, ce, a, prod);
        grp_sum<3, CS>(a.v, sh);
        cs[0] = a.v[0]; cs[1] = a.v[1]; cs[2] = a.v[2];
    }
    if (threadIdx.x == 0) {
        for (int l = L.a_lid0; l < L.a_lid1; l++) {
            rs[0] += g.longA[(size_t)l * 2];
            rs[1] += g.longA[(size_t)l * 2 + 1];
        }
        for (int l = L.at_lid0; l < L.at_lid1; l++) {
            cs[0] += g.longAt[(size_t)l * 3];
            cs[1] += g.longAt[(size_t)l * 3 + 1];
            cs[2] += g.longAt[(size_t)l * 3 + 2];
        }
        out->primal = sqrt(rs[0]);
        out->primal_scale = C.pscale;
        out->dual = sqrt(cs[0]);
        out->dual_scale = C.dscale;
        out->gap = fabs((cs[2] + rs[1]) + cs[1]);
        out->gap_scale = (1.0 + fabs(rs[1] + cs[1])) + fabs(cs[2]);
    }
    Grp<CS>::sync();  // the long-row terms are rewritten by the next pass
}

// solve(milp, algo) for the LP in C.  Every CTA of the group keeps its own copy
// of C and updates it identically; rank 0 alone reads the clock and the cancel
// flag and the others copy those two values from it.
template <int ITEMS, class T, int CS>
__device__ __forceinline__ void solve_one(const BatchArgs<T>& g, BatchCtl& C, T* prod,
                                          double* sh) {
    const int tid = threadIdx.x;
    const int rank = Grp<CS>::rank();
    const int gt = rank * BT + tid;  // thread index in the group
    constexpr int GT = BT * CS;      // threads in the group
    const bool pdlp = g.prm.algorithm == CPDLP_ALGO_PDLP;
    const int c0 = C.L.col_off, c1 = c0 + C.L.n, r0 = C.L.row_off, r1 = r0 + C.L.m;
    // ---- step size from the power method's estimate (step_size.jl:22-27),
    // scales and primal weight (step_size.jl:29-40, errors.jl:79-85)
    const double eta = g.prm.invnorm_scaling * (1.0 / sqrt(g.theta[C.lp]));
    double omega;
    {
        double q[4] = {0, 0, 0, 0};
        for (int i = r0 + gt; i < r1; i += GT) {
            const double cb = combine((double)g.lc[i], (double)g.uc[i]);
            const double sv = g.invD1[i] * cb;
            q[0] += sv * sv;
            q[1] += cb * cb;
        }
        for (int j = c0 + gt; j < c1; j += GT) {
            const double cj = (double)g.c[j];
            const double sv = g.invD2[j] * cj;
            q[2] += sv * sv;
            q[3] += cj * cj;
        }
        grp_sum<4, CS>(q, sh);
        const double cn = sqrt(q[3]), bn = sqrt(q[1]);
        omega = !pdlp ? 1.0 : (cn > g.prm.zero_tol && bn > g.prm.zero_tol) ? cn / bn : 1.0;
        if (pdlp && C.L.omega0 > 0) omega = C.L.omega0;
        if (tid == 0) {
            C.pscale = 1.0 + sqrt(q[0]);
            C.dscale = 1.0 + sqrt(q[2]);
            C.power_it = g.power_iters[C.lp];
        }
    }
    // ---- initial iterates: sol = precondition(sol_init) (preconditioning.jl:45-51),
    // sol_last = 0, avg = sol, avg_last = 0, restart = sol (pdlp.jl:45-67)
    for (int j = c0 + gt; j < c1; j += GT) {
        const T v = (C.L.warm && g.x_init) ? (T)__ddiv_rn(g.x_init[j], g.D2[j]) : T(0);
        g.x[0][j] = v; g.x[1][j] = T(0); g.xa[0][j] = v; g.xa[1][j] = T(0);
        g.xr[j] = v; g.xbar[j] = T(0);
    }
    for (int i = r0 + gt; i < r1; i += GT) {
        const T v = (C.L.warm && g.y_init) ? (T)__ddiv_rn(g.y_init[i], g.D1[i]) : T(0);
        g.y[0][i] = v; g.y[1][i] = T(0); g.ya[0][i] = v; g.ya[1][i] = T(0);
        g.yr[i] = v;
    }
    int cur = 0;
    if (tid == 0) {
        C.passes = C.outer = C.inner = C.total = 0;
        C.best_rel = INFINITY;
        C.mark = 0;
        C.stalled = 0;
        C.restart_valid = 0;
        C.from_avg = 0;
        C.status = CPDLP_STILL_RUNNING;
        C.stop = 0;
        C.omega = omega;
        C.eta_sum = 0.0;
        fill_coef<T>(C, 0, eta, omega, 0.0);
    }
    Grp<CS>::sync();
    int stepc = 0;  // steps taken (the coefficient slot of the next step is stepc & 1)
    if (C.L.m == 0 && C.L.zero_cost) {  // early exit (common.jl:194-198)
        for (int j = c0 + gt; j < c1; j += GT) g.x[0][j] = proj_box(T(0), g.lv[j], g.uv[j]);
        if (tid == 0) {
            C.status = CPDLP_OPTIMAL;
            C.stop = 1;
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            C.e_sol = cpdlp_kkt_errors{nan, nan, nan, nan, nan, nan};
        }
        Grp<CS>::sync();
    }
    const double tlim_ns = C.L.time_limit * 1e9;
    while (!C.stop) {
        // ---- check_every steps (pdlp.jl:96-124, averaging :126-136)
        for (int st = 0; st < g.prm.check_every; st++) {
            // coefficients computed by thread 0 one step ahead (FP64 division is
            // slow, so not every thread does it); the slot of the next step was
            // last read two barriers ago
            const int sl = stepc & 1;
            StepCoef<T> k;
            k.tau = (T)C.kd[sl][0];
            k.sigma = (T)C.kd[sl][1];
            k.inv_sigma = (T)C.kd[sl][2];
            k.a = (T)C.kd[sl][3];
            k.b = (T)C.kd[sl][4];
            if (tid == 0) {
                if (pdlp) C.eta_sum += eta;
                fill_coef<T>(C, sl ^ 1, eta, C.omega, C.eta_sum);
            }
            const int o = cur, nw = cur ^ 1;
            {
                PrimalEpi<T, true> pe{g.x[o], g.c, g.lv, g.uv, g.x[nw], g.xbar, g.xa[o], g.xa[nw],
                                      {k}, pdlp ? 1 : 0};
                NoAcc a;
                lp_tiles<ITEMS, CS>(g.At, C.L.at_t0, C.L.at_t1, C.L.at_l0, C.L.at_l1, g.y[o], pe, a, prod);
            }
            Grp<CS>::sync();
            {
                DualEpi<T, true> de{g.y[o], g.lc, g.uc, g.y[nw], g.ya[o], g.ya[nw], {k}, pdlp ? 1 : 0};
                NoAcc a;
                lp_tiles<ITEMS, CS>(g.A, C.L.a_t0, C.L.a_t1, C.L.a_l0, C.L.a_l1, g.xbar, de, a, prod);
            }
            Grp<CS>::sync();
            cur ^= 1;
            stepc++;
        }
        // ---- KKT errors of sol, avg, sol_last, avg_last (errors.jl:65-109)
        const int nv = pdlp ? 4 : 1;
        for (int p = 0; p < nv; p++) {
            const T* xv = p == 0 ? g.x[cur] : p == 1 ? g.xa[cur] : p == 2 ? g.x[cur ^ 1] : g.xa[cur ^ 1];
            const T* yv = p == 0 ? g.y[cur] : p == 1 ? g.ya[cur] : p == 2 ? g.y[cur ^ 1] : g.ya[cur ^ 1];
            lp_kkt<ITEMS, CS, T>(g, C, xv, yv, &C.e[p], prod, sh);
        }
        // ---- the clock and the cancel flag, read once for the group by rank 0
        if (rank == 0 && tid == 0) {
            C.tl_hit = (double)(global_ns() - C.t_start) >= tlim_ns ? 1 : 0;
            C.cancelled = *(volatile const int*)g.cancel;
        }
        if constexpr (CS > 1) {
            Grp<CS>::sync();
            if (rank != 0 && tid == 0) {
                const BatchCtl* c0p = Grp<CS>::at(&C, 0);
                C.tl_hit = c0p->tl_hit;
                C.cancelled = c0p->cancelled;
            }
        }
        // ---- termination (common.jl:218-231) and restart decision (pdlp.jl:138-170)
        if (tid == 0) {
            C.passes += g.prm.check_every;
            if (pdlp) {
                C.inner += g.prm.check_every;
                C.total += g.prm.check_every;
            }
            C.e_sol = C.e[0];
            int32_t stt = CPDLP_STILL_RUNNING;
            if (rel_err(C.e_sol) <= C.L.reltol) stt = CPDLP_OPTIMAL;
            else if (C.tl_hit) stt = CPDLP_TIME_LIMIT;
            else if (C.passes >= C.L.max_passes) stt = CPDLP_ITERATION_LIMIT;
            // stall: the relative error has not halved over stall_passes passes
            const double rel = rel_err(C.e_sol);
            if (rel < 0.5 * C.best_rel) {
                C.best_rel = rel;
                C.mark = C.passes;
            } else if (stt == CPDLP_STILL_RUNNING && C.L.stall_passes > 0 &&
                       C.passes - C.mark >= C.L.stall_passes) {
                stt = CPDLP_ITERATION_LIMIT;
                C.stalled = 1;
            }
            const int cancelled = C.cancelled;
            int flag = 0;
            if (stt == CPDLP_STILL_RUNNING && !cancelled && pdlp) {
                const double w = C.omega;
                if (abs_err(C.e[0], w) < abs_err(C.e[1], w)) { C.from_avg = 0; C.e_cand = C.e[0]; }
                else { C.from_avg = 1; C.e_cand = C.e[1]; }
                C.e[2] = (abs_err(C.e[2], w) < abs_err(C.e[3], w)) ? C.e[2] : C.e[3];
                flag = 2;  // the restart point's errors are needed first
                if (C.restart_valid)
                    flag = should_restart(g.prm, abs_err(C.e_cand, w), abs_err(C.e_restart, w),
                                          abs_err(C.e[2], w), C.inner, C.total) ? 3 : 0;
            }
            C.status = stt;
            C.stop = (stt != CPDLP_STILL_RUNNING) || cancelled;
            C.flag = flag;
        }
        __syncthreads();
        int flag = C.flag;
        __syncthreads();
        if (flag == 2) {
            // errors of the initial restart point (sol_restart = the start)
            lp_kkt<ITEMS, CS, T>(g, C, g.xr, g.yr, &C.e_restart, prod, sh);
            if (tid == 0) {
                C.restart_valid = 1;
                const double w = C.omega;
                C.flag = should_restart(g.prm, abs_err(C.e_cand, w), abs_err(C.e_restart, w),
                                        abs_err(C.e[2], w), C.inner, C.total) ? 3 : 0;
            }
            __syncthreads();
            flag = C.flag;
            __syncthreads();
        }
        if (flag == 3) {
            // restart! + primal_weight_update! (pdlp.jl:172-196, step_size.jl:58-75)
            const T* cx = C.from_avg ? g.xa[cur] : g.x[cur];
            const T* cy = C.from_avg ? g.ya[cur] : g.y[cur];
            double q[2] = {0.0, 0.0};
            for (int j = c0 + gt; j < c1; j += GT) {
                const double d = (double)cx[j] - (double)g.xr[j];
                q[0] += d * d;
            }
            for (int i = r0 + gt; i < r1; i += GT) {
                const double d = (double)cy[i] - (double)g.yr[i];
                q[1] += d * d;
            }
            grp_sum<2, CS>(q, sh);
            const double dx = sqrt(q[0]), dy = sqrt(q[1]), th = g.prm.primal_weight_damping;
            if (dx > g.prm.zero_tol && dy > g.prm.zero_tol)
                omega = exp(th * log(dy / dx) + (1.0 - th) * log(omega));
            for (int j = c0 + gt; j < c1; j += GT) {
                const T v = cx[j];
                g.x[cur][j] = v;
                g.xr[j] = v;
                g.xa[cur][j] = T(0);
            }
            for (int i = r0 + gt; i < r1; i += GT) {
                const T v = cy[i];
                g.y[cur][i] = v;
                g.yr[i] = v;
                g.ya[cur][i] = T(0);
            }
            if (tid == 0) {
                C.omega = omega;
                C.eta_sum = 0.0;
                fill_coef<T>(C, stepc & 1, eta, omega, 0.0);
                C.e_restart = C.e_cand;
                C.outer += 1;
                C.inner = 0;
            }
            Grp<CS>::sync();
        }
    }
    // ---- get_solution (common.jl:233-235): unscaled, double
    for (int j = c0 + gt; j < c1; j += GT) g.out_x[j] = g.D2[j] * (double)g.x[cur][j];
    for (int i = r0 + gt; i < r1; i += GT) g.out_y[i] = g.D1[i] * (double)g.y[cur][i];
    __threadfence_system();
    Grp<CS>::sync();
    if (rank == 0 && tid == 0) {
        BatchResult R;
        R.err = C.e_sol;
        R.kkt_passes = C.passes;
        R.outer = C.outer;
        R.inner = C.inner;
        R.total = C.total;
        R.power_iterations = C.power_it;
        R.eta = eta;
        R.theta = g.theta[C.lp];
        R.omega = omega;
        R.eta_sum = C.eta_sum;
        R.time_elapsed = (double)(global_ns() - C.t_start) * 1e-9;
        R.status = C.status;
        R.restart_from_avg = C.from_avg;
        R.stalled = C.stalled;
        R.pad = 0;
        g.res[C.lp] = R;
        __threadfence_system();
        *(volatile int*)(g.done + C.lp) = 1;
    }
}

// an LP dequeued after a cancellation: not started
template <class T, int CS>
__device__ __forceinline__ void skip_one(const BatchArgs<T>& g, const BatchCtl& C) {
    const int gt = Grp<CS>::rank() * BT + threadIdx.x;
    for (int j = C.L.col_off + gt; j < C.L.col_off + C.L.n; j += BT * CS) g.out_x[j] = 0.0;
    for (int i = C.L.row_off + gt; i < C.L.row_off + C.L.m; i += BT * CS) g.out_y[i] = 0.0;
    __threadfence_system();
    Grp<CS>::sync();
    if (Grp<CS>::rank() == 0 && threadIdx.x == 0) {
        BatchResult R;
        memset(&R, 0, sizeof(R));
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        R.err = cpdlp_kkt_errors{nan, nan, nan, nan, nan, nan};
        R.status = CPDLP_STILL_RUNNING;
        g.res[C.lp] = R;
        __threadfence_system();
        *(volatile int*)(g.done + C.lp) = 1;
    }
}

// powm! on A'A with IterativeSolvers' stopping rule (linalg.jl:86-96), FP64
// vectors; one group (a CTA or a cluster) per LP from a queue.  With FP32
// iterates the loop also stops once the residual is below power_rtol * theta
// (BatchLP.power_rtol > 0).
template <int ITEMS, class V, int CS>
__global__ void __launch_bounds__(BT) k_batch_power(PowerArgs<V> g) {
    __shared__ __align__(16) double prod[BW * tile_buf<ITEMS>()];
    __shared__ double sh[BW * 8 + 8];
    __shared__ BatchLP L;
    __shared__ int s_lp;
    const int tid = threadIdx.x;
    const int rank = Grp<CS>::rank();
    const int gt = rank * BT + tid;
    constexpr int GT = BT * CS;
    for (int guard = 0; guard <= g.count; guard++) {
        if (rank == 0 && tid == 0) {
            const int q = atomicAdd(g.next, 1);
            s_lp = q < g.count ? g.order[q] : -1;
        }
        if constexpr (CS > 1) {
            Grp<CS>::sync();
            if (rank != 0 && tid == 0) s_lp = *Grp<CS>::at(&s_lp, 0);
            Grp<CS>::sync();  // rank 0's copy is read before it changes or exits
        }
        if (tid == 0 && s_lp >= 0) L = g.lps[s_lp];
        __syncthreads();
        if (s_lp < 0) break;
        if (L.theta0 >= 0) {  // carried over from an earlier run of the same LP
            if (rank == 0 && tid == 0) {
                g.theta[s_lp] = L.theta0;
                g.iters[s_lp] = 0;
            }
            Grp<CS>::sync();
            continue;
        }
        const int c0 = L.col_off, c1 = c0 + L.n;
        for (int j = c0 + gt; j < c1; j += GT) g.x[j] = g.x_start[j];
        Grp<CS>::sync();
        double theta = 0.0, residual = INFINITY;
        int64_t it = 0;
        while (!(it > L.power_maxiter || residual <= L.power_tol ||
                 (L.power_rtol > 0 && residual <= L.power_rtol * theta))) {
            {
                StoreEpi<double> se{g.s};
                NoAcc a;
                lp_tiles<ITEMS, CS>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, g.x, se, a, prod);
            }
            Grp<CS>::sync();
            double th, inv;
            {
                PowerEpi<double> pe{g.x, g.Atx, nullptr, g.longAt};
                PowerEpi<double>::Acc a;
                pe.init(a);
                lp_tiles<ITEMS, CS>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, g.s, pe, a, prod);
                grp_sum<2, CS>(a.v, sh);
                double s0 = a.v[0], s1 = a.v[1];
                for (int l = L.at_lid0; l < L.at_lid1; l++) {
                    s0 += g.longAt[(size_t)l * 2];
                    s1 += g.longAt[(size_t)l * 2 + 1];
                }
                th = s0;
                inv = 1.0 / sqrt(s1);
            }
            double racc[1] = {0.0};
            for (int j = c0 + gt; j < c1; j += GT) {
                const double r = add_rn(mul_rn(-th, g.x[j]), g.Atx[j]);
                racc[0] += r * r;
                g.x[j] = mul_rn(g.Atx[j], inv);
            }
            grp_sum<1, CS>(racc, sh);  // its barriers also order the long-row terms' reuse
            residual = sqrt(racc[0]);
            theta = th;
            it++;
        }
        if (rank == 0 && tid == 0) {
            g.theta[s_lp] = theta;
            g.iters[s_lp] = it;
        }
        Grp<CS>::sync();
    }
    Grp<CS>::sync();  // no CTA exits while another may read its shared memory
}

// The solve kernel: each group (a CTA, or a cluster of CS CTAs) takes LPs from
// the queue until it is empty.  Rank 0 dequeues and reads the cancel flag; the
// other CTAs copy both from it, so every CTA of a group leaves the loop at the
// same LP.
template <int ITEMS, class T, int CS>
__global__ void __launch_bounds__(BT, batch_min_blocks<T>()) k_batch_pdlp(BatchArgs<T> g) {
    __shared__ __align__(16) T prod[BW * tile_buf<ITEMS>()];
    __shared__ double sh[BW * 8 + 8];
    __shared__ BatchCtl C;
    const int rank = Grp<CS>::rank();
    for (int guard = 0; guard <= g.count; guard++) {
        if (rank == 0 && threadIdx.x == 0) {
            const int q = atomicAdd(g.next, 1);
            C.lp = q < g.count ? g.order[q] : -1;
            C.cancelled = C.lp >= 0 ? *(volatile const int*)g.cancel : 0;
        }
        if constexpr (CS > 1) {
            Grp<CS>::sync();
            if (rank != 0 && threadIdx.x == 0) {
                const BatchCtl* c0p = Grp<CS>::at(&C, 0);
                C.lp = c0p->lp;
                C.cancelled = c0p->cancelled;
            }
            // rank 0's shared memory must outlive every read of it: no CTA
            // leaves (or rank 0 dequeues again) before all copies are done
            Grp<CS>::sync();
        }
        if (threadIdx.x == 0 && C.lp >= 0) {
            C.L = g.lps[C.lp];
            C.t_start = global_ns();
        }
        __syncthreads();
        if (C.lp < 0) break;
        if (C.cancelled) skip_one<T, CS>(g, C);
        else solve_one<ITEMS, T, CS>(g, C, prod, sh);
        Grp<CS>::sync();
    }
    // every CTA of a group leaves at the same LP; none exits while another
    // may still read its shared memory
    Grp<CS>::sync();
}

uint64_t splitmix64_at_host(uint64_t seed, uint64_t counter) {
    uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double powm_tol(int64_t n, bool f32) {
    uint64_t un = (uint64_t)n;
    int64_t n3 = (int64_t)(un * un * un);  // Int64 wrap, as IterativeSolvers' default
    return (f32 ? 1.1920928955078125e-07 : 2.220446049250313e-16) * (double)n3;
}

// one LP as the job keeps it: its own copies of the caller's arrays
struct LPData {
    cpdlp_lp v{};
    std::vector<int64_t> colptr, rowval;
    std::vector<double> nzval, c, lv, uv, lc, uc;
    void own() {
        colptr.assign(v.colptr, v.colptr + v.n + 1);
        rowval.assign(v.rowval, v.rowval + v.nnz);
        nzval.assign(v.nzval, v.nzval + v.nnz);
        c.assign(v.c, v.c + v.n); lv.assign(v.lv, v.lv + v.n); uv.assign(v.uv, v.uv + v.n);
        lc.assign(v.lc, v.lc + v.m); uc.assign(v.uc, v.uc + v.m);
        v.colptr = colptr.data(); v.rowval = rowval.data(); v.nzval = nzval.data();
        v.c = c.data(); v.lv = lv.data(); v.uv = uv.data(); v.lc = lc.data(); v.uc = uc.data();
    }
};

void check_lp(const cpdlp_lp& L) {
    if (L.m < 0 || L.n < 0 || L.nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative LP size in batch");
    if (!L.colptr || (L.nnz > 0 && (!L.rowval || !L.nzval)))
        fail(CPDLP_ERR_ARGUMENT, "null CSC array in batch");
    if (L.n > 0 && (!L.c || !L.lv || !L.uv)) fail(CPDLP_ERR_ARGUMENT, "null c/lv/uv in batch");
    if (L.m > 0 && (!L.lc || !L.uc)) fail(CPDLP_ERR_ARGUMENT, "null lc/uc in batch");
    if (L.colptr[0] != 1 || L.colptr[L.n] != L.nnz + 1)
        fail(CPDLP_ERR_ARGUMENT, "invalid CSC column pointer in batch");
    for (int64_t q = 0; q < L.nnz; q++)
        if (L.rowval[q] < 1 || L.rowval[q] > L.m)
            fail(CPDLP_ERR_ARGUMENT, "invalid CSC in batch: row index out of range");
}

// what one phase asks for each of its LPs
struct PhaseLP {
    int64_t id;        // index in the job
    double reltol, time_limit;
    int64_t max_passes, stall_passes;
    const double* x0;  // warm start (original units) or null
    const double* y0;
    double theta0 = -1.0;  // >= 0: skip the power method with this |A|^2 estimate
    double omega0 = 0.0;   // > 0: start from this primal weight
};

// One launch pair (power method, then the solve kernel) over a set of LPs on
// its own stream.  Results land in a mapped host block taken from the parent
// handle's pool: res[count] | done[count] | x[N] | y[M].
struct RunBase {
    virtual ~RunBase() = default;
    std::vector<PhaseLP> lps;
    std::vector<int64_t> row_off, col_off;
    int phase = 1;             // 1: first phase, 2: FP64 phase
    Handle rh;                 // the device, this run's stream
    Handle* parent = nullptr;  // owner of the host block pool
    cudaEvent_t ev = nullptr;  // recorded after both solve kernels
    cudaStream_t s2 = nullptr; // the cluster kernel's stream
    cudaEvent_t ev2 = nullptr; // orders s2 after the power method and ev after s2
    void* block = nullptr;
    BatchResult* h_res = nullptr;
    int* h_done = nullptr;
    double* h_x = nullptr;
    double* h_y = nullptr;
    std::vector<char> taken;   // per LP: result already taken by the job
    int64_t ntaken = 0;
    double setup = 0;
    bool done(int64_t k) const { return __atomic_load_n(h_done + k, __ATOMIC_ACQUIRE) != 0; }
    bool kernel_finished() {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaErrorNotReady) return false;
        CK(e);
        return true;
    }
    void open(Handle& h, int64_t count, int64_t N, int64_t M) {
        parent = &h;
        rh.device = h.device;
        rh.num_sms = h.num_sms;
        rh.pinned = h.pinned_area(sizeof(double) * 64);   // shared: runs start one at a time
        rh.pinned_bytes = sizeof(double) * 64;
        CK(cudaStreamCreateWithFlags(&rh.stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev2, cudaEventDisableTiming));
        const size_t a = ((size_t)count * sizeof(BatchResult) + 255) & ~(size_t)255;
        const size_t b = ((size_t)count * sizeof(int) + 255) & ~(size_t)255;
        const size_t bytes = a + b + sizeof(double) * (size_t)(std::max<int64_t>(N, 1) + std::max<int64_t>(M, 1));
        block = h.host_get(bytes);
        char* base = static_cast<char*>(block);
        h_res = reinterpret_cast<BatchResult*>(base);
        h_done = reinterpret_cast<int*>(base + a);
        h_x = reinterpret_cast<double*>(base + a + b);
        h_y = h_x + std::max<int64_t>(N, 1);
        memset(h_done, 0, sizeof(int) * (size_t)count);
        taken.assign((size_t)count, 0);
    }
    template <class P>
    P* dev(P* host) {
        void* d = nullptr;
        CK(cudaHostGetDevicePointer(&d, host, 0));
        return static_cast<P*>(d);
    }
    // waits for the kernels (a run is dropped early only when its job is)
    void close() {
        if (ev) cudaEventSynchronize(ev);
        if (rh.stream) cudaStreamSynchronize(rh.stream);
        release_device();
        if (s2) cudaStreamSynchronize(s2);
        if (ev) cudaEventDestroy(ev);
        if (ev2) cudaEventDestroy(ev2);
        ev2 = nullptr;
        if (s2) cudaStreamDestroy(s2);
        s2 = nullptr;
        ev = nullptr;
        if (rh.stream) cudaStreamDestroy(rh.stream);
        rh.stream = nullptr;
        if (block && parent) parent->host_put(block);
        block = nullptr;
    }
    virtual void release_device() = 0;
};

template <class T>
struct Run : RunBase {
    std::unique_ptr<ProblemBase> PB;
    TilePlan planA, planAt;
    DBuf<T> partA, partAt;
    DBuf<T> bx[2], by[2], bxa[2], bya[2], bxr, byr, bxbar;
    DBuf<double> d_x0, d_y0, longA, longAt, d_theta;
    DBuf<int64_t> d_piters;
    DBuf<BatchLP> d_desc;
    DBuf<int32_t> d_order;
    DBuf<int> d_next;
    DBuf<double> pw_x, pw_Atx, pw_s, pw_start, pw_pA, pw_pAt;  // power-method scratch

    ~Run() override { close(); }

    void launch(Handle& h, const std::vector<LPData>& all, const cpdlp_params& prm,
                const int* cancel, int items, int64_t max_ctas) {
        const double t0 = now_seconds();
        const int64_t count = (int64_t)lps.size();
        row_off.assign(count + 1, 0);
        col_off.assign(count + 1, 0);
        std::vector<int64_t> nz_off(count + 1, 0);
        for (int64_t k = 0; k < count; k++) {
            const cpdlp_lp& L = all[lps[k].id].v;
            row_off[k + 1] = row_off[k] + L.m;
            col_off[k + 1] = col_off[k] + L.n;
            nz_off[k + 1] = nz_off[k] + L.nnz;
        }
        const int64_t M = row_off[count], N = col_off[count], NZ = nz_off[count];
        if (M >= INT32_MAX || N >= INT32_MAX || NZ >= INT32_MAX)
            fail(CPDLP_ERR_UNSUPPORTED, "batch too large for int32 indices");
        open(h, count, N, M);
        cudaStream_t s = rh.stream;
        AllocScope scope(s);
        // occupancy first: it loads the kernels, which must not wait behind
        // this run's own queued work
        auto pk = (items == 8) ? k_batch_power<8, T, 1> : k_batch_power<4, T, 1>;
        auto pkc = (items == 8) ? k_batch_power<8, T, CLUSTER_CTAS> : k_batch_power<4, T, CLUSTER_CTAS>;
        auto kern = (items == 8) ? k_batch_pdlp<8, T, 1> : k_batch_pdlp<4, T, 1>;
        auto kclu = (items == 8) ? k_batch_pdlp<8, T, CLUSTER_CTAS> : k_batch_pdlp<4, T, CLUSTER_CTAS>;
        int per_sm_p = 0, per_sm = 0, nclusters = 0, nclusters_p = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_p, pk, BT, 0));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT, 0));
        cudaLaunchAttribute cattr[1];
        cattr[0].id = cudaLaunchAttributeClusterDimension;
        cattr[0].val.clusterDim.x = CLUSTER_CTAS;
        cattr[0].val.clusterDim.y = 1;
        cattr[0].val.clusterDim.z = 1;
        cudaLaunchConfig_t ccfg = {};
        ccfg.gridDim = dim3(CLUSTER_CTAS);
        ccfg.blockDim = dim3(BT);
        ccfg.dynamicSmemBytes = 0;
        ccfg.stream = s2;
        ccfg.attrs = cattr;
        ccfg.numAttrs = 1;
        CK(cudaOccupancyMaxActiveClusters(&nclusters, kclu, &ccfg));
        CK(cudaOccupancyMaxActiveClusters(&nclusters_p, pkc, &ccfg));
        // block-diagonal concatenation (1-based CSC)
        std::vector<int64_t> colptr((size_t)N + 1), rowval((size_t)std::max<int64_t>(NZ, 1));
        std::vector<double> nzval(rowval.size()), c((size_t)std::max<int64_t>(N, 1)),
            lv(c.size()), uv(c.size()), lc((size_t)std::max<int64_t>(M, 1)), uc(lc.size());
        colptr[0] = 1;
        // each LP's slices are disjoint: host threads copy LPs in parallel
        parallel_for(count, [&](int64_t k) {
            const cpdlp_lp& L = all[lps[k].id].v;
            for (int64_t j = 0; j < L.n; j++) colptr[col_off[k] + j + 1] = nz_off[k] + L.colptr[j + 1];
            for (int64_t q = 0; q < L.nnz; q++) {
                rowval[nz_off[k] + q] = row_off[k] + L.rowval[q];
                nzval[nz_off[k] + q] = L.nzval[q];
            }
            if (L.n > 0) {
                std::copy(L.c, L.c + L.n, c.begin() + col_off[k]);
                std::copy(L.lv, L.lv + L.n, lv.begin() + col_off[k]);
                std::copy(L.uv, L.uv + L.n, uv.begin() + col_off[k]);
            }
            if (L.m > 0) {
                std::copy(L.lc, L.lc + L.m, lc.begin() + row_off[k]);
                std::copy(L.uc, L.uc + L.m, uc.begin() + row_off[k]);
            }
        });
        cpdlp_lp big{M, N, NZ, colptr.data(), rowval.data(), nzval.data(), c.data(), lv.data(),
                     uv.data(), lc.data(), uc.data()};
        // the batched kernels read the scaled values (no narrow +-1 storage)
        // and cut their own tile plans at LP boundaries (the problem builds none)
        cpdlp_params pprm = prm;
        pprm.tile_flags |= CPDLP_TILE_NO_NARROW;
        PB.reset(problem_create(rh, &big, &pprm, false));
        auto& P = static_cast<ProblemT<T>&>(*PB);
        // tile plans with LP boundaries
        std::vector<int32_t> hpA((size_t)M + 1), hpAt((size_t)N + 1);
        CK(cudaMemcpyAsync(hpA.data(), P.a_ptr.p, sizeof(int32_t) * (M + 1), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hpAt.data(), P.at_ptr.p, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        std::vector<int32_t> aT, aL, aI, atT, atL, atI;
        build_tile_plan(hpA, (int32_t)M, items, planA, s, &row_off, &aT, &aL, &aI, 32 * BATCH_RPL);
        build_tile_plan(hpAt, (int32_t)N, items, planAt, s, &col_off, &atT, &atL, &atI, 32 * BATCH_RPL);
        partA.alloc((size_t)std::max(planA.npieces, 1));
        partAt.alloc((size_t)std::max(planAt.npieces, 1));
        // per-LP descriptors and the largest-first queue order
        std::vector<BatchLP> desc((size_t)count);
        bool any_warm = false;
        for (int64_t k = 0; k < count; k++) {
            const cpdlp_lp& L = all[lps[k].id].v;
            BatchLP& d = desc[(size_t)k];
            d.m = (int32_t)L.m; d.n = (int32_t)L.n;
            d.row_off = (int32_t)row_off[k]; d.col_off = (int32_t)col_off[k];
            d.a_t0 = aT[k]; d.a_t1 = aT[k + 1]; d.a_l0 = aL[k]; d.a_l1 = aL[k + 1];
            d.at_t0 = atT[k]; d.at_t1 = atT[k + 1]; d.at_l0 = atL[k]; d.at_l1 = atL[k + 1];
            d.a_lid0 = aI[k]; d.a_lid1 = aI[k + 1]; d.at_lid0 = atI[k]; d.at_lid1 = atI[k + 1];
            bool zc = true;
            for (int64_t j = 0; j < L.n; j++)
                if (L.c[j] != 0.0) { zc = false; break; }
            d.zero_cost = zc ? 1 : 0;
            d.warm = (lps[k].x0 || lps[k].y0) ? 1 : 0;
            any_warm = any_warm || d.warm;
            // the power method runs in FP64 for either iterate type
            d.power_tol = prm.power_tol_override > 0 ? prm.power_tol_override : powm_tol(d.n, false);
            d.power_maxiter = prm.power_maxiter_override > 0 ? prm.power_maxiter_override : d.n;
            // FP32 iterates need theta to about 1%, not to eps(Float64) n^3
            d.power_rtol = std::is_same<T, float>::value ? POWER_RTOL_F32 : 0.0;
            d.reltol = lps[k].reltol;
            d.time_limit = lps[k].time_limit;
            d.max_passes = lps[k].max_passes;
            d.stall_passes = lps[k].stall_passes;
            d.theta0 = lps[k].theta0;
            d.omega0 = lps[k].omega0;
        }
        std::vector<int32_t> order((size_t)count);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            return nz_off[a + 1] - nz_off[a] > nz_off[b + 1] - nz_off[b];
        });
        // largest first: the first nbig LPs of the order go to the cluster kernel
        // (the routing depends on the LP and its phase alone, so its arithmetic
        // does too)
        const int64_t cmin = phase == 2 ? PHASE_CLUSTER_MIN_NNZ : CLUSTER_MIN_NNZ;
        int64_t nbig = 0;
        if (nclusters > 0 && nclusters_p > 0)
            while (nbig < count && nz_off[order[nbig] + 1] - nz_off[order[nbig]] >= cmin) nbig++;
        // power-method start vectors: the single-LP generator, per LP from counter
        // 0, so every LP's vector is a prefix of one vector (computed once)
        int64_t nmax = 0;
        for (int64_t k = 0; k < count; k++) nmax = std::max(nmax, col_off[k + 1] - col_off[k]);
        std::vector<double> g0((size_t)nmax);
        for (int64_t j = 0; j < nmax; j++) {
            const double u1 = (double)((splitmix64_at_host(prm.power_seed, 2 * (uint64_t)j) >> 11) + 1) *
                              (1.0 / 9007199254740992.0);
            const double u2 = (double)((splitmix64_at_host(prm.power_seed, 2 * (uint64_t)j + 1) >> 11) + 1) *
                              (1.0 / 9007199254740992.0);
            g0[(size_t)j] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        }
        std::vector<double> xs((size_t)std::max<int64_t>(N, 1));
        for (int64_t k = 0; k < count; k++)
            std::copy(g0.begin(), g0.begin() + (col_off[k + 1] - col_off[k]), xs.begin() + col_off[k]);
        const size_t nz = (size_t)std::max<int64_t>(N, 1), mz = (size_t)std::max<int64_t>(M, 1);
        std::vector<double> hx0, hy0;
        if (any_warm) {
            hx0.assign(nz, 0.0);
            hy0.assign(mz, 0.0);
            for (int64_t k = 0; k < count; k++) {
                if (lps[k].x0) std::copy(lps[k].x0, lps[k].x0 + (col_off[k + 1] - col_off[k]), hx0.begin() + col_off[k]);
                if (lps[k].y0) std::copy(lps[k].y0, lps[k].y0 + (row_off[k + 1] - row_off[k]), hy0.begin() + row_off[k]);
            }
        }
        // device buffers
        for (int b = 0; b < 2; b++) { bx[b].alloc(nz); by[b].alloc(mz); bxa[b].alloc(nz); bya[b].alloc(mz); }
        bxr.alloc(nz); byr.alloc(mz); bxbar.alloc(nz);
        d_desc.alloc((size_t)std::max<int64_t>(count, 1));
        d_order.alloc((size_t)std::max<int64_t>(count, 1));
        d_theta.alloc((size_t)std::max<int64_t>(count, 1));
        d_piters.alloc((size_t)std::max<int64_t>(count, 1));
        longA.alloc((size_t)std::max(planA.nlong, 1) * 2);
        longAt.alloc((size_t)std::max(planAt.nlong, 1) * 3);
        d_next.alloc(4);
        if (any_warm) {
            d_x0.alloc(nz);
            d_y0.alloc(mz);
            CK(cudaMemcpyAsync(d_x0.p, hx0.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(d_y0.p, hy0.data(), sizeof(double) * mz, cudaMemcpyHostToDevice, s));
        }
        CK(cudaMemcpyAsync(d_desc.p, desc.data(), sizeof(BatchLP) * desc.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_order.p, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(d_next.p, 0, 4 * sizeof(int), s));
        // power method: FP64 vectors; the cluster-sized LPs on s2, the others on s
        pw_x.alloc(nz); pw_Atx.alloc(nz); pw_s.alloc(mz); pw_start.alloc(nz);
        pw_pA.alloc((size_t)std::max(planA.npieces, 1));
        pw_pAt.alloc((size_t)std::max(planAt.npieces, 1));
        CK(cudaMemcpyAsync(pw_start.p, xs.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, s));
        PowerArgs<T> pg;
        pg.A = CsrView<T, double>{P.a_ptr.p, P.a_idx.p, P.a_val.p, planA.tasks.p, planA.ntasks,
                                  planA.ltasks.p, planA.nltasks, planA.counters.p, pw_pA.p};
        pg.At = CsrView<T, double>{P.at_ptr.p, P.at_idx.p, P.at_val.p, planAt.tasks.p,
                                   planAt.ntasks, planAt.ltasks.p, planAt.nltasks,
                                   planAt.counters.p, pw_pAt.p};
        pg.x = pw_x.p; pg.Atx = pw_Atx.p; pg.s = pw_s.p; pg.x_start = pw_start.p;
        pg.lps = d_desc.p; pg.theta = d_theta.p; pg.iters = d_piters.p; pg.longAt = longAt.p;
        if (nbig > 0) {  // s2 starts after everything queued on s so far
            CK(cudaEventRecord(ev2, s));
            CK(cudaStreamWaitEvent(s2, ev2, 0));
            PowerArgs<T> pb = pg;
            pb.order = d_order.p;
            pb.count = (int32_t)nbig;
            pb.next = d_next.p + 3;
            int64_t nc = std::min<int64_t>(nbig, nclusters_p);
            if (max_ctas > 0) nc = std::min<int64_t>(nc, std::max<int64_t>(max_ctas / CLUSTER_CTAS, 1));
            ccfg.gridDim = dim3((unsigned)(nc * CLUSTER_CTAS));
            CK(cudaLaunchKernelEx(&ccfg, pkc, pb));
        }
        if (count > nbig) {
            PowerArgs<T> ps1 = pg;
            ps1.order = d_order.p + nbig;
            ps1.count = (int32_t)(count - nbig);
            ps1.next = d_next.p + 1;
            int64_t pgrid = std::min<int64_t>(count - nbig, (int64_t)std::max(per_sm_p, 1) * rh.num_sms);
            if (max_ctas > 0) pgrid = std::min(pgrid, max_ctas);
            pgrid = std::max<int64_t>(pgrid, 1);
            pk<<<(unsigned)pgrid, BT, 0, s>>>(ps1);
            CK_LAUNCH();
        }
        int64_t grid = std::min<int64_t>(count, (int64_t)std::max(per_sm, 1) * rh.num_sms);
        if (max_ctas > 0) grid = std::min(grid, max_ctas);
        grid = std::max<int64_t>(grid, 1);
        BatchArgs<T> g;
        g.A = CsrView<T, T>{P.a_ptr.p, P.a_idx.p, P.a_val.p, planA.tasks.p, planA.ntasks,
                            planA.ltasks.p, planA.nltasks, planA.counters.p, partA.p};
        g.At = CsrView<T, T>{P.at_ptr.p, P.at_idx.p, P.at_val.p, planAt.tasks.p, planAt.ntasks,
                             planAt.ltasks.p, planAt.nltasks, planAt.counters.p, partAt.p};
        g.c = P.c.p; g.lv = P.lv.p; g.uv = P.uv.p; g.lc = P.lc.p; g.uc = P.uc.p;
        g.invD1 = P.invD1.p; g.invD2 = P.invD2.p; g.D1 = P.D1.p; g.D2 = P.D2.p;
        g.invD1t = P.invD1_T(); g.invD2t = P.invD2_T();
        for (int b = 0; b < 2; b++) { g.x[b] = bx[b].p; g.y[b] = by[b].p; g.xa[b] = bxa[b].p; g.ya[b] = bya[b].p; }
        g.xr = bxr.p; g.yr = byr.p; g.xbar = bxbar.p;
        g.theta = d_theta.p;
        g.power_iters = d_piters.p;
        g.x_init = any_warm ? d_x0.p : nullptr;
        g.y_init = any_warm ? d_y0.p : nullptr;
        g.lps = d_desc.p; g.order = d_order.p;
        g.res = dev(h_res); g.out_x = dev(h_x); g.out_y = dev(h_y); g.done = dev(h_done);
        g.longA = longA.p; g.longAt = longAt.p;
        g.next = d_next.p; g.cancel = cancel; g.count = (int32_t)count;
        g.prm = BatchParams{prm.algorithm, prm.check_every > 0 ? prm.check_every : 100,
                            prm.invnorm_scaling, prm.primal_weight_damping, prm.zero_tol,
                            prm.sufficient_decay, prm.necessary_decay, prm.artificial_decay};
        setup = now_seconds() - t0;
        if (nbig > 0) {
            // the cluster kernel on its own stream, after its LPs' power method
            BatchArgs<T> gb = g;
            gb.order = d_order.p;
            gb.count = (int32_t)nbig;
            gb.next = d_next.p + 2;
            int64_t nc = std::min<int64_t>(nbig, nclusters);
            if (max_ctas > 0) nc = std::min<int64_t>(nc, std::max<int64_t>(max_ctas / CLUSTER_CTAS, 1));
            ccfg.gridDim = dim3((unsigned)(nc * CLUSTER_CTAS));
            CK(cudaLaunchKernelEx(&ccfg, kclu, gb));  // after s2's power method
            CK(cudaEventRecord(ev2, s2));
        }
        if (count > nbig) {
            g.order = d_order.p + nbig;
            g.count = (int32_t)(count - nbig);
            grid = std::max<int64_t>(std::min<int64_t>(grid, count - nbig), 1);
            kern<<<(unsigned)grid, BT, 0, s>>>(g);
            CK_LAUNCH();
        }
        if (nbig > 0) CK(cudaStreamWaitEvent(s, ev2, 0));
        CK(cudaEventRecord(ev, s));
    }
    void release_device() override {
        AllocScope scope(rh.stream);
        PB.reset();
        for (int b = 0; b < 2; b++) { bx[b].release(); by[b].release(); bxa[b].release(); bya[b].release(); }
        bxr.release(); byr.release(); bxbar.release(); partA.release(); partAt.release();
        d_x0.release(); d_y0.release(); longA.release(); longAt.release(); d_desc.release();
        d_order.release(); d_theta.release(); d_piters.release(); d_next.release();
        pw_x.release(); pw_Atx.release(); pw_s.release(); pw_start.release();
        pw_pA.release(); pw_pAt.release();
        planA = TilePlan();
        planAt = TilePlan();
    }
};

}  // namespace

// ---- jobs ---------------------------------------------------------------------
// A job owns copies of its LPs and the runs in flight.  poll() takes every LP
// whose done flag is set (so an LP is available as soon as its CTA finishes,
// not when the whole launch does), starts an FP64 run for the LPs that need
// one, and drops runs whose kernels have finished.
struct Job {
    Handle* parent = nullptr;
    Handle jh;                 // device and a stream for the cancel flag
    cpdlp_params prm{};
    int items = BATCH_ITEMS;
    int64_t max_ctas = 0;      // > 0: at most this many CTAs per launch
    std::vector<LPData> lps;
    std::vector<double> target;  // final relative KKT tolerance per LP
    std::vector<std::vector<double>> x, y;
    std::vector<cpdlp_stats> st;
    std::vector<char> final_;  // LP finished for good
    int64_t remaining = 0;
    std::vector<std::unique_ptr<RunBase>> runs;
    bool cancelled = false;
    DBuf<int> d_cancel;

    ~Job() {
        runs.clear();          // each run waits for its kernels
        d_cancel.release();
        if (jh.stream) {
            cudaStreamSynchronize(jh.stream);
            cudaStreamDestroy(jh.stream);
        }
    }

    void start(const std::vector<PhaseLP>& phase_lps, int32_t float_type, int phase) {
        cpdlp_params p = prm;
        p.float_type = float_type;
        std::unique_ptr<RunBase> r;
        if (float_type == CPDLP_VAL_F32) r.reset(new Run<float>());
        else r.reset(new Run<double>());
        r->lps = phase_lps;
        r->phase = phase;
        if (float_type == CPDLP_VAL_F32)
            static_cast<Run<float>&>(*r).launch(*parent, lps, p, d_cancel.p, items, max_ctas);
        else
            static_cast<Run<double>&>(*r).launch(*parent, lps, p, d_cancel.p, items, max_ctas);
        runs.push_back(std::move(r));
    }

    // takes LP k of run r; returns true if it continues in the FP64 phase
    bool take(RunBase& r, size_t k, PhaseLP& next) {
        const int64_t id = r.lps[k].id;
        const cpdlp_lp& L = lps[id].v;
        const BatchResult R = r.h_res[k];
        const bool first = r.phase == 1;
        x[id].assign(r.h_x + r.col_off[k], r.h_x + r.col_off[k + 1]);
        y[id].assign(r.h_y + r.row_off[k], r.h_y + r.row_off[k + 1]);
        cpdlp_stats& S = st[id];
        const int64_t passes_before = first ? 0 : S.kkt_passes;
        const double time_before = first ? 0.0 : S.time_elapsed;
        const int64_t launches_before = first ? 0 : S.kernel_launches;
        memset(&S, 0, sizeof(S));
        S.err = R.err;
        S.time_elapsed = time_before + R.time_elapsed;
        S.kkt_passes = passes_before + R.kkt_passes;
        S.refine_kkt_passes = first ? 0 : R.kkt_passes;
        S.termination_status = R.status;
        S.restart_from_avg = R.restart_from_avg;
        S.outer = R.outer; S.inner = R.inner; S.total = R.total;
        S.eta = R.eta; S.eta_sum = R.eta_sum; S.omega = R.omega;
        S.power_iterations = R.power_iterations;
        S.setup_seconds = r.setup;
        S.kernel_launches = launches_before + 2;  // power method + solve
        const bool early = L.m == 0 && R.status == CPDLP_OPTIMAL && R.kkt_passes == 0;
        // FP64 phase: LPs that reached the FP32 tolerance but target a tighter
        // one, and LPs whose FP32 iterates stalled
        const bool refine = R.status == CPDLP_OPTIMAL && target[id] < r.lps[k].reltol;
        const bool rescue = R.stalled && R.kkt_passes < prm.max_kkt_passes;
        if (first && prm.float_type == CPDLP_VAL_F32 && !cancelled && !early && (refine || rescue)) {
            next.id = id;
            next.reltol = target[id];
            next.max_passes = std::max<int64_t>(prm.max_kkt_passes - R.kkt_passes, 1);
            next.stall_passes = 0;
            next.time_limit = prm.time_limit - R.time_elapsed;
            // continuation: the FP64 run keeps the FP32 run's |A|^2 estimate (an FP64
            // power method over the same values up to FP32 rounding).  After a
            // converged FP32 run it starts from the FP32 solution with its primal
            // weight; after a stalled one it starts cold (a stalled FP32 iterate
            // can be a poor start: one LP of the 4,096-LP workload ran out of
            // 93,400 FP64 passes from it and needs 3,400 from zero)
            next.x0 = refine ? x[id].data() : nullptr;
            next.y0 = refine ? y[id].data() : nullptr;
            next.theta0 = R.theta;
            next.omega0 = refine ? R.omega : 0.0;
            return true;
        }
        final_[id] = 1;
        remaining--;
        return false;
    }

    bool poll() {
        std::vector<PhaseLP> next;
        for (auto& rp : runs) {
            RunBase& r = *rp;
            if (r.ntaken == (int64_t)r.lps.size()) continue;
            // the kernel's state is read before the flags, so that a finished
            // kernel with an unset flag (an error) is seen
            const bool kdone = r.kernel_finished();
            for (size_t k = 0; k < r.lps.size(); k++) {
                if (r.taken[k] || !r.done((int64_t)k)) continue;
                r.taken[k] = 1;
                r.ntaken++;
                PhaseLP q;
                if (take(r, k, q)) next.push_back(q);
            }
            if (kdone && r.ntaken != (int64_t)r.lps.size())
                fail(CPDLP_ERR_CUDA, "batched solve kernel ended without finishing every LP");
        }
        // drop runs that are complete
        for (auto& rp : runs)
            if (rp && rp->ntaken == (int64_t)rp->lps.size() && rp->kernel_finished()) rp.reset();
        runs.erase(std::remove(runs.begin(), runs.end(), nullptr), runs.end());
        if (!next.empty()) start(next, CPDLP_VAL_F64, 2);
        return remaining == 0 && runs.empty();
    }
};

Job* job_submit(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                const double* reltol, const double* const* x0, const double* const* y0,
                int64_t max_ctas) {
    if (count < 0) fail(CPDLP_ERR_ARGUMENT, "negative batch size");
    if (count > 0 && !lps) fail(CPDLP_ERR_ARGUMENT, "null LP array");
    if (!params) fail(CPDLP_ERR_ARGUMENT, "null params");
    if (params->check_every <= 0) fail(CPDLP_ERR_ARGUMENT, "check_every must be positive");
    if (params->float_type != CPDLP_VAL_F64 && params->float_type != CPDLP_VAL_F32)
        fail(CPDLP_ERR_ARGUMENT, "float_type must be CPDLP_VAL_F64 or CPDLP_VAL_F32");
    // the density-order bits concern single-LP solves (batched LPs run in their own order)
    if (params->tile_flags & ~(CPDLP_TILE_NO_NARROW | CPDLP_TILE_DENSITY_ORDER | CPDLP_TILE_NO_DENSITY_ORDER))
        fail(CPDLP_ERR_ARGUMENT, "unknown tile_flags bits");
    if (count > INT32_MAX) fail(CPDLP_ERR_UNSUPPORTED, "batch too large");
    if (max_ctas < 0) fail(CPDLP_ERR_ARGUMENT, "max_ctas must be >= 0");
    for (int64_t k = 0; k < count; k++) check_lp(lps[k]);
    std::unique_ptr<Job> J(new Job());
    J->parent = &h;
    J->prm = *params;
    J->max_ctas = max_ctas;
    J->items = params->tile_nnz > 0 ? choose_items(0, 1, params->tile_nnz) : BATCH_ITEMS;
    if (J->items != 4 && J->items != 8) J->items = 8;
    J->jh.device = h.device;
    J->jh.num_sms = h.num_sms;
    CK(cudaStreamCreateWithFlags(&J->jh.stream, cudaStreamNonBlocking));
    {
        AllocScope scope(J->jh.stream);
        J->d_cancel.alloc(1);
        CK(cudaMemsetAsync(J->d_cancel.p, 0, sizeof(int), J->jh.stream));
        CK(cudaStreamSynchronize(J->jh.stream));
    }
    J->lps.resize((size_t)count);
    J->target.resize((size_t)count);
    J->x.resize((size_t)count);
    J->y.resize((size_t)count);
    J->st.assign((size_t)count, cpdlp_stats{});
    J->final_.assign((size_t)count, 0);
    J->remaining = count;
    const bool f32 = params->float_type == CPDLP_VAL_F32;
    std::vector<PhaseLP> first((size_t)count);
    for (int64_t k = 0; k < count; k++) {
        J->lps[k].v = lps[k];
        J->lps[k].own();
        double t = reltol ? reltol[k] : (f32 && params->refine_reltol > 0 ? params->refine_reltol
                                                                         : params->termination_reltol);
        if (!(t >= 0)) fail(CPDLP_ERR_ARGUMENT, "relative tolerance must be >= 0");
        J->target[k] = t;
        PhaseLP& q = first[k];
        q.id = k;
        // FP32 iterates stop at the FP32 phase's tolerance; tighter targets refine in FP64
        q.reltol = f32 ? std::max(t, params->termination_reltol) : t;
        q.max_passes = params->max_kkt_passes;
        q.stall_passes = f32 ? BATCH_STALL_CHECKS * (int64_t)params->check_every : 0;
        q.time_limit = params->time_limit;
        q.x0 = x0 ? x0[k] : nullptr;
        q.y0 = y0 ? y0[k] : nullptr;
    }
    if (count > 0) J->start(first, params->float_type, 1);
    return J.release();
}

bool job_poll(Job* j) { return j->poll(); }

void job_wait(Job* j) {
    while (!j->poll()) {
        // sleep on the oldest run's kernel; its LPs are taken by the next poll
        if (!j->runs.empty()) CK(cudaEventSynchronize(j->runs.front()->ev));
    }
}

void job_cancel(Job* j) {
    if (j->remaining == 0) return;
    j->cancelled = true;
    // the runs' streams are busy with their kernels: set the flag from the job's stream
    static const int one = 1;
    CK(cudaMemcpyAsync(j->d_cancel.p, &one, sizeof(int), cudaMemcpyHostToDevice, j->jh.stream));
    CK(cudaStreamSynchronize(j->jh.stream));
}

void job_ready(const Job* j, int32_t* ready) {
    for (size_t k = 0; k < j->final_.size(); k++) ready[k] = j->final_[k] ? 1 : 0;
}

void job_collect_lp(Job* j, int64_t k, double* x_out, double* y_out, cpdlp_stats* stats) {
    if (k < 0 || k >= (int64_t)j->lps.size()) fail(CPDLP_ERR_ARGUMENT, "LP index out of range");
    if (!j->final_[(size_t)k]) fail(CPDLP_ERR_ARGUMENT, "LP not finished (poll until it is ready)");
    if (x_out) std::copy(j->x[k].begin(), j->x[k].end(), x_out);
    if (y_out) std::copy(j->y[k].begin(), j->y[k].end(), y_out);
    if (stats) *stats = j->st[k];
}

void job_collect(Job* j, double* const* x_out, double* const* y_out, cpdlp_stats* stats) {
    if (j->remaining != 0) fail(CPDLP_ERR_ARGUMENT, "job not finished (poll until it reports done)");
    for (size_t k = 0; k < j->lps.size(); k++)
        job_collect_lp(j, (int64_t)k, x_out ? x_out[k] : nullptr, y_out ? y_out[k] : nullptr,
                       stats ? stats + k : nullptr);
}

int64_t job_count(const Job* j) { return (int64_t)j->lps.size(); }

void job_destroy(Job* j) { delete j; }

int64_t batch_footprint(int64_t count, const cpdlp_lp* lps, const cpdlp_params* params) {
    const int64_t sv = params && params->float_type == CPDLP_VAL_F32 ? 4 : 8;
    int64_t m = 0, n = 0, nnz = 0;
    for (int64_t k = 0; k < count; k++) {
        m += std::max<int64_t>(lps[k].m, 0);
        n += std::max<int64_t>(lps[k].n, 0);
        nnz += std::max<int64_t>(lps[k].nnz, 0);
    }
    // matrices: CSR of A and A' (index, value, padding) plus the preprocessing's
    // FP64 CSC copies and sort buffers; vectors: 7 iterates of n and 5 of m,
    // bounds and costs, FP64 scalings, power-method vectors
    const int64_t mat = nnz * (2 * (4 + sv) + 40) + (m + n) * 16 + (1 << 16);
    const int64_t vec = n * (10 * sv + 6 * 8) + m * (8 * sv + 5 * 8);
    return mat + vec + count * 256 + (4 << 20);
}

void batch_solve(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 double* const* x_out, double* const* y_out, cpdlp_stats* stats) {
    if (count == 0) return;
    std::unique_ptr<Job> J(job_submit(h, count, lps, params, nullptr, nullptr, nullptr, 0));
    job_wait(J.get());
    job_collect(J.get(), x_out, y_out, stats);
}

}  // namespace cpdlp

