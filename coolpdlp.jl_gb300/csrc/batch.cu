// batch.cu -- many independent LPs in one persistent launch.
//
// The LPs are concatenated block-diagonally on the host and preprocessed once
// by the single-LP device pipeline: Ruiz and Pock-Chambolle scaling work on
// rows and columns, so the scaling of the concatenation equals the scaling of
// each LP.  The tile partitions are then rebuilt so that no tile crosses an LP
// boundary.  One CTA solves one LP at a time and takes the next LP from an
// atomic counter when it finishes: power method (linalg.jl:86-96), primal
// weight (step_size.jl:29-40), then blocks of check_every fused PDHG steps
// (pdlp.jl:96-136) with the four-iterate KKT check, restart and termination
// logic (pdlp.jl:138-196, restart.jl:40-57, termination.jl:89-101) run by the
// CTA itself, thread 0 taking the FP64 decisions.  Every loop is bounded by
// max_kkt_passes and the time limit; no CTA waits on another.
//
// The solve(milp, algo) semantics per LP are those of the single-LP path
// (common.jl:186-209) except that no error history is recorded.
#include <algorithm>
#include <memory>
#include <type_traits>

#include "batch.cuh"
#include "epilogues.cuh"
#include "solver.cuh"

namespace cpdlp {

namespace {

constexpr int BW = TILE_WARPS;  // warps per CTA
constexpr int BT = BW * 32;

struct BatchLP {
    int32_t m, n, row_off, col_off;
    int32_t a_t0, a_t1, a_l0, a_l1;
    int32_t at_t0, at_t1, at_l0, at_l1;
    int32_t a_lid0, a_lid1, at_lid0, at_lid1;
    int32_t zero_cost, pad;
    double power_tol;
    int64_t power_maxiter;
};

struct BatchResult {
    cpdlp_kkt_errors err;
    int64_t kkt_passes, outer, inner, total, power_iterations;
    double eta, omega, eta_sum, time_elapsed;
    int32_t status, restart_from_avg;
};

struct BatchParams {
    int32_t algorithm, check_every;
    int64_t max_kkt_passes;
    double termination_reltol, time_limit;
    double invnorm_scaling, primal_weight_damping, zero_tol;
    double sufficient_decay, necessary_decay, artificial_decay;
};

template <class T>
struct BatchArgs {
    CsrView<T, T> A, At;
    const T *c, *lv, *uv, *lc, *uc;
    const double *invD1, *invD2, *D1, *D2;
    T *x[2], *y[2], *xa[2], *ya[2], *xr, *yr, *xbar;
    const double* x_start;
    const BatchLP* lps;
    BatchResult* res;
    double* out_x;
    double* out_y;
    double* red;      // per CTA: 32 doubles
    double* longA;    // row-side long-row terms (2 per long row of A)
    double* longAt;   // column-side long-row terms (3 per long row of A')
    StepCoef<T>* coef;  // per CTA
    int* next;
    int32_t count;
    BatchParams prm;
};

// -- block-wide helpers ---------------------------------------------------------
template <int Q>
__device__ __forceinline__ void block_sum(double (&v)[Q], double* sh) {
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
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; q++) v[q] = sh[BW * Q + q];
    __syncthreads();
}

// the LP's tiles of one matrix, warps striding over its tasks
template <int ITEMS, class T, class Epi>
__device__ __forceinline__ void lp_tiles(const CsrView<T, T>& V, int t0, int t1, int l0, int l1,
                                         const T* xin, Epi& epi, typename Epi::Acc& acc,
                                         T* prod) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const VecSet<T, 1> xs{{xin}};
    for (int t = l0 + w; t < l1; t += BW) long_piece<ITEMS, 1>(V, xs, epi, acc, V.ltasks[t], lane);
    for (int t = t0 + w; t < t1; t += BW) {
        const int4 tk = V.tasks[t];
        short_tile<ITEMS, 1>(V, xs, epi, acc, tk.x, tk.y, tk.z, tk.w, lane, prod + w * 32 * ITEMS);
    }
}

__device__ __forceinline__ double rel_err(const cpdlp_kkt_errors& e) {
    return jl_max(jl_max(e.primal / e.primal_scale, e.dual / e.dual_scale), e.gap / e.gap_scale);
}
__device__ __forceinline__ double abs_err(const cpdlp_kkt_errors& e, double w) {
    return sqrt((w * w) * (e.primal * e.primal) + (1.0 / (w * w)) * (e.dual * e.dual) +
                e.gap * e.gap);
}

template <int ITEMS, class T>
__global__ void __launch_bounds__(BT) k_batch_pdlp(BatchArgs<T> g) {
    __shared__ T prod[BW * 32 * ITEMS];
    __shared__ double sh[BW * 8 + 8];
    __shared__ int s_lp;
    __shared__ double s_eta, s_omega, s_eta_sum, s_pscale, s_dscale;
    __shared__ T s_theta, s_inv;
    __shared__ int s_flag;
    __shared__ cpdlp_kkt_errors s_e[4];
    StepCoef<T>* coef = g.coef + blockIdx.x;
    double* red = g.red + (size_t)blockIdx.x * 32;
    const int tid = threadIdx.x;
    const bool pdlp = g.prm.algorithm == CPDLP_ALGO_PDLP;
    for (int iter_guard = 0; iter_guard < g.count; iter_guard++) {
        if (tid == 0) s_lp = atomicAdd(g.next, 1);
        __syncthreads();
        const int k = s_lp;
        __syncthreads();
        if (k >= g.count) break;
        const BatchLP L = g.lps[k];
        const uint64_t t_start = global_ns();
        const int c0 = L.col_off, c1 = L.col_off + L.n, r0 = L.row_off, r1 = L.row_off + L.m;
        BatchResult R;
        memset(&R, 0, sizeof(R));
        // ---- power method on A'A (linalg.jl:86-96): buffers xa[1] (x), xbar (Ax), ya[1] (A x)
        T* px = g.xa[1];
        T* pAx = g.xbar;
        T* ps = g.ya[1];
        for (int j = c0 + tid; j < c1; j += BT) px[j] = (T)g.x_start[j];
        __syncthreads();
        double theta_d = 0.0, residual = INFINITY;
        int64_t it = 0;
        while (!(it > L.power_maxiter || residual <= L.power_tol)) {
            {
                StoreEpi<T> se{ps};
                NoAcc a;
                lp_tiles<ITEMS, T>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, px, se, a, prod);
            }
            __syncthreads();
            {
                PowerEpi<T> pe{px, pAx, red, g.longAt};
                typename PowerEpi<T>::Acc a;
                pe.init(a);
                lp_tiles<ITEMS, T>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, ps, pe, a, prod);
                block_sum<2>(a.v, sh);
                if (tid == 0) {
                    double s0 = a.v[0], s1 = a.v[1];
                    for (int l = L.at_lid0; l < L.at_lid1; l++) {
                        s0 += g.longAt[(size_t)l * 2];
                        s1 += g.longAt[(size_t)l * 2 + 1];
                    }
                    s_theta = (T)s0;
                    const T nrm = (T)sqrt(s1);
                    s_inv = T(1) / nrm;
                }
                __syncthreads();
            }
            double racc[1] = {0.0};
            const T th = s_theta, inv = s_inv;
            for (int j = c0 + tid; j < c1; j += BT) {
                const T r = add_rn(mul_rn(-th, px[j]), pAx[j]);
                racc[0] += (double)r * (double)r;
                px[j] = mul_rn(pAx[j], inv);
            }
            block_sum<1>(racc, sh);
            residual = sqrt(racc[0]);
            theta_d = (double)th;
            it++;
        }
        R.power_iterations = it;
        // ---- scales and primal weight (errors.jl:79-85, step_size.jl:29-40)
        {
            double q[4] = {0, 0, 0, 0};
            for (int i = r0 + tid; i < r1; i += BT) {
                const double cb = combine((double)g.lc[i], (double)g.uc[i]);
                const double sv = g.invD1[i] * cb;
                q[0] += sv * sv;
                q[1] += cb * cb;
            }
            for (int j = c0 + tid; j < c1; j += BT) {
                const double cj = (double)g.c[j];
                const double sv = g.invD2[j] * cj;
                q[2] += sv * sv;
                q[3] += cj * cj;
            }
            block_sum<4>(q, sh);
            if (tid == 0) {
                s_pscale = 1.0 + sqrt(q[0]);
                s_dscale = 1.0 + sqrt(q[2]);
                s_eta = g.prm.invnorm_scaling * (1.0 / sqrt(theta_d));
                const double cn = sqrt(q[3]), bn = sqrt(q[1]);
                s_omega = !pdlp ? 1.0
                        : (cn > g.prm.zero_tol && bn > g.prm.zero_tol) ? cn / bn : 1.0;
                s_eta_sum = 0.0;
            }
        }
        // ---- initial iterates: x = 0, y = 0 (solve(milp, algo), common.jl:203-209)
        for (int j = c0 + tid; j < c1; j += BT) {
            g.x[0][j] = T(0); g.x[1][j] = T(0); g.xa[0][j] = T(0); g.xa[1][j] = T(0);
            g.xr[j] = T(0); g.xbar[j] = T(0);
        }
        for (int i = r0 + tid; i < r1; i += BT) {
            g.y[0][i] = T(0); g.y[1][i] = T(0); g.ya[0][i] = T(0); g.ya[1][i] = T(0);
            g.yr[i] = T(0);
        }
        __syncthreads();
        int cur = 0;
        int32_t status = CPDLP_STILL_RUNNING;
        int32_t from_avg = 0;
        int64_t passes = 0, outer = 0, inner = 0, total = 0;
        bool restart_valid = false;
        cpdlp_kkt_errors e_cand{}, e_restart{}, e_sol{};
        if (L.m == 0 && L.zero_cost) {  // common.jl:194-198
            for (int j = c0 + tid; j < c1; j += BT) g.x[0][j] = proj_box(T(0), g.lv[j], g.uv[j]);
            status = CPDLP_OPTIMAL;
        }
        const double tlim_ns = g.prm.time_limit * 1e9;
        while (status == CPDLP_STILL_RUNNING) {
            // ---- check_every steps (pdlp.jl:96-124)
            for (int st = 0; st < g.prm.check_every; st++) {
                if (tid == 0) {
                    const double eta = s_eta, om = s_omega, es = s_eta_sum;
                    const double sigma = eta * om;
                    coef->tau = (T)(eta / om);
                    coef->sigma = (T)sigma;
                    coef->inv_sigma = (T)(1.0 / sigma);
                    coef->a = (T)(eta / (eta + es));
                    coef->b = (T)(es / (eta + es));
                    if (pdlp) s_eta_sum = es + eta;
                }
                __syncthreads();
                const int o = cur, nw = cur ^ 1;
                {
                    PrimalEpi<T> pe{g.x[o], g.c, g.lv, g.uv, g.x[nw], g.xbar, g.xa[o], g.xa[nw],
                                    coef, pdlp ? 1 : 0};
                    NoAcc a;
                    lp_tiles<ITEMS, T>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, g.y[o], pe, a, prod);
                }
                __syncthreads();
                {
                    DualEpi<T> de{g.y[o], g.lc, g.uc, g.y[nw], g.ya[o], g.ya[nw], coef, pdlp ? 1 : 0};
                    NoAcc a;
                    lp_tiles<ITEMS, T>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, g.xbar, de, a, prod);
                }
                __syncthreads();
                cur ^= 1;
            }
            passes += g.prm.check_every;
            if (pdlp) {
                inner += g.prm.check_every;
                total += g.prm.check_every;
            }
            // ---- KKT errors of sol, avg, sol_last, avg_last (errors.jl:65-109)
            const int nv = pdlp ? 4 : 1;
            for (int p = 0; p < nv; p++) {
                const T* xv = p == 0 ? g.x[cur] : p == 1 ? g.xa[cur] : p == 2 ? g.x[cur ^ 1] : g.xa[cur ^ 1];
                const T* yv = p == 0 ? g.y[cur] : p == 1 ? g.ya[cur] : p == 2 ? g.y[cur ^ 1] : g.ya[cur ^ 1];
                double rs[2], cs[3];
                {
                    KktRowEpi<T, 1> re;
                    re.lc = g.lc; re.uc = g.uc; re.invD1 = g.invD1; re.y[0] = yv;
                    re.block_out = red; re.long_out = g.longA;
                    typename KktRowEpi<T, 1>::Acc a;
                    re.init(a);
                    lp_tiles<ITEMS, T>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, xv, re, a, prod);
                    block_sum<2>(a.v, sh);
                    rs[0] = a.v[0]; rs[1] = a.v[1];
                }
                {
                    KktColEpi<T, 1> ce;
                    ce.c = g.c; ce.lv = g.lv; ce.uv = g.uv; ce.invD2 = g.invD2; ce.x[0] = xv;
                    ce.block_out = red; ce.long_out = g.longAt;
                    typename KktColEpi<T, 1>::Acc a;
                    ce.init(a);
                    lp_tiles<ITEMS, T>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, yv, ce, a, prod);
                    block_sum<3>(a.v, sh);
                    cs[0] = a.v[0]; cs[1] = a.v[1]; cs[2] = a.v[2];
                }
                if (tid == 0) {
                    for (int l = L.a_lid0; l < L.a_lid1; l++) {
                        rs[0] += g.longA[(size_t)l * 2];
                        rs[1] += g.longA[(size_t)l * 2 + 1];
                    }
                    for (int l = L.at_lid0; l < L.at_lid1; l++) {
                        cs[0] += g.longAt[(size_t)l * 3];
                        cs[1] += g.longAt[(size_t)l * 3 + 1];
                        cs[2] += g.longAt[(size_t)l * 3 + 2];
                    }
                    cpdlp_kkt_errors& e = s_e[p];
                    e.primal = sqrt(rs[0]);
                    e.primal_scale = s_pscale;
                    e.dual = sqrt(cs[0]);
                    e.dual_scale = s_dscale;
                    e.gap = fabs((cs[2] + rs[1]) + cs[1]);
                    e.gap_scale = (1.0 + fabs(rs[1] + cs[1])) + fabs(cs[2]);
                }
                __syncthreads();
            }
            // ---- termination (common.jl:218-231) and restart (pdlp.jl:138-196)
            if (tid == 0) {
                e_sol = s_e[0];
                const double elapsed = (double)(global_ns() - t_start);
                int32_t stt = CPDLP_STILL_RUNNING;
                if (rel_err(e_sol) <= g.prm.termination_reltol) stt = CPDLP_OPTIMAL;
                else if (elapsed >= tlim_ns) stt = CPDLP_TIME_LIMIT;
                else if (passes >= g.prm.max_kkt_passes) stt = CPDLP_ITERATION_LIMIT;
                int flag = 0;
                if (stt == CPDLP_STILL_RUNNING && pdlp) {
                    const double w = s_omega;
                    if (abs_err(s_e[0], w) < abs_err(s_e[1], w)) { from_avg = 0; e_cand = s_e[0]; }
                    else { from_avg = 1; e_cand = s_e[1]; }
                    const cpdlp_kkt_errors el = (abs_err(s_e[2], w) < abs_err(s_e[3], w)) ? s_e[2] : s_e[3];
                    flag = restart_valid ? 1 : 2;  // 2: the restart point's errors are needed first
                    if (restart_valid) {
                        const double ac = abs_err(e_cand, w), ar = abs_err(e_restart, w),
                                     acl = abs_err(el, w);
                        const bool restart = (ac <= g.prm.sufficient_decay * ar) ||
                                             ((ac <= g.prm.necessary_decay * ar) && (ac > acl)) ||
                                             ((double)inner >= g.prm.artificial_decay * (double)total);
                        flag = restart ? 3 : 0;
                    }
                    s_e[2] = el;
                }
                status = stt;
                s_flag = flag;
                sh[0] = (double)stt;
            }
            __syncthreads();
            status = (int32_t)sh[0];
            int flag = s_flag;
            __syncthreads();
            if (flag == 2) {
                // errors of the initial restart point (sol_restart = the start)
                double rs[2], cs[3];
                {
                    KktRowEpi<T, 1> re;
                    re.lc = g.lc; re.uc = g.uc; re.invD1 = g.invD1; re.y[0] = g.yr;
                    re.block_out = red; re.long_out = g.longA;
                    typename KktRowEpi<T, 1>::Acc a;
                    re.init(a);
                    lp_tiles<ITEMS, T>(g.A, L.a_t0, L.a_t1, L.a_l0, L.a_l1, g.xr, re, a, prod);
                    block_sum<2>(a.v, sh);
                    rs[0] = a.v[0]; rs[1] = a.v[1];
                }
                {
                    KktColEpi<T, 1> ce;
                    ce.c = g.c; ce.lv = g.lv; ce.uv = g.uv; ce.invD2 = g.invD2; ce.x[0] = g.xr;
                    ce.block_out = red; ce.long_out = g.longAt;
                    typename KktColEpi<T, 1>::Acc a;
                    ce.init(a);
                    lp_tiles<ITEMS, T>(g.At, L.at_t0, L.at_t1, L.at_l0, L.at_l1, g.yr, ce, a, prod);
                    block_sum<3>(a.v, sh);
                    cs[0] = a.v[0]; cs[1] = a.v[1]; cs[2] = a.v[2];
                }
                if (tid == 0) {
                    for (int l = L.a_lid0; l < L.a_lid1; l++) {
                        rs[0] += g.longA[(size_t)l * 2];
                        rs[1] += g.longA[(size_t)l * 2 + 1];
                    }
                    for (int l = L.at_lid0; l < L.at_lid1; l++) {
                        cs[0] += g.longAt[(size_t)l * 3];
                        cs[1] += g.longAt[(size_t)l * 3 + 1];
                        cs[2] += g.longAt[(size_t)l * 3 + 2];
                    }
                    e_restart.primal = sqrt(rs[0]);
                    e_restart.primal_scale = s_pscale;
                    e_restart.dual = sqrt(cs[0]);
                    e_restart.dual_scale = s_dscale;
                    e_restart.gap = fabs((cs[2] + rs[1]) + cs[1]);
                    e_restart.gap_scale = (1.0 + fabs(rs[1] + cs[1])) + fabs(cs[2]);
                    restart_valid = true;
                    const double w = s_omega;
                    const double ac = abs_err(e_cand, w), ar = abs_err(e_restart, w),
                                 acl = abs_err(s_e[2], w);
                    const bool restart = (ac <= g.prm.sufficient_decay * ar) ||
                                         ((ac <= g.prm.necessary_decay * ar) && (ac > acl)) ||
                                         ((double)inner >= g.prm.artificial_decay * (double)total);
                    s_flag = restart ? 3 : 0;
                }
                __syncthreads();
                flag = s_flag;
                __syncthreads();
            }
            if (flag == 3) {
                // restart! + primal_weight_update! (pdlp.jl:172-196, step_size.jl:58-75)
                const T* cx = from_avg ? g.xa[cur] : g.x[cur];
                const T* cy = from_avg ? g.ya[cur] : g.y[cur];
                double q[2] = {0.0, 0.0};
                for (int j = c0 + tid; j < c1; j += BT) {
                    const double d = (double)cx[j] - (double)g.xr[j];
                    q[0] += d * d;
                }
                for (int i = r0 + tid; i < r1; i += BT) {
                    const double d = (double)cy[i] - (double)g.yr[i];
                    q[1] += d * d;
                }
                block_sum<2>(q, sh);
                if (tid == 0) {
                    s_eta_sum = 0.0;
                    const double dx = sqrt(q[0]), dy = sqrt(q[1]), th = g.prm.primal_weight_damping;
                    if (dx > g.prm.zero_tol && dy > g.prm.zero_tol)
                        s_omega = exp(th * log(dy / dx) + (1.0 - th) * log(s_omega));
                    e_restart = e_cand;
                }
                for (int j = c0 + tid; j < c1; j += BT) {
                    const T v = cx[j];
                    g.x[cur][j] = v;
                    g.xr[j] = v;
                    g.xa[cur][j] = T(0);
                }
                for (int i = r0 + tid; i < r1; i += BT) {
                    const T v = cy[i];
                    g.y[cur][i] = v;
                    g.yr[i] = v;
                    g.ya[cur][i] = T(0);
                }
                outer += 1;
                inner = 0;
                __syncthreads();
            }
        }
        // ---- get_solution (common.jl:233-235): unscaled, double
        for (int j = c0 + tid; j < c1; j += BT) g.out_x[j] = g.D2[j] * (double)g.x[cur][j];
        for (int i = r0 + tid; i < r1; i += BT) g.out_y[i] = g.D1[i] * (double)g.y[cur][i];
        if (tid == 0) {
            R.err = (L.m == 0 && L.zero_cost) ? cpdlp_kkt_errors{NAN, NAN, NAN, NAN, NAN, NAN} : e_sol;
            R.kkt_passes = passes;
            R.outer = outer;
            R.inner = inner;
            R.total = total;
            R.eta = s_eta;
            R.omega = s_omega;
            R.eta_sum = s_eta_sum;
            R.time_elapsed = (double)(global_ns() - t_start) * 1e-9;
            R.status = status;
            R.restart_from_avg = from_avg;
            g.res[k] = R;
        }
        __syncthreads();
    }
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

template <class T>
void batch_T(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
             double* const* x_out, double* const* y_out, cpdlp_stats* stats) {
    cudaStream_t s = h.stream;
    const double t0 = now_seconds();
    // block-diagonal concatenation (1-based CSC)
    std::vector<int64_t> row_off(count + 1, 0), col_off(count + 1, 0), nz_off(count + 1, 0);
    for (int64_t k = 0; k < count; k++) {
        const cpdlp_lp& L = lps[k];
        if (L.m < 0 || L.n < 0 || L.nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative LP size in batch");
        row_off[k + 1] = row_off[k] + L.m;
        col_off[k + 1] = col_off[k] + L.n;
        nz_off[k + 1] = nz_off[k] + L.nnz;
    }
    const int64_t M = row_off[count], N = col_off[count], NZ = nz_off[count];
    if (M >= INT32_MAX || N >= INT32_MAX || NZ >= INT32_MAX)
        fail(CPDLP_ERR_UNSUPPORTED, "batch too large for int32 indices");
    std::vector<int64_t> colptr((size_t)N + 1), rowval((size_t)std::max<int64_t>(NZ, 1));
    std::vector<double> nzval((size_t)std::max<int64_t>(NZ, 1)), c((size_t)std::max<int64_t>(N, 1)),
        lv(c.size()), uv(c.size()), lc((size_t)std::max<int64_t>(M, 1)), uc(lc.size());
    colptr[0] = 1;
    for (int64_t k = 0; k < count; k++) {
        const cpdlp_lp& L = lps[k];
        if (!L.colptr || (L.nnz > 0 && (!L.rowval || !L.nzval)))
            fail(CPDLP_ERR_ARGUMENT, "null CSC array in batch");
        if (L.colptr[0] != 1 || L.colptr[L.n] != L.nnz + 1)
            fail(CPDLP_ERR_ARGUMENT, "invalid CSC column pointer in batch");
        for (int64_t j = 0; j < L.n; j++) colptr[col_off[k] + j + 1] = nz_off[k] + L.colptr[j + 1];
        for (int64_t q = 0; q < L.nnz; q++) {
            if (L.rowval[q] < 1 || L.rowval[q] > L.m)
                fail(CPDLP_ERR_ARGUMENT, "invalid CSC in batch: row index out of range");
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
    }
    cpdlp_lp big{M, N, NZ, colptr.data(), rowval.data(), nzval.data(), c.data(), lv.data(),
                 uv.data(), lc.data(), uc.data()};
    // rows were checked against each LP's own range above; monotone column
    // pointers and row order are validated by problem_create
    std::unique_ptr<ProblemBase> PB(problem_create(h, &big, params));
    auto& P = static_cast<ProblemT<T>&>(*PB);
    // tile plans with LP boundaries
    const int items = (NZ / std::max<int64_t>(count, 1) > 32 * 1024) ? 8 : 4;
    std::vector<int32_t> hpA((size_t)M + 1), hpAt((size_t)N + 1);
    CK(cudaMemcpyAsync(hpA.data(), P.a_ptr.p, sizeof(int32_t) * (M + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hpAt.data(), P.at_ptr.p, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    TilePlan planA, planAt;
    std::vector<int32_t> aT, aL, aI, atT, atL, atI;
    build_tile_plan(hpA, (int32_t)M, items, planA, s, &row_off, &aT, &aL, &aI);
    build_tile_plan(hpAt, (int32_t)N, items, planAt, s, &col_off, &atT, &atL, &atI);
    DBuf<T> partA((size_t)std::max(planA.npieces, 1)), partAt((size_t)std::max(planAt.npieces, 1));
    // per-LP descriptors
    const bool f32 = std::is_same<T, float>::value;
    std::vector<BatchLP> desc((size_t)count);
    for (int64_t k = 0; k < count; k++) {
        BatchLP& d = desc[(size_t)k];
        d.m = (int32_t)lps[k].m; d.n = (int32_t)lps[k].n;
        d.row_off = (int32_t)row_off[k]; d.col_off = (int32_t)col_off[k];
        d.a_t0 = aT[k]; d.a_t1 = aT[k + 1]; d.a_l0 = aL[k]; d.a_l1 = aL[k + 1];
        d.at_t0 = atT[k]; d.at_t1 = atT[k + 1]; d.at_l0 = atL[k]; d.at_l1 = atL[k + 1];
        d.a_lid0 = aI[k]; d.a_lid1 = aI[k + 1]; d.at_lid0 = atI[k]; d.at_lid1 = atI[k + 1];
        bool zc = true;
        for (int64_t j = 0; j < lps[k].n; j++)
            if (lps[k].c[j] != 0.0) { zc = false; break; }
        d.zero_cost = zc ? 1 : 0;
        d.power_tol = params->power_tol_override > 0 ? params->power_tol_override : powm_tol(d.n, f32);
        d.power_maxiter = params->power_maxiter_override > 0 ? params->power_maxiter_override : d.n;
    }
    // power-method start vectors: the single-LP generator, per LP from counter 0
    std::vector<double> xs((size_t)std::max<int64_t>(N, 1));
    for (int64_t k = 0; k < count; k++) {
        for (int64_t j = 0; j < lps[k].n; j++) {
            const double u1 = (double)((splitmix64_at_host(params->power_seed, 2 * (uint64_t)j) >> 11) + 1) *
                              (1.0 / 9007199254740992.0);
            const double u2 = (double)((splitmix64_at_host(params->power_seed, 2 * (uint64_t)j + 1) >> 11) + 1) *
                              (1.0 / 9007199254740992.0);
            xs[(size_t)(col_off[k] + j)] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        }
    }
    // device buffers
    const size_t nz = (size_t)std::max<int64_t>(N, 1), mz = (size_t)std::max<int64_t>(M, 1);
    DBuf<T> bx[2], by[2], bxa[2], bya[2], bxr(nz), byr(mz), bxbar(nz);
    for (int b = 0; b < 2; b++) { bx[b].alloc(nz); by[b].alloc(mz); bxa[b].alloc(nz); bya[b].alloc(mz); }
    DBuf<double> d_xs(nz), d_outx(nz), d_outy(mz);
    DBuf<BatchLP> d_desc((size_t)std::max<int64_t>(count, 1));
    DBuf<BatchResult> d_res((size_t)std::max<int64_t>(count, 1));
    DBuf<double> longA((size_t)std::max(planA.nlong, 1) * 2), longAt((size_t)std::max(planAt.nlong, 1) * 3);
    DBuf<int> d_next(1);
    CK(cudaMemcpyAsync(d_xs.p, xs.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_desc.p, desc.data(), sizeof(BatchLP) * desc.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d_next.p, 0, sizeof(int), s));
    int per_sm = 0;
    auto kern = (items == 8) ? k_batch_pdlp<8, T> : k_batch_pdlp<4, T>;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT, 0));
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(count, (int64_t)std::max(per_sm, 1) * h.num_sms));
    DBuf<double> d_red((size_t)grid * 32);
    DBuf<StepCoef<T>> d_coef((size_t)grid);
    BatchArgs<T> g;
    g.A = CsrView<T, T>{P.a_ptr.p, P.a_idx.p, P.a_val.p, planA.tasks.p, planA.ntasks,
                        planA.ltasks.p, planA.nltasks, planA.counters.p, partA.p};
    g.At = CsrView<T, T>{P.at_ptr.p, P.at_idx.p, P.at_val.p, planAt.tasks.p, planAt.ntasks,
                         planAt.ltasks.p, planAt.nltasks, planAt.counters.p, partAt.p};
    g.c = P.c.p; g.lv = P.lv.p; g.uv = P.uv.p; g.lc = P.lc.p; g.uc = P.uc.p;
    g.invD1 = P.invD1.p; g.invD2 = P.invD2.p; g.D1 = P.D1.p; g.D2 = P.D2.p;
    for (int b = 0; b < 2; b++) { g.x[b] = bx[b].p; g.y[b] = by[b].p; g.xa[b] = bxa[b].p; g.ya[b] = bya[b].p; }
    g.xr = bxr.p; g.yr = byr.p; g.xbar = bxbar.p;
    g.x_start = d_xs.p;
    g.lps = d_desc.p; g.res = d_res.p; g.out_x = d_outx.p; g.out_y = d_outy.p;
    g.red = d_red.p; g.longA = longA.p; g.longAt = longAt.p; g.coef = d_coef.p;
    g.next = d_next.p; g.count = (int32_t)count;
    g.prm = BatchParams{params->algorithm, params->check_every > 0 ? params->check_every : 100,
                        params->max_kkt_passes, params->termination_reltol,
                        params->time_limit - (now_seconds() - t0), params->invnorm_scaling,
                        params->primal_weight_damping, params->zero_tol, params->sufficient_decay,
                        params->necessary_decay, params->artificial_decay};
    const double setup = now_seconds() - t0;
    kern<<<(unsigned)grid, BT, 0, s>>>(g);
    CK_LAUNCH();
    std::vector<BatchResult> res((size_t)count);
    std::vector<double> ox(nz), oy(mz);
    CK(cudaMemcpyAsync(res.data(), d_res.p, sizeof(BatchResult) * count, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ox.data(), d_outx.p, sizeof(double) * nz, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(oy.data(), d_outy.p, sizeof(double) * mz, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int64_t k = 0; k < count; k++) {
        if (x_out && x_out[k]) std::copy(ox.begin() + col_off[k], ox.begin() + col_off[k + 1], x_out[k]);
        if (y_out && y_out[k]) std::copy(oy.begin() + row_off[k], oy.begin() + row_off[k + 1], y_out[k]);
        if (stats) {
            cpdlp_stats& st = stats[k];
            const BatchResult& r = res[(size_t)k];
            memset(&st, 0, sizeof(st));
            st.err = r.err;
            st.time_elapsed = r.time_elapsed;
            st.kkt_passes = r.kkt_passes;
            st.termination_status = r.status;
            st.restart_from_avg = r.restart_from_avg;
            st.outer = r.outer; st.inner = r.inner; st.total = r.total;
            st.eta = r.eta; st.eta_sum = r.eta_sum; st.omega = r.omega;
            st.power_iterations = r.power_iterations;
            st.setup_seconds = setup;
            st.kernel_launches = 1;
        }
    }
}

}  // namespace

void batch_solve(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 double* const* x_out, double* const* y_out, cpdlp_stats* stats) {
    if (count == 0) return;
    if (params->check_every <= 0) fail(CPDLP_ERR_ARGUMENT, "check_every must be positive");
    if (params->float_type == CPDLP_VAL_F32) batch_T<float>(h, count, lps, params, x_out, y_out, stats);
    else if (params->float_type == CPDLP_VAL_F64) batch_T<double>(h, count, lps, params, x_out, y_out, stats);
    else fail(CPDLP_ERR_ARGUMENT, "float_type must be CPDLP_VAL_F64 or CPDLP_VAL_F32");
}

}  // namespace cpdlp
