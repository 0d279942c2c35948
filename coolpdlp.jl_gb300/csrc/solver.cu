// solver.cu -- single-LP PDLP / PDHG on one GB300.
//
// Per PDHG step two fused kernels run (pdlp.jl:96-124):
//   primal: s = (A' y)_j (warp tiles over the rows of A')  ->
//           x+ = proj_box(x - tau*(c - s), lv, uv), xbar = 2x+ - x,
//           avg_x = a*x+ + b*avg_x_last                      (pdlp.jl:110-113, :126-136)
//   dual:   s = (A xbar)_i (warp tiles over the rows of A)  ->
//           y+ = y - sigma*s - sigma*proj_box(y/sigma - s, -uc, -lc),
//           avg_y = a*y+ + b*avg_y_last                      (pdlp.jl:115-117)
// Iterates ping-pong between two buffers (the reference swaps sol/sol_last,
// pdlp.jl:101, and copies avg into avg_last, :129; here the average ping-pongs
// too).  check_every steps are captured once as a CUDA graph per buffer parity.
// Every check evaluates the KKT errors of sol, avg, sol_last and avg_last in
// ONE pass over both matrices (four gathered vectors per nonzero), with FP64
// accumulation, a deterministic block-then-tree reduction and one small
// device->host read; restart and termination decisions run on the host in
// FP64 exactly as restart.jl:40-57, termination.jl:89-101 state them.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <exception>
#include <chrono>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <memory>
#include <type_traits>

#include "ell.cuh"
#include "epilogues.cuh"
#include "solver.cuh"

namespace cpdlp {

double now_seconds() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

namespace {

constexpr int RED_THREADS = TILE_WARPS * 32;
int trace_level();  // CPDLP_TRACE (defined with the refinement's traces)

// ---------------------------------------------------------------------------
// preconditioning kernels (FP64, preconditioning.jl:37-155)
// ---------------------------------------------------------------------------
enum NormKind { NK_INF = 0, NK_ONE = 1, NK_TWO = 2, NK_ZERO = 3, NK_P = 4 };

// d[r] = 1/sqrt(norm(row r)), 1 when the norm is zero (preconditioning.jl:102-111).
// One warp per 32 consecutive rows.  Rows of at most 64 entries are summed by
// one lane sequentially in storage order, like the reference's column_norm
// (linalg.jl:98-99) on short columns, so they match the oracle bit for bit;
// longer rows are reduced by the whole warp (lane-strided partials, fixed
// shuffle tree), as the reference's BLAS-backed norm also reorders long sums.
__device__ __forceinline__ double norm_term(int kind, double x, double p) {
    switch (kind) {
        case NK_ONE: return fabs(x);
        case NK_TWO: return __dmul_rn(x, x);
        case NK_ZERO: return (x != 0.0) ? 1.0 : 0.0;
        case NK_P: return pow(fabs(x), p);
        default: return fabs(x);
    }
}
__device__ __forceinline__ double norm_finish(int kind, double s, double p, bool nonempty) {
    if (kind == NK_TWO) return sqrt(s);
    if (kind == NK_P && nonempty) return pow(s, 1.0 / p);
    return s;
}
__global__ void k_row_norm_scale(const int32_t* __restrict__ ptr, const double* __restrict__ v,
                                 int64_t rows, int kind, double p, double* __restrict__ d) {
    const int lane = threadIdx.x & 31;
    const int64_t r0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane);
    if (r0 >= rows) return;
    const int64_t r = r0 + lane;
    int a = 0, b = 0;
    if (r < rows) {
        a = ptr[r];
        b = ptr[r + 1];
        if (b - a <= 64) {
            double s = 0.0;
            for (int k = a; k < b; k++) {
                const double t = norm_term(kind, v[k], p);
                s = (kind == NK_INF) ? jl_max(s, t) : __dadd_rn(s, t);
            }
            s = norm_finish(kind, s, p, b > a);
            d[r] = (s == 0.0) ? 1.0 : 1.0 / sqrt(s);
        }
    }
    unsigned longs = __ballot_sync(0xffffffffu, r < rows && b - a > 64);
    while (longs) {
        const int l = __ffs(longs) - 1;
        longs &= longs - 1;
        const int la = __shfl_sync(0xffffffffu, a, l), lb = __shfl_sync(0xffffffffu, b, l);
        double s = 0.0;
        for (int k = la + lane; k < lb; k += 32) {
            const double t = norm_term(kind, v[k], p);
            s = (kind == NK_INF) ? jl_max(s, t) : __dadd_rn(s, t);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(0xffffffffu, s, o);
            s = (kind == NK_INF) ? jl_max(s, t) : __dadd_rn(s, t);
        }
        if (lane == 0) {
            s = norm_finish(kind, s, p, true);
            d[r0 + l] = (s == 0.0) ? 1.0 : 1.0 / sqrt(s);
        }
    }
}

// A_p = D1*A*D2 on A's CSC values (S1 order): (d1_i * a_ij) * d2_j
__global__ void k_scale_S1(const int32_t* __restrict__ idx1, const int32_t* __restrict__ col1,
                           const double* __restrict__ vin, const double* __restrict__ d1,
                           const double* __restrict__ d2, double* __restrict__ vout, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) vout[k] = __dmul_rn(__dmul_rn(d1[idx1[k]], vin[k]), d2[col1[k]]);
}
// At_p = D2*At*D1 on At's CSC values (S2 order): (d2_j * a_ij) * d1_i
__global__ void k_scale_S2(const int32_t* __restrict__ idx2, const int32_t* __restrict__ row2,
                           const double* __restrict__ vin, const double* __restrict__ d1,
                           const double* __restrict__ d2, double* __restrict__ vout, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) vout[k] = __dmul_rn(__dmul_rn(d2[idx2[k]], vin[k]), d1[row2[k]]);
}
// r[i] = d[i] * r[i]  (products of diagonal preconditioners commute exactly)
__global__ void k_mul_into(double* __restrict__ r, const double* __restrict__ d, int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) r[i] = __dmul_rn(d[i], r[i]);
}
__global__ void k_fill(double* __restrict__ r, double v, int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) r[i] = v;
}
__global__ void k_invert_perm(const int32_t* __restrict__ p21, int32_t* __restrict__ p12, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) p12[p21[k]] = (int32_t)k;
}
// narrow +-1 storage: the index of a -1 entry becomes ~col (sign of v[k])
__global__ void k_encode_sign(int32_t* __restrict__ idx, const double* __restrict__ v, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz && v[k] < 0.0) idx[k] = ~idx[k];
}
template <class T>
__global__ void k_narrow(const double* __restrict__ v, T* __restrict__ out, int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = (T)v[i];
}
// out = a .* b (the pre-scaled copies D2 x, D1 y of a narrow matrix's products)
template <class T>
__global__ void k_mul_vec(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out,
                          int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = mul_rn(a[i], b[i]);
}
// The gathered vectors of a KKT pass: NV iterates interleaved (X[NV*j + p] =
// x_p[j]), times the narrow matrix's column scale d (D2 for x, D1 for y) when
// d is non-null; y alike.  With NV = 4 one request per nonzero gathers all four.
template <class T, int NV>
struct PackSrc {
    const T* v[NV];
};
template <class T, int NV>
__global__ void k_pack(PackSrc<T, NV> xs, const T* __restrict__ dx, int64_t n, T* __restrict__ X,
                       PackSrc<T, NV> ys, const T* __restrict__ dy, int64_t m,
                       T* __restrict__ Y) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const T d = dx ? dx[j] : T(1);
#pragma unroll
        for (int p = 0; p < NV; p++) X[NV * j + p] = dx ? mul_rn(xs.v[p][j], d) : xs.v[p][j];
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const T d = dy ? dy[i] : T(1);
#pragma unroll
        for (int p = 0; p < NV; p++) Y[NV * i + p] = dy ? mul_rn(ys.v[p][i], d) : ys.v[p][i];
    }
}
// Infeasibility certificates (an extension): the rays are the change of the
// iterates since the previous check, x projected onto the recession cone of
// [lv, uv] and y onto the multiplier cone of [lc, uc] (>= 0 with only lc
// finite, <= 0 with only uc finite, 0 for a free row); FP64.  rxs / rys
// (narrow storage): D2 .* rx and D1 .* ry, the vectors its products gather.
template <class T>
__global__ void k_ray(const T* __restrict__ x, const T* __restrict__ xp, const T* __restrict__ lv,
                      const T* __restrict__ uv, double* __restrict__ rx, double* __restrict__ rxs,
                      const double* __restrict__ D2, int64_t n, const T* __restrict__ y,
                      const T* __restrict__ yp, const T* __restrict__ lc,
                      const T* __restrict__ uc, double* __restrict__ ry,
                      double* __restrict__ rys, const double* __restrict__ D1, int64_t m) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        double d = __dsub_rn((double)x[j], (double)xp[j]);
        const bool lo = !isinf((double)lv[j]), up = !isinf((double)uv[j]);
        d = (lo && up) ? 0.0 : lo ? fmax(d, 0.0) : up ? fmin(d, 0.0) : d;
        rx[j] = d;
        if (rxs) rxs[j] = __dmul_rn(D2[j], d);
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double d = __dsub_rn((double)y[i], (double)yp[i]);
        const bool lo = !isinf((double)lc[i]), up = !isinf((double)uc[i]);
        d = (lo && up) ? d : lo ? fmax(d, 0.0) : up ? fmin(d, 0.0) : 0.0;
        ry[i] = d;
        if (rys) rys[i] = __dmul_rn(D1[i], d);
    }
}
// precondition(milp, prec) on the vectors (preconditioning.jl:61-91)
template <class T>
__global__ void k_scale_vec_n(const double* __restrict__ c, const double* __restrict__ lv,
                              const double* __restrict__ uv, const double* __restrict__ D2,
                              T* __restrict__ co, T* __restrict__ lvo, T* __restrict__ uvo,
                              double* __restrict__ invD2, int64_t n) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double d = D2[j];
    co[j] = (T)__dmul_rn(d, c[j]);
    lvo[j] = (T)__ddiv_rn(lv[j], d);
    uvo[j] = (T)__ddiv_rn(uv[j], d);
    invD2[j] = __drcp_rn(d);
}
template <class T>
__global__ void k_scale_vec_m(const double* __restrict__ lc, const double* __restrict__ uc,
                              const double* __restrict__ D1, T* __restrict__ lco, T* __restrict__ uco,
                              double* __restrict__ invD1, int64_t m) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const double d = D1[i];
    lco[i] = (T)__dmul_rn(d, lc[i]);
    uco[i] = (T)__dmul_rn(d, uc[i]);
    invD1[i] = __drcp_rn(d);
}
// constant parts of the KKT errors and of primal_weight_init:
// q0 = sum (invD1*combine(lc,uc))^2, q1 = sum combine(lc,uc)^2 (m side)
// q2 = sum (invD2*c)^2, q3 = sum c^2 (n side)
template <class T>
__global__ void k_scales(const T* __restrict__ lc, const T* __restrict__ uc,
                         const double* __restrict__ invD1, int64_t m, const T* __restrict__ c,
                         const double* __restrict__ invD2, int64_t n, double* __restrict__ part) {
    double acc[4] = {0, 0, 0, 0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double cb = combine((double)lc[i], (double)uc[i]);
        double s = invD1[i] * cb;
        acc[0] += s * s;
        acc[1] += cb * cb;
    }
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        double cj = (double)c[j];
        double s = invD2[j] * cj;
        acc[2] += s * s;
        acc[3] += cj * cj;
    }
    block_reduce_store<4>(acc, part);
}

// ---------------------------------------------------------------------------
// epilogues of the tile engine
// ---------------------------------------------------------------------------
// One power-method iteration is captured as a graph and runs without the host:
//   k_power_theta:    theta = x.Ax, inv = 1/||Ax|| from the reduced partials
//   k_power_residual: r = Ax - theta*x, x = Ax * inv (block partials of ||r||^2)
//   k_power_finish:   ||r||, then the iteration's (theta, ||r||) go to slot it % depth
//                     of a mapped host ring and the device iteration counter advances
// so the host can queue several iterations ahead and check each one's stopping
// rule when its slot is written (powm!, linalg.jl:86-96, IterativeSolvers 0.9.4).
struct PowerSlot {
    double theta, residual;
};
__global__ void k_power_theta(const double* __restrict__ q, double* __restrict__ scal,
                              const int* __restrict__ it, PowerSlot* ring, int depth) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double theta = q[0];
        const double nrm = sqrt(q[1]);
        scal[0] = theta;
        scal[1] = 1.0 / nrm;
        ring[*it % depth].theta = theta;
    }
}
// (d2, xs non-null: a narrow matrix, whose first product gathers xs = d2 .* x)
__global__ void __launch_bounds__(RED_THREADS)
    k_power_residual(double* __restrict__ x, const double* __restrict__ Ax,
                     const double* __restrict__ scal, int64_t n, double* __restrict__ part,
                     const double* __restrict__ d2, double* __restrict__ xs) {
    const double theta = scal[0], inv = scal[1];
    double acc[1] = {0.0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const double r = add_rn(mul_rn(-theta, x[j]), Ax[j]);
        acc[0] += r * r;
        const double xn = mul_rn(Ax[j], inv);
        x[j] = xn;
        if (xs) xs[j] = mul_rn(d2[j], xn);
    }
    block_reduce_store<1>(acc, part);
}
__global__ void k_power_finish(const double* __restrict__ r2, int* it, PowerSlot* ring,
                               int depth) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ring[*it % depth].residual = sqrt(r2[0]);
        __threadfence_system();
        *it += 1;
    }
}

// ||a - b||^2 over x (n) and y (m): primal_weight_update! (step_size.jl:58-75)
template <class T>
__global__ void __launch_bounds__(RED_THREADS)
    k_diff_norms(const T* __restrict__ ax, const T* __restrict__ bx, int64_t n,
                 const T* __restrict__ ay, const T* __restrict__ by, int64_t m,
                 double* __restrict__ part) {
    double acc[2] = {0.0, 0.0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        double d = (double)ax[j] - (double)bx[j];
        acc[0] += d * d;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double d = (double)ay[i] - (double)by[i];
        acc[1] += d * d;
    }
    block_reduce_store<2>(acc, part);
}

template <class T>
__global__ void k_unscale(const T* __restrict__ v, const double* __restrict__ D, double* __restrict__ out,
                          int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = __dmul_rn(D[i], (double)v[i]);
}
template <class T>
__global__ void k_prescale(const double* __restrict__ v, const double* __restrict__ D, T* __restrict__ out,
                           int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = (T)__ddiv_rn(v[i], D[i]);
}
template <class T>
__global__ void k_widen(const T* __restrict__ v, double* __restrict__ out, int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = (double)v[i];
}
template <class T>
__global__ void k_proj_zero(T* __restrict__ x, const T* __restrict__ lv, const T* __restrict__ uv, int64_t n) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) x[j] = proj_box(T(0), lv[j], uv[j]);
}

inline unsigned red_grid(Handle& h, int64_t items) {
    int64_t g = (items + RED_THREADS - 1) / RED_THREADS;
    int64_t cap = (int64_t)(h.num_sms > 0 ? h.num_sms : 152) * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

template <class T>
CsrView<T, T> view_A(ProblemT<T>& P) {
    return CsrView<T, T>{P.a_ptr.p, P.a_idx.p, P.a_val.p, P.planA.tasks.p, P.planA.ntasks,
                         P.planA.ltasks.p, P.planA.nltasks, P.planA.counters.p, P.partA.p};
}
template <class T>
CsrView<T, T> view_At(ProblemT<T>& P) {
    return CsrView<T, T>{P.at_ptr.p, P.at_idx.p, P.at_val.p, P.planAt.tasks.p, P.planAt.ntasks,
                         P.planAt.ltasks.p, P.planAt.nltasks, P.planAt.counters.p, P.partAt.p};
}
// the same matrices in narrow +-1 storage (signs in the indices, no values)
template <class T>
CsrView<Pm1, T> view_A_pm1(ProblemT<T>& P) {
    return CsrView<Pm1, T>{P.a_ptr.p, P.a_idx.p, nullptr, P.planA.tasks.p, P.planA.ntasks,
                           P.planA.ltasks.p, P.planA.nltasks, P.planA.counters.p, P.partA.p};
}
template <class T>
CsrView<Pm1, T> view_At_pm1(ProblemT<T>& P) {
    return CsrView<Pm1, T>{P.at_ptr.p, P.at_idx.p, nullptr, P.planAt.tasks.p, P.planAt.ntasks,
                           P.planAt.ltasks.p, P.planAt.nltasks, P.planAt.counters.p, P.partAt.p};
}

// ---- the product of one matrix of the problem (side 0: rows of A, the dual
// step; side 1: rows of A', the primal step) in its chosen format ----------
template <class T>
int64_t side_rows(const ProblemT<T>& P, int side) { return side == 0 ? P.m : P.n; }

// blocks of a launch over `side` with `warps` warps per block (the
// block-partial rows of a reducing epilogue; its long-row outputs follow)
template <class T>
int64_t side_blocks(const ProblemT<T>& P, int side, int warps) {
    if (P.fmt[side] == CPDLP_FMT_ELL) return side_rows(P, side) > 0 ? ell_grid(side_rows(P, side), warps) : 0;
    return tiles_grid(side == 0 ? P.planA : P.planAt, warps);
}
// all partial rows a reducing epilogue writes over `side`
template <class T>
int64_t side_partials(const ProblemT<T>& P, int side, int warps) {
    const int64_t longs = P.fmt[side] == CPDLP_FMT_ELL ? 0 : (side == 0 ? P.planA : P.planAt).nlong;
    return side_blocks(P, side, warps) + longs;
}
// the same for the four-iterate pass (its grid capped at P.kkt4_cap blocks)
template <class T>
int64_t side_blocks4(const ProblemT<T>& P, int side, int warps) {
    if (P.fmt[side] == CPDLP_FMT_ELL)
        return side_rows(P, side) > 0 ? ell4_grid(side_rows(P, side), warps, P.kkt4_cap) : 0;
    const TilePlan& pl = side == 0 ? P.planA : P.planAt;
    return (pl.ntasks + pl.nltasks) > 0 ? tiles4_grid(pl, warps, P.kkt4_cap) : 0;
}
template <class T>
int64_t side_partials4(const ProblemT<T>& P, int side, int warps) {
    const int64_t longs = P.fmt[side] == CPDLP_FMT_ELL ? 0 : (side == 0 ? P.planA : P.planAt).nlong;
    return side_blocks4(P, side, warps) + longs;
}

template <class V, class VT, class T>
EllView<V, VT> ell_view(const ProblemT<T>& P, int side, const int32_t* ptr) {
    const V* val = nullptr;
    if constexpr (!is_pm1<V>::value) val = P.ell_val[side].p;
    return EllView<V, VT>{ptr, P.ell_idx[side].p, val, side_rows(P, side)};
}

// One product over `side` with the fused epilogue `epi`, in the side's
// format: the CSR view's tile plan, or the ELL slabs (the view's row pointer
// gives the row lengths).  W: warps per block (the epilogue's block size).
template <int W = TILE_WARPS, int NVEC, class V, class VT, class Epi, class T>
void launch_side(const ProblemT<T>& P, int side, const CsrView<V, VT>& view,
                 const VecSet<VT, NVEC>& xs, const Epi& epi, cudaStream_t s) {
    if (P.fmt[side] == CPDLP_FMT_ELL)
        launch_ell<W>(ell_view<V, VT>(P, side, view.ptr), xs, epi, s);
    else
        launch_tiles_w<W>(side == 0 ? P.planA : P.planAt, view, xs, epi, s);
}
// four packed iterates (the KKT pass)
template <int W, class V, class VT, class Epi, class T>
void launch_side4(const ProblemT<T>& P, int side, const CsrView<V, VT>& view, const VT* x4,
                  const Epi& epi, cudaStream_t s) {
    if (P.fmt[side] == CPDLP_FMT_ELL)
        launch_ell4<W>(ell_view<V, VT>(P, side, view.ptr), x4, epi, P.kkt4_cap, s);
    else
        launch_tiles4<W>(side == 0 ? P.planA : P.planAt, view, x4, epi, P.kkt4_cap, s);
}

// the ELL slabs of a CSR (0-based; narrow storage keeps the signed index):
// entry k of row r at r + k*rows, padding index 0 and value 0 (never read)
template <class T>
__global__ void k_csr_to_ell(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const T* __restrict__ val, int64_t rows, int64_t width,
                             int32_t* __restrict__ eidx, T* __restrict__ eval) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int a = ptr[r], len = ptr[r + 1] - a;
    for (int64_t k = 0; k < width; k++) {
        const bool in = k < len;
        eidx[r + k * rows] = in ? idx[a + k] : 0;
        if (eval) eval[r + k * rows] = in ? val[a + k] : T(0);
    }
}
template <class T>
void build_ell(Handle& h, ProblemT<T>& P, int side, const std::vector<int32_t>& hp) {
    const int64_t rows = side_rows(P, side);
    int64_t width = 0;
    for (int64_t r = 0; r < rows; r++) width = std::max<int64_t>(width, hp[r + 1] - hp[r]);
    const size_t slots = (size_t)std::max<int64_t>(rows * width, 1);
    P.ell_width[side] = width;
    P.ell_idx[side].alloc(slots);
    if (!P.pm1) P.ell_val[side].alloc(slots);
    if (rows > 0 && width > 0) {
        k_csr_to_ell<T><<<grid_for(rows, 256), 256, 0, h.stream>>>(
            side == 0 ? P.a_ptr.p : P.at_ptr.p, side == 0 ? P.a_idx.p : P.at_idx.p,
            P.pm1 ? nullptr : (side == 0 ? P.a_val.p : P.at_val.p), rows, width,
            P.ell_idx[side].p, P.pm1 ? nullptr : P.ell_val[side].p);
        CK_LAUNCH();
    }
}

// Autotuner of one matrix's product (side 0: rows of A, side 1: rows of A'):
// each candidate -- CSR tile shapes (nonzeros per lane) and, when allowed,
// ELL -- runs the fused step kernel that uses the matrix (the primal step for
// A', the dual step for A) on scratch vectors, timed with CUDA events on the
// handle's stream.  The heuristic's tile shape is kept unless another
// candidate is at least 3% faster.  Decisions are cached per matrix shape and
// requested format for the process.  With ELL chosen the slabs stay in P.
constexpr int64_t AUTOTUNE_MIN_NNZ = 1 << 21;
// ELL is a candidate when its slabs hold at most this many times the nonzeros
constexpr int64_t ELL_MAX_PADDING = 3;

struct SideChoice {
    int fmt;
    int items;
};

template <class T, class Launch>
SideChoice tune_side(Handle& h, ProblemT<T>& P, int side, const std::vector<int32_t>& hp,
                     int heuristic, bool try_csr, bool try_ell, int which, Launch&& launch) {
    static std::mutex mu;
    static std::map<std::tuple<int64_t, int64_t, int64_t, int, int, int, int>, SideChoice> cache;
    const int64_t rows = side_rows(P, side), cols = side_rows(P, 1 - side);
    const auto key = std::make_tuple(rows, cols, P.nnz, (int)sizeof(T), h.device, which,
                                     (int)try_csr * 2 + (int)try_ell);
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            if (it->second.fmt == CPDLP_FMT_ELL) {
                build_ell(h, P, side, hp);
                P.fmt[side] = CPDLP_FMT_ELL;
            }
            return it->second;
        }
    }
    cudaStream_t s = h.stream;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    SideChoice best{try_csr ? CPDLP_FMT_CSR : CPDLP_FMT_ELL, heuristic};
    float best_ms = INFINITY;
    auto timed = [&](int fmt, TilePlan& pl, T* part) {
        launch(fmt, pl, part);
        CK(cudaEventRecord(e0, s));
        for (int r = 0; r < 4; r++) launch(fmt, pl, part);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
    };
    try {
        if (try_csr) {
            const int cands[3] = {heuristic, heuristic == 4 ? 8 : 4, heuristic == 16 ? 8 : 16};
            for (int items : cands) {
                TilePlan plan;
                build_tile_plan(hp, (int32_t)rows, items, plan, s);
                DBuf<T> part((size_t)std::max(plan.npieces, 1));
                const float ms = timed(CPDLP_FMT_CSR, plan, part.p);
                if (items == heuristic ? ms < best_ms : ms < 0.97f * best_ms) {
                    best_ms = ms;
                    best = SideChoice{CPDLP_FMT_CSR, items};
                }
            }
        }
        if (try_ell) {
            build_ell(h, P, side, hp);
            P.fmt[side] = CPDLP_FMT_ELL;
            TilePlan none;
            const float ms = timed(CPDLP_FMT_ELL, none, nullptr);
            if (!try_csr || ms < 0.97f * best_ms) {
                best_ms = ms;
                best = SideChoice{CPDLP_FMT_ELL, heuristic};
            } else {
                P.fmt[side] = CPDLP_FMT_CSR;
                P.ell_idx[side] = DBuf<int32_t>();
                P.ell_val[side] = DBuf<T>();
                P.ell_width[side] = 0;
            }
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = best;
    return best;
}

// device reduction of (rows x q) partials into host doubles
void fetch_reduced(Handle& h, const double* part, int64_t rows, int q, double* dev_out,
                   double* host_out) {
    reduce_partials(part, rows, q, dev_out, h.stream);
    double* pin = h.pinned_area(sizeof(double) * 64);
    CK(cudaMemcpyAsync(pin, dev_out, sizeof(double) * q, cudaMemcpyDeviceToHost, h.stream));
    CK(cudaStreamSynchronize(h.stream));
    memcpy(host_out, pin, sizeof(double) * q);
}

// ---------------------------------------------------------------------------
// density order: the order of the reference's sort_rows_columns
// (permutation.jl:1-46) -- rows and columns by increasing length, ties in
// index order (Julia's stable sortperm) -- applied inside the solver
// ---------------------------------------------------------------------------
// A problem's matrices in density order (internal row i = row orow[i] of A,
// internal column j = column ocol[j]), built next to the problem's own
template <class T>
struct DensityOrder {
    std::vector<int32_t> hp2, hp1;   // row pointers of A and A' in the new order
    DBuf<int32_t> orow, ocol;        // new -> old
    DBuf<int32_t> a_ptr, a_idx, at_ptr, at_idx;
    DBuf<T> a_val, at_val;
};

template <class T>
void build_density_order(Handle& h, const ProblemT<T>& P, DensityOrder<T>& o) {
    cudaStream_t s = h.stream;
    const int64_t m = P.m, n = P.n, nnz = P.nnz;
    const size_t mz = (size_t)std::max<int64_t>(m, 1), nz = (size_t)std::max<int64_t>(n, 1),
                 zn = (size_t)std::max<int64_t>(nnz, 1);
    // stable sorts of the row lengths on the device (rows of A: the constraints,
    // rows of A': the variables)
    DBuf<int32_t> dirow(mz), dicol(nz);
    o.orow.alloc(mz);
    o.ocol.alloc(nz);
    order_by_length(P.a_ptr.p, m, nnz, o.orow.p, dirow.p, s);
    order_by_length(P.at_ptr.p, n, nnz, o.ocol.p, dicol.p, s);
    o.a_ptr.alloc((size_t)m + 1);
    o.at_ptr.alloc((size_t)n + 1);
    // index arrays carry the tile engine's 16 padding elements, value arrays PAD_ELEMS
    o.a_idx.alloc(zn + 16);
    o.at_idx.alloc(zn + 16);
    CK(cudaMemsetAsync(o.a_idx.p, 0, sizeof(int32_t) * (zn + 16), s));
    CK(cudaMemsetAsync(o.at_idx.p, 0, sizeof(int32_t) * (zn + 16), s));
    if (!P.pm1) {
        o.a_val.alloc(zn + PAD_ELEMS);
        o.at_val.alloc(zn + PAD_ELEMS);
        CK(cudaMemsetAsync(o.a_val.p, 0, sizeof(T) * (zn + PAD_ELEMS), s));
        CK(cudaMemsetAsync(o.at_val.p, 0, sizeof(T) * (zn + PAD_ELEMS), s));
    }
    reorder_csr<T>(P.a_ptr.p, P.a_idx.p, P.pm1 ? nullptr : P.a_val.p, m, nnz, o.orow.p, dicol.p,
                   o.a_ptr.p, o.a_idx.p, P.pm1 ? nullptr : o.a_val.p, s);
    reorder_csr<T>(P.at_ptr.p, P.at_idx.p, P.pm1 ? nullptr : P.at_val.p, n, nnz, o.ocol.p, dirow.p,
                   o.at_ptr.p, o.at_idx.p, P.pm1 ? nullptr : o.at_val.p, s);
    o.hp2.assign((size_t)m + 1, 0);
    o.hp1.assign((size_t)n + 1, 0);
    CK(cudaMemcpyAsync(o.hp2.data(), o.a_ptr.p, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(o.hp1.data(), o.at_ptr.p, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
}

// exchanges the problem's matrices with the reordered ones
template <class T>
void swap_matrices(ProblemT<T>& P, DensityOrder<T>& o) {
    std::swap(P.a_ptr, o.a_ptr);
    std::swap(P.a_idx, o.a_idx);
    std::swap(P.at_ptr, o.at_ptr);
    std::swap(P.at_idx, o.at_idx);
    std::swap(P.a_val, o.a_val);
    std::swap(P.at_val, o.at_val);
}

// makes the reordered matrices (already swapped in) the problem's: its
// vectors follow the new order and it keeps the orders for the ABI boundary
template <class T>
void adopt_density_order(Handle& h, ProblemT<T>& P, DensityOrder<T>& o) {
    cudaStream_t s = h.stream;
    auto reorder = [&](auto& v, const int32_t* ord, int64_t len) {
        using E = typename std::remove_reference<decltype(*v.p)>::type;
        if (!v.p || len <= 0) return;
        std::remove_reference_t<decltype(v)> t(v.n);
        gather_values<E, E>(v.p, ord, t.p, len, s);
        std::swap(v, t);
        CK(cudaStreamSynchronize(s));
    };
    for (DBuf<T>* v : {&P.c, &P.lv, &P.uv, &P.d2t, &P.invD2t}) reorder(*v, o.ocol.p, P.n);
    for (DBuf<T>* v : {&P.lc, &P.uc, &P.d1t, &P.invD1t}) reorder(*v, o.orow.p, P.m);
    for (DBuf<double>* v : {&P.D2, &P.invD2}) reorder(*v, o.ocol.p, P.n);
    for (DBuf<double>* v : {&P.D1, &P.invD1}) reorder(*v, o.orow.p, P.m);
    P.order_row = std::move(o.orow);
    P.order_col = std::move(o.ocol);
    P.ordered = true;
}

__global__ void k_scatter_order(const double* __restrict__ in, const int32_t* __restrict__ order,
                                double* __restrict__ out, int64_t n) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[order[k]] = in[k];
}

}  // namespace

// a device vector over P's rows (side 0) or columns (side 1), from the
// caller's order into the solver's, in place
void order_to_internal(const ProblemBase& P, int side, double* v, cudaStream_t s) {
    const int64_t len = side == 0 ? P.m : P.n;
    if (!P.ordered || len <= 0) return;
    DBuf<double> t((size_t)len);
    CK(cudaMemcpyAsync(t.p, v, sizeof(double) * len, cudaMemcpyDeviceToDevice, s));
    gather_values<double, double>(t.p, (side == 0 ? P.order_row : P.order_col).p, v, len, s);
    CK(cudaStreamSynchronize(s));
}
// ... and back into the caller's order
void order_to_user(const ProblemBase& P, int side, double* v, cudaStream_t s) {
    const int64_t len = side == 0 ? P.m : P.n;
    if (!P.ordered || len <= 0) return;
    DBuf<double> t((size_t)len);
    CK(cudaMemcpyAsync(t.p, v, sizeof(double) * len, cudaMemcpyDeviceToDevice, s));
    k_scatter_order<<<grid_for(len, 256), 256, 0, s>>>(t.p, (side == 0 ? P.order_row : P.order_col).p,
                                                       v, len);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s));
}

namespace {

// ---------------------------------------------------------------------------
// problem creation: preprocess (common.jl:154-169) on the device
// ---------------------------------------------------------------------------
template <class T>
ProblemBase* make_problem(Handle& h, const cpdlp_lp* lp, const cpdlp_params* prm, bool plans) {
    double t0 = now_seconds();
    cudaStream_t s = h.stream;
    // CPDLP_TRACE=1: the time of each setup phase (synchronised only when tracing)
    double t_mark = t0;
    auto mark = [&](const char* what) {
        if (trace_level() <= 0) return;
        CK(cudaStreamSynchronize(s));
        const double t = now_seconds();
        fprintf(stderr, "[cpdlp setup] %-28s %8.2f ms\n", what, 1e3 * (t - t_mark));
        t_mark = t;
    };
    auto* P = new ProblemT<T>();
    std::unique_ptr<ProblemT<T>> guard(P);
    P->h = &h;
    P->vt = std::is_same<T, float>::value ? CPDLP_VAL_F32 : CPDLP_VAL_F64;
    P->prm = *prm;
    const int64_t m = lp->m, n = lp->n;
    for (const double* v : {lp->c, lp->lv, lp->uv})
        if (n > 0 && !v) fail(CPDLP_ERR_ARGUMENT, "null variable vector (c, lv or uv)");
    for (const double* v : {lp->lc, lp->uc})
        if (m > 0 && !v) fail(CPDLP_ERR_ARGUMENT, "null constraint vector (lc or uc)");
    CscPair S;
    build_csc_pair(h, m, n, lp->nnz, lp->colptr, lp->rowval, lp->nzval, S);
    mark("upload, check, transpose");
    const int64_t nnz = S.nnz;
    P->m = m; P->n = n; P->nnz = nnz;
    const size_t zn = (size_t)(nnz > 0 ? nnz : 1), mz = (size_t)(m > 0 ? m : 1),
                 nzv = (size_t)(n > 0 ? n : 1);
    // vA: A's values in S1 order, vAt: At's values in S2 order
    DBuf<double> vA(std::move(S.val1)), vAt(zn), wA(zn), wAt(zn), tA(zn), tAt(zn);
    gather_values<double, double>(vA.p, S.p21.p, vAt.p, nnz, s);
    DBuf<double> d1(mz), d2(nzv), r1(mz), r2(nzv), D1(mz), D2(nzv);
    const unsigned gm = grid_for(m, 256), gn = grid_for(n, 256), gz = grid_for(nnz, 256);
    k_fill<<<gm, 256, 0, s>>>(r1.p, 1.0, m);
    k_fill<<<gn, 256, 0, s>>>(r2.p, 1.0, n);
    CK_LAUNCH();
    // Ruiz (preconditioning.jl:117-125)
    if (prm->ruiz_iter > 0 && nnz > 0) {
        CK(cudaMemcpyAsync(wA.p, vA.p, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(wAt.p, vAt.p, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));
    }
    for (int it = 0; it < prm->ruiz_iter; it++) {
        k_row_norm_scale<<<gn, 256, 0, s>>>(S.ptr1.p, wA.p, n, NK_INF, 0.0, d2.p);
        k_row_norm_scale<<<gm, 256, 0, s>>>(S.ptr2.p, wAt.p, m, NK_INF, 0.0, d1.p);
        if (nnz > 0) {
            k_scale_S1<<<gz, 256, 0, s>>>(S.idx1.p, S.col1.p, wA.p, d1.p, d2.p, tA.p, nnz);
            k_scale_S2<<<gz, 256, 0, s>>>(S.idx2.p, S.row2.p, wAt.p, d1.p, d2.p, tAt.p, nnz);
            std::swap(wA, tA);
            std::swap(wAt, tAt);
        }
        k_mul_into<<<gm, 256, 0, s>>>(r1.p, d1.p, m);
        k_mul_into<<<gn, 256, 0, s>>>(r2.p, d2.p, n);
        CK_LAUNCH();
    }
    mark("Ruiz");
    // Pock-Chambolle on the Ruiz-scaled ORIGINAL matrix (preconditioning.jl:146-155)
    if (nnz > 0) {
        k_scale_S1<<<gz, 256, 0, s>>>(S.idx1.p, S.col1.p, vA.p, r1.p, r2.p, tA.p, nnz);
        k_scale_S2<<<gz, 256, 0, s>>>(S.idx2.p, S.row2.p, vAt.p, r1.p, r2.p, tAt.p, nnz);
        CK_LAUNCH();
    }
    auto kind_of = [](double p, int& kind) {
        if (std::isinf(p) && p > 0) kind = NK_INF;
        else if (p == 1.0) kind = NK_ONE;
        else if (p == 2.0) kind = NK_TWO;
        else if (p == 0.0) kind = NK_ZERO;
        else kind = NK_P;
    };
    const double alpha = prm->chambolle_pock_alpha;
    int kc, kr;
    kind_of(alpha, kc);
    kind_of(2.0 - alpha, kr);
    k_row_norm_scale<<<gn, 256, 0, s>>>(S.ptr1.p, tA.p, n, kc, alpha, d2.p);
    k_row_norm_scale<<<gm, 256, 0, s>>>(S.ptr2.p, tAt.p, m, kr, 2.0 - alpha, d1.p);
    CK_LAUNCH();
    // prec = prec_r * prec_cp: D1 = r1 .* d1_cp, D2 = d2_cp .* r2
    CK(cudaMemcpyAsync(D1.p, d1.p, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(D2.p, d2.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    k_mul_into<<<gm, 256, 0, s>>>(D1.p, r1.p, m);
    k_mul_into<<<gn, 256, 0, s>>>(D2.p, r2.p, n);
    CK_LAUNCH();
    // precondition(milp, prec): final values from the original ones
    if (nnz > 0) {
        k_scale_S1<<<gz, 256, 0, s>>>(S.idx1.p, S.col1.p, vA.p, D1.p, D2.p, tA.p, nnz);
        k_scale_S2<<<gz, 256, 0, s>>>(S.idx2.p, S.row2.p, vAt.p, D1.p, D2.p, tAt.p, nnz);
        CK_LAUNCH();
    }
    // solver matrices: A rows = S2 structure with A's values; A' rows = S1 with A''s values
    DBuf<int32_t> p12(zn);
    if (nnz > 0) {
        k_invert_perm<<<gz, 256, 0, s>>>(S.p21.p, p12.p, nnz);
        CK_LAUNCH();
    }
    // narrow +-1 storage: FP32 iterates and every value exactly +-1 (the
    // products with the sign pattern are exact; D1, D2 are applied per row)
    bool pm1 = std::is_same<T, float>::value && !(prm->tile_flags & CPDLP_TILE_NO_NARROW) &&
               nnz > 0;
    for (int64_t k = 0; pm1 && k < lp->nnz; k++) pm1 = std::fabs(lp->nzval[k]) == 1.0;
    P->pm1 = pm1;
    if (pm1) {
        // rows of A: S2 order, original values vAt; rows of A': S1 order, vA
        k_encode_sign<<<gz, 256, 0, s>>>(S.idx2.p, vAt.p, nnz);
        k_encode_sign<<<gz, 256, 0, s>>>(S.idx1.p, vA.p, nnz);
        CK_LAUNCH();
    } else {
        P->a_val.alloc(zn + PAD_ELEMS);
        P->at_val.alloc(zn + PAD_ELEMS);
        CK(cudaMemsetAsync(P->a_val.p, 0, sizeof(T) * (zn + PAD_ELEMS), s));
        CK(cudaMemsetAsync(P->at_val.p, 0, sizeof(T) * (zn + PAD_ELEMS), s));
        gather_values<T, double>(tA.p, S.p21.p, P->a_val.p, nnz, s);
        gather_values<T, double>(tAt.p, p12.p, P->at_val.p, nnz, s);
    }
    P->a_ptr = std::move(S.ptr2);
    P->a_idx = std::move(S.idx2);
    P->at_ptr = std::move(S.ptr1);
    P->at_idx = std::move(S.idx1);
    // vectors
    DBuf<double> hc(nzv), hlv(nzv), huv(nzv), hlc(mz), huc(mz);
    if (n > 0) {
        CK(cudaMemcpyAsync(hc.p, lp->c, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(hlv.p, lp->lv, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(huv.p, lp->uv, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    }
    if (m > 0) {
        CK(cudaMemcpyAsync(hlc.p, lp->lc, sizeof(double) * m, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(huc.p, lp->uc, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    }
    P->c.alloc(nzv); P->lv.alloc(nzv); P->uv.alloc(nzv); P->lc.alloc(mz); P->uc.alloc(mz);
    P->invD1.alloc(mz); P->invD2.alloc(nzv);
    k_scale_vec_n<T><<<gn, 256, 0, s>>>(hc.p, hlv.p, huv.p, D2.p, P->c.p, P->lv.p, P->uv.p,
                                        P->invD2.p, n);
    k_scale_vec_m<T><<<gm, 256, 0, s>>>(hlc.p, huc.p, D1.p, P->lc.p, P->uc.p, P->invD1.p, m);
    CK_LAUNCH();
    if (pm1) {
        P->d1t.alloc(mz);
        P->d2t.alloc(nzv);
        k_narrow<T><<<gm, 256, 0, s>>>(D1.p, P->d1t.p, m);
        k_narrow<T><<<gn, 256, 0, s>>>(D2.p, P->d2t.p, n);
        CK_LAUNCH();
    }
    if constexpr (!std::is_same<T, double>::value) {
        P->invD1t.alloc(mz);
        P->invD2t.alloc(nzv);
        k_narrow<T><<<gm, 256, 0, s>>>(P->invD1.p, P->invD1t.p, m);
        k_narrow<T><<<gn, 256, 0, s>>>(P->invD2.p, P->invD2t.p, n);
        CK_LAUNCH();
    }
    P->D1 = std::move(D1);
    P->D2 = std::move(D2);
    mark("Pock-Chambolle, values, vectors");
    if (!plans) {  // the batched solver partitions the matrices itself
        P->zero_cost = false;
        CK(cudaStreamSynchronize(s));
        P->setup_seconds = now_seconds() - t0;
        guard.release();
        return P;
    }
    // tile plans from the row pointers
    std::vector<int32_t> hp2((size_t)m + 1), hp1((size_t)n + 1);
    CK(cudaMemcpyAsync(hp2.data(), P->a_ptr.p, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hp1.data(), P->at_ptr.p, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int items_A = choose_items(nnz, m, prm->tile_nnz), items_At = choose_items(nnz, n, prm->tile_nnz);
    // the product format: matrix_type (COO solves on the CSR engine), or the
    // autotuner's choice for large matrices
    const int32_t mt = prm->matrix_type;
    if (mt != CPDLP_FMT_AUTO && mt != CPDLP_FMT_CSR && mt != CPDLP_FMT_ELL && mt != CPDLP_FMT_COO)
        fail(CPDLP_ERR_ARGUMENT, "matrix_type must be CPDLP_FMT_AUTO, _CSR, _ELL or _COO");
    const bool order_on = (prm->tile_flags & CPDLP_TILE_DENSITY_ORDER) != 0;
    const bool order_off = (prm->tile_flags & CPDLP_TILE_NO_DENSITY_ORDER) != 0;
    if (order_on && order_off)
        fail(CPDLP_ERR_ARGUMENT, "CPDLP_TILE_DENSITY_ORDER and CPDLP_TILE_NO_DENSITY_ORDER both set");
    mark("row pointers to the host");
    if (order_on && nnz > 0) {
        DensityOrder<T> o;
        build_density_order(h, *P, o);
        swap_matrices(*P, o);
        adopt_density_order(h, *P, o);
        hp2 = std::move(o.hp2);
        hp1 = std::move(o.hp1);
    }
    auto ell_fits = [&](const std::vector<int32_t>& hp, int64_t rows) {
        int64_t w = 0;
        for (int64_t r = 0; r < rows; r++) w = std::max<int64_t>(w, hp[r + 1] - hp[r]);
        return rows * w <= ELL_MAX_PADDING * std::max<int64_t>(nnz, 1);
    };
    const bool tune = mt == CPDLP_FMT_AUTO ? nnz >= AUTOTUNE_MIN_NNZ
                                           : (mt != CPDLP_FMT_ELL && prm->tile_nnz == 0 &&
                                              nnz >= AUTOTUNE_MIN_NNZ);
    if (mt == CPDLP_FMT_ELL) {
        build_ell(h, *P, 0, hp2);
        build_ell(h, *P, 1, hp1);
        P->fmt[0] = P->fmt[1] = CPDLP_FMT_ELL;
    } else if (tune) {
        const bool try_csr = true;
        const bool ell_A = mt == CPDLP_FMT_AUTO && ell_fits(hp2, m);
        const bool ell_At = mt == CPDLP_FMT_AUTO && ell_fits(hp1, n);
        // scratch iterates (zeros) for the fused step kernels being timed
        DBuf<T> vx(nzv), vxn(nzv), vxb(nzv), vxa(nzv), vxa2(nzv), vy(mz), vyn(mz), vya(mz),
            vya2(mz), vys(pm1 ? mz : 1);
        for (DBuf<T>* b : {&vx, &vxn, &vxb, &vxa, &vxa2, &vy, &vyn, &vya, &vya2, &vys})
            CK(cudaMemsetAsync(b->p, 0, sizeof(T) * b->n, s));
        DBuf<StepCoef<T>> cf(1);
        CK(cudaMemsetAsync(cf.p, 0, sizeof(StepCoef<T>), s));
        ProblemT<T>* Q = P;
        // the primal step over A' and the dual step over A, with the
        // problem's current matrices
        auto launch_At = [&](int fmt, TilePlan& pl, T* part) {
            if (pm1) {
                const CsrView<Pm1, T> V{Q->at_ptr.p, Q->at_idx.p, nullptr, pl.tasks.p, pl.ntasks,
                                        pl.ltasks.p, pl.nltasks, pl.counters.p, part};
                PrimalEpi<T, false, true> pe{vx.p, Q->c.p, Q->lv.p, Q->uv.p, vxn.p, vxb.p,
                                             vxa.p, vxa2.p, {cf.p}, 1, Q->d2t.p};
                if (fmt == CPDLP_FMT_ELL) launch_ell<TILE_WARPS>(ell_view<Pm1, T>(*Q, 1, Q->at_ptr.p), VecSet<T, 1>{{vy.p}}, pe, s);
                else launch_tiles<1>(pl, V, VecSet<T, 1>{{vy.p}}, pe, s);
            } else {
                const CsrView<T, T> V{Q->at_ptr.p, Q->at_idx.p, Q->at_val.p, pl.tasks.p, pl.ntasks,
                                      pl.ltasks.p, pl.nltasks, pl.counters.p, part};
                PrimalEpi<T> pe{vx.p, Q->c.p, Q->lv.p, Q->uv.p, vxn.p, vxb.p, vxa.p, vxa2.p, {cf.p}, 1};
                if (fmt == CPDLP_FMT_ELL) launch_ell<TILE_WARPS>(ell_view<T, T>(*Q, 1, Q->at_ptr.p), VecSet<T, 1>{{vy.p}}, pe, s);
                else launch_tiles<1>(pl, V, VecSet<T, 1>{{vy.p}}, pe, s);
            }
        };
        auto launch_A = [&](int fmt, TilePlan& pl, T* part) {
            if (pm1) {
                const CsrView<Pm1, T> V{Q->a_ptr.p, Q->a_idx.p, nullptr, pl.tasks.p, pl.ntasks,
                                        pl.ltasks.p, pl.nltasks, pl.counters.p, part};
                DualEpi<T, false, true> de{vy.p, Q->lc.p, Q->uc.p, vyn.p, vya.p, vya2.p, {cf.p}, 1,
                                           Q->d1t.p, vys.p};
                if (fmt == CPDLP_FMT_ELL) launch_ell<TILE_WARPS>(ell_view<Pm1, T>(*Q, 0, Q->a_ptr.p), VecSet<T, 1>{{vxb.p}}, de, s);
                else launch_tiles<1>(pl, V, VecSet<T, 1>{{vxb.p}}, de, s);
            } else {
                const CsrView<T, T> V{Q->a_ptr.p, Q->a_idx.p, Q->a_val.p, pl.tasks.p, pl.ntasks,
                                      pl.ltasks.p, pl.nltasks, pl.counters.p, part};
                DualEpi<T> de{vy.p, Q->lc.p, Q->uc.p, vyn.p, vya.p, vya2.p, {cf.p}, 1};
                if (fmt == CPDLP_FMT_ELL) launch_ell<TILE_WARPS>(ell_view<T, T>(*Q, 0, Q->a_ptr.p), VecSet<T, 1>{{vxb.p}}, de, s);
                else launch_tiles<1>(pl, V, VecSet<T, 1>{{vxb.p}}, de, s);
            }
        };
        const SideChoice cAt = tune_side<T>(h, *P, 1, hp1, items_At, try_csr, ell_At, pm1 ? 3 : 1,
                                            launch_At);
        const SideChoice cA = tune_side<T>(h, *P, 0, hp2, items_A, try_csr, ell_A, pm1 ? 2 : 0,
                                           launch_A);
        items_A = cA.items;
        items_At = cAt.items;
        // density order as a candidate (CSR on both matrices): both step
        // kernels timed in each order, the density order kept when it is at
        // least 3% faster; decided once per matrix shape for the process
        if (mt == CPDLP_FMT_AUTO && !order_on && !order_off && P->fmt[0] == CPDLP_FMT_CSR &&
            P->fmt[1] == CPDLP_FMT_CSR) {
            static std::mutex mu;
            static std::map<std::tuple<int64_t, int64_t, int64_t, int, int, int>, bool> cache;
            const auto key = std::make_tuple(m, n, nnz, (int)sizeof(T), h.device, (int)pm1);
            int decided = -1;
            {
                std::lock_guard<std::mutex> lock(mu);
                auto it = cache.find(key);
                if (it != cache.end()) decided = it->second ? 1 : 0;
            }
            cudaEvent_t e0, e1;
            CK(cudaEventCreate(&e0));
            CK(cudaEventCreate(&e1));
            auto time_steps = [&](const std::vector<int32_t>& pa, const std::vector<int32_t>& pat) {
                TilePlan plA, plAt;
                build_tile_plan(pa, (int32_t)m, items_A, plA, s);
                build_tile_plan(pat, (int32_t)n, items_At, plAt, s);
                DBuf<T> partA((size_t)std::max(plA.npieces, 1)), partAt((size_t)std::max(plAt.npieces, 1));
                launch_At(CPDLP_FMT_CSR, plAt, partAt.p);
                launch_A(CPDLP_FMT_CSR, plA, partA.p);
                CK(cudaEventRecord(e0, s));
                for (int r = 0; r < 4; r++) {
                    launch_At(CPDLP_FMT_CSR, plAt, partAt.p);
                    launch_A(CPDLP_FMT_CSR, plA, partA.p);
                }
                CK(cudaEventRecord(e1, s));
                CK(cudaEventSynchronize(e1));
                float ms = 0.f;
                CK(cudaEventElapsedTime(&ms, e0, e1));
                return ms;
            };
            try {
                if (decided != 0) {
                    DensityOrder<T> o;
                    build_density_order(h, *P, o);
                    bool keep = decided == 1;
                    if (decided < 0) {
                        const float t_plain = time_steps(hp2, hp1);
                        swap_matrices(*P, o);
                        const float t_order = time_steps(o.hp2, o.hp1);
                        swap_matrices(*P, o);
                        keep = t_order < 0.97f * t_plain;
                        std::lock_guard<std::mutex> lock(mu);
                        cache[key] = keep;
                    }
                    if (keep) {
                        swap_matrices(*P, o);
                        adopt_density_order(h, *P, o);
                        hp2 = std::move(o.hp2);
                        hp1 = std::move(o.hp1);
                    }
                }
            } catch (...) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                throw;
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
    }
    mark("formats, autotuner, density order");
    // the CSR plans (also kept for an ELL side: the tuner and the exports use them),
    // the two on two host threads (each a sequential pass over its rows)
    {
        std::exception_ptr err;
        std::thread t([&] {
            try {
                CK(cudaSetDevice(h.device));
                AllocScope scope(s);
                build_tile_plan(hp1, (int32_t)n, items_At, P->planAt, s);
            } catch (...) {
                err = std::current_exception();
            }
        });
        try {
            build_tile_plan(hp2, (int32_t)m, items_A, P->planA, s);
        } catch (...) {
            t.join();
            throw;
        }
        t.join();
        if (err) std::rethrow_exception(err);
    }
    P->partA.alloc((size_t)(P->planA.npieces > 0 ? P->planA.npieces : 1) * 4);
    P->partAt.alloc((size_t)(P->planAt.npieces > 0 ? P->planAt.npieces : 1) * 4);
    P->rows_A_partials = side_partials(*P, 0, TILE_WARPS);
    P->rows_At_partials = side_partials(*P, 1, TILE_WARPS);
    P->rows_A_kkt = side_partials(*P, 0, kkt_warps<T>());
    P->rows_At_kkt = side_partials(*P, 1, kkt_warps<T>());
    P->kkt4_cap = (int64_t)h.num_sms * kkt_blocks_per_sm<T>();
    P->rows_A_kkt4 = side_partials4(*P, 0, kkt_warps<T>());
    P->rows_At_kkt4 = side_partials4(*P, 1, kkt_warps<T>());
    int64_t rows_max = std::max<int64_t>(std::max(P->rows_A_partials, P->rows_At_partials),
                                         (int64_t)h.num_sms * 4 + 8);
    rows_max = std::max<int64_t>(rows_max, std::max(P->rows_A_kkt, P->rows_At_kkt));
    rows_max = std::max<int64_t>(rows_max, std::max(P->rows_A_kkt4, P->rows_At_kkt4));
    P->red_rows.alloc((size_t)rows_max * 12);
    P->red_cols.alloc((size_t)rows_max * 12);
    P->red_out.alloc(64);
    // constant scales (errors.jl:79-85)
    {
        unsigned g = red_grid(h, std::max(m, n));
        k_scales<T><<<g, RED_THREADS, 0, s>>>(P->lc.p, P->uc.p, P->invD1.p, m, P->c.p, P->invD2.p,
                                              n, P->red_rows.p);
        CK_LAUNCH();
        double q[4];
        fetch_reduced(h, P->red_rows.p, g, 4, P->red_out.p, q);
        P->primal_scale = 1.0 + sqrt(q[0]);
        P->dual_scale = 1.0 + sqrt(q[2]);
    }
    bool zc = true;
    for (int64_t j = 0; j < n; j++)
        if (lp->c[j] != 0.0) { zc = false; break; }
    P->zero_cost = zc;
    mark("tile plans, scales");
    CK(cudaStreamSynchronize(s));
    P->setup_seconds = now_seconds() - t0;
    guard.release();
    return P;
}

// ---------------------------------------------------------------------------
// spectral norm: IterativeSolvers.powm! on Symmetrized(A, A') (linalg.jl:60-96)
// ---------------------------------------------------------------------------
uint64_t splitmix64_at(uint64_t seed, uint64_t counter) {
    uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Gaussian start vector: SplitMix64 + Box-Muller, element i from counters 2i, 2i+1
void gaussian_vector(uint64_t seed, int64_t len, std::vector<double>& out) {
    out.resize((size_t)len);
    // entry i depends only on (seed, i): blocks of 4,096 entries on host threads
    // (one thread took 80-130 ms for 4M columns, most of a large LP's state setup)
    const int64_t block = 4096;
    parallel_for((len + block - 1) / block, [&](int64_t b) {
        const int64_t end = std::min(len, (b + 1) * block);
        for (int64_t i = b * block; i < end; i++) {
            double u1 = (double)((splitmix64_at(seed, 2 * (uint64_t)i) >> 11) + 1) * (1.0 / 9007199254740992.0);
            double u2 = (double)((splitmix64_at(seed, 2 * (uint64_t)i + 1) >> 11) + 1) * (1.0 / 9007199254740992.0);
            out[(size_t)i] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        }
    });
}

double powm_default_tol(int64_t n, bool f32) {
    uint64_t un = (uint64_t)n;
    int64_t n3 = (int64_t)(un * un * un);  // Julia Int64 arithmetic wraps modulo 2^64
    double eps = f32 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
    return eps * (double)n3;
}

// powm! on A'A (linalg.jl:86-96).  The vectors and every product are FP64 for
// both value types (FP32 matrix values promote exactly), and the stopping rule
// is IterativeSolvers' default for Float64 (eps * n^3): with eps(Float32) that
// rule stops large FP32 problems after one iteration, and the step size
// eta = 0.9 / |A| then overshoots.
// `deadline` (now_seconds() clock): the iterations also stop there.  The
// reference's default rule can ask for n iterations (tol = eps * n^3 wraps
// negative for some n), which a solve's time limit then bounds.
template <class V>
double spectral_norm_T(Handle& h, ProblemT<V>& P, const cpdlp_params* prm, int64_t* iters_out,
                       double deadline = INFINITY) {
    cudaStream_t s = h.stream;
    const int64_t m = P.m, n = P.n;
    double tol = prm->power_tol_override > 0 ? prm->power_tol_override : powm_default_tol(n, false);
    int64_t maxiter = prm->power_maxiter_override > 0 ? prm->power_maxiter_override : n;
    // FP32 iterates need theta to about 1%, not to eps(Float64) n^3 (which
    // can ask for n iterations on small or, through the Int64 wrap, huge LPs)
    const double rtol = std::is_same<V, float>::value ? POWER_RTOL_F32 : -1.0;
    std::vector<double> x0;
    gaussian_vector(prm->power_seed, n, x0);
    DBuf<double> x((size_t)(n > 0 ? n : 1)), Ax((size_t)(n > 0 ? n : 1)), sv((size_t)(m > 0 ? m : 1));
    DBuf<double> pA((size_t)std::max(P.planA.npieces, 1)), pAt((size_t)std::max(P.planAt.npieces, 1));
    DBuf<double> scal(4);
    DBuf<int> d_it(1);
    if (n > 0) CK(cudaMemcpyAsync(x.p, x0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    order_to_internal(P, 1, x.p, s);  // the start vector of the caller's column order
    CK(cudaMemsetAsync(d_it.p, 0, sizeof(int), s));
    const CsrView<V, double> A{P.a_ptr.p, P.a_idx.p, P.a_val.p, P.planA.tasks.p, P.planA.ntasks,
                               P.planA.ltasks.p, P.planA.nltasks, P.planA.counters.p, pA.p};
    const CsrView<V, double> At{P.at_ptr.p, P.at_idx.p, P.at_val.p, P.planAt.tasks.p,
                                P.planAt.ntasks, P.planAt.ltasks.p, P.planAt.nltasks,
                                P.planAt.counters.p, pAt.p};
    // narrow +-1 storage: A = D1 S D2; the first product gathers xs = D2 x and
    // stores D1 (A x) = D1 D1 (S xs), the second multiplies S' (D1 A x) by D2
    const CsrView<Pm1, double> A1{P.a_ptr.p, P.a_idx.p, nullptr, P.planA.tasks.p,
                                  P.planA.ntasks, P.planA.ltasks.p, P.planA.nltasks,
                                  P.planA.counters.p, pA.p};
    const CsrView<Pm1, double> At1{P.at_ptr.p, P.at_idx.p, nullptr, P.planAt.tasks.p,
                                   P.planAt.ntasks, P.planAt.ltasks.p, P.planAt.nltasks,
                                   P.planAt.counters.p, pAt.p};
    DBuf<double> xs((size_t)(P.pm1 && n > 0 ? n : 1));
    if (P.pm1 && n > 0) {
        k_mul_vec<double><<<grid_for(n, 256), 256, 0, s>>>(x.p, P.D2.p, xs.p, n);
        CK_LAUNCH();
    }
    constexpr int DEPTH = 8;  // iterations queued ahead of the host's stopping check
    void* block = h.host_get(sizeof(PowerSlot) * DEPTH);
    PowerSlot* ring = static_cast<PowerSlot*>(block);
    PowerSlot* dring = nullptr;
    CK(cudaHostGetDevicePointer((void**)&dring, ring, 0));
    struct Cleanup {
        Handle& h; void* block; cudaStream_t s; cudaGraphExec_t exec = nullptr;
        cudaEvent_t ev[DEPTH] = {};
        ~Cleanup() {
            cudaStreamSynchronize(s);  // speculative iterations finish before buffers go
            if (exec) cudaGraphExecDestroy(exec);
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            h.host_put(block);
        }
    } cleanup{h, block, s};
    for (int k = 0; k < DEPTH; k++)
        CK(cudaEventCreateWithFlags(&cleanup.ev[k], cudaEventDisableTiming));
    const unsigned gr = red_grid(h, n);
    {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        double* const blk = P.red_cols.p;
        double* const lng = P.red_cols.p + (size_t)side_blocks(P, 1, TILE_WARPS) * 2;
        if (P.pm1) {
            launch_side(P, 0, A1, VecSet<double, 1>{{xs.p}}, ScaledStoreEpi<double>{sv.p, P.D1.p}, s);
            PowerEpi<double, true> pe{x.p, Ax.p, blk, lng, P.D2.p};
            launch_side(P, 1, At1, VecSet<double, 1>{{sv.p}}, pe, s);
        } else {
            launch_side(P, 0, A, VecSet<double, 1>{{x.p}}, StoreEpi<double>{sv.p}, s);
            PowerEpi<double> pe{x.p, Ax.p, blk, lng};
            launch_side(P, 1, At, VecSet<double, 1>{{sv.p}}, pe, s);
        }
        reduce_partials(P.red_cols.p, P.rows_At_partials, 2, P.red_out.p, s);
        k_power_theta<<<1, 32, 0, s>>>(P.red_out.p, scal.p, d_it.p, dring, DEPTH);
        k_power_residual<<<gr, RED_THREADS, 0, s>>>(x.p, Ax.p, scal.p, n, P.red_rows.p,
                                                    P.pm1 ? P.D2.p : nullptr,
                                                    P.pm1 ? xs.p : nullptr);
        reduce_partials(P.red_rows.p, gr, 1, P.red_out.p + 2, s);
        k_power_finish<<<1, 32, 0, s>>>(P.red_out.p + 2, d_it.p, dring, DEPTH);
        const cudaError_t launch_err = cudaGetLastError();
        const cudaError_t end_err = cudaStreamEndCapture(s, &g);
        CK(launch_err);
        CK(end_err);
        const cudaError_t inst = cudaGraphInstantiate(&cleanup.exec, g, 0);
        cudaGraphDestroy(g);
        CK(inst);
    }
    // powm!: iterate while !(it > maxiter || residual <= tol); it counts iterations run.
    // Iterations are queued ahead of the host's check, 2 at first and twice as
    // many each time a result is read, up to DEPTH: an LP that stops after 2
    // iterations (C1 with FP32 iterates) runs no 6 extra ones.
    double theta_d = 0.0;
    int64_t launched = 0, it = 0, ahead = 2;
    for (;;) {
        while (launched - it < ahead && launched <= maxiter) {
            CK(cudaGraphLaunch(cleanup.exec, s));
            CK(cudaEventRecord(cleanup.ev[launched % DEPTH], s));
            launched++;
        }
        CK(cudaEventSynchronize(cleanup.ev[it % DEPTH]));
        const PowerSlot slot = ring[it % DEPTH];
        it++;
        ahead = std::min<int64_t>(2 * ahead, DEPTH);
        theta_d = slot.theta;
        if (it > maxiter || slot.residual <= tol || slot.residual <= rtol * slot.theta) break;
        if (now_seconds() >= deadline) break;
    }
    if (iters_out) *iters_out = it;
    return std::sqrt(theta_d);
}

// ---------------------------------------------------------------------------
// solver state
// ---------------------------------------------------------------------------
template <class T>
struct StateT : StateBase {
    ProblemT<T>* PT = nullptr;
    Handle* h = nullptr;
    DBuf<T> x[2], y[2], xa[2], ya[2], xr, yr, xbar;
    int cur = 0;  // sol = (x[cur], y[cur]); sol_last = (x[cur^1], y[cur^1]); same for averages
    // narrow +-1 storage: ys[b] = D1 .* y[b] (the primal product's gather; the
    // dual step writes it beside y), xbar holds D2 .* xbar
    DBuf<T> ys[2];
    // the KKT pass's packed (and, for a narrow matrix, scaled) gathered vectors
    DBuf<T> kx4, ky4;
    // refinement round on the residual LP: the dual step's activity offset
    // (scaled base multipliers), and the KKT evaluation of the combined iterate
    // (base + correction) that replaces the state's own
    const double* yoff = nullptr;
    // infeasibility detection (prm.infeasibility_tol > 0): the iterates at the
    // previous check and the FP64 rays
    DBuf<T> xprev, yprev;
    DBuf<double> rx, ry, rxs, rys, rpart_A, rpart_At;
    bool have_prev = false;
    std::function<void(int, const T* const*, const T* const*, cpdlp_kkt_errors*)> kkt_hook;
    DBuf<StepCoef<T>> coef, coef1;
    std::vector<StepCoef<T>> coef_host;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_len = 0;

    ~StateT() override {
        for (auto& g : graph)
            if (g) cudaGraphExecDestroy(g);
    }

    bool pdlp() const { return prm.algorithm == CPDLP_ALGO_PDLP; }
    int step_launches() const { return tiles_launches(PT->planA) + tiles_launches(PT->planAt); }

    StepCoef<T> coef_for(double eta_sum_k) const {
        StepCoef<T> k;
        const double tau = eta / omega, sigma = eta * omega;
        k.tau = (T)tau;
        k.sigma = (T)sigma;
        k.inv_sigma = (T)(1.0 / sigma);
        k.a = (T)(eta / (eta + eta_sum_k));
        k.b = (T)(eta_sum_k / (eta + eta_sum_k));
        return k;
    }

    // primal step: x+ = proj(x - tau (c - A'y)), xbar, the running average
    // (narrow storage: gathers yg = D1 y, and xb receives D2 xbar)
    void launch_primal(const T* xo, T* xn, T* xb, const T* xao, T* xan, const T* yg,
                       const StepCoef<T>* c, cudaStream_t s) {
        ProblemT<T>& P = *PT;
        const int avg = pdlp() ? 1 : 0;
        if (P.pm1) {
            PrimalEpi<T, false, true> pe{xo, P.c.p, P.lv.p, P.uv.p, xn, xb, xao, xan, {c}, avg,
                                         P.d2t.p};
            launch_side(P, 1, view_At_pm1(P), VecSet<T, 1>{{yg}}, pe, s);
        } else {
            PrimalEpi<T> pe{xo, P.c.p, P.lv.p, P.uv.p, xn, xb, xao, xan, {c}, avg};
            launch_side(P, 1, view_At(P), VecSet<T, 1>{{yg}}, pe, s);
        }
    }
    // dual step: y+ from A xbar (narrow storage: also writes ysn = D1 y+)
    void launch_dual(const T* yo, T* yn, T* ysn, const T* yao, T* yan, const T* xg,
                     const StepCoef<T>* c, cudaStream_t s) {
        ProblemT<T>& P = *PT;
        const int avg = pdlp() ? 1 : 0;
        if (P.pm1 && yoff) {
            DualEpi<T, false, true, true> de{yo, P.lc.p, P.uc.p, yn, yao, yan, {c}, avg,
                                             P.d1t.p, ysn, yoff};
            launch_side(P, 0, view_A_pm1(P), VecSet<T, 1>{{xg}}, de, s);
        } else if (P.pm1) {
            DualEpi<T, false, true> de{yo, P.lc.p, P.uc.p, yn, yao, yan, {c}, avg, P.d1t.p, ysn};
            launch_side(P, 0, view_A_pm1(P), VecSet<T, 1>{{xg}}, de, s);
        } else if (yoff) {
            DualEpi<T, false, false, true> de{yo, P.lc.p, P.uc.p, yn, yao, yan, {c}, avg,
                                              nullptr, nullptr, yoff};
            launch_side(P, 0, view_A(P), VecSet<T, 1>{{xg}}, de, s);
        } else {
            DualEpi<T> de{yo, P.lc.p, P.uc.p, yn, yao, yan, {c}, avg};
            launch_side(P, 0, view_A(P), VecSet<T, 1>{{xg}}, de, s);
        }
    }

    // One step!: kernels only.  `c` points at this step's coefficients.
    void enqueue_step(int parity_in, const StepCoef<T>* c, cudaStream_t s) {
        const bool pm = PT->pm1;
        const int o = parity_in, nw = parity_in ^ 1;  // read old, write new
        launch_primal(x[o].p, x[nw].p, xbar.p, xa[o].p, xa[nw].p, pm ? ys[o].p : y[o].p, c, s);
        launch_dual(y[o].p, y[nw].p, pm ? ys[nw].p : nullptr, ya[o].p, ya[nw].p, xbar.p, c, s);
    }

    void advance_counters(int64_t k) {
        kkt_passes += k;
        if (pdlp()) {
            inner += k;
            total += k;
        }
    }

    void build_graph(int parity, int len) {
        cudaStream_t s = h->stream;
        cudaGraph_t g;
        // the step kernels' L1 carveout hint (prefer_l1) is set outside a
        // capture: walk one step's launches without launching them
        tiles_dry_run() = true;
        try {
            enqueue_step(parity, coef.p, s);
        } catch (...) {
            tiles_dry_run() = false;
            throw;
        }
        tiles_dry_run() = false;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int par = parity;
        for (int k = 0; k < len; k++) {
            enqueue_step(par, coef.p + k, s);
            par ^= 1;
        }
        CK(cudaStreamEndCapture(s, &g));
        if (graph[parity]) cudaGraphExecDestroy(graph[parity]);
        CK(cudaGraphInstantiate(&graph[parity], g, 0));
        cudaGraphDestroy(g);
    }

    // `len` steps as one graph launch (len == check_every).
    void run_block(int len) {
        cudaStream_t s = h->stream;
        if (len != graph_len) {
            for (auto& g : graph)
                if (g) { cudaGraphExecDestroy(g); g = nullptr; }
            graph_len = len;
            coef.alloc((size_t)len);
            coef_host.resize((size_t)len);
        }
        if (!graph[cur]) build_graph(cur, len);
        double es = eta_sum;
        for (int k = 0; k < len; k++) {
            coef_host[(size_t)k] = coef_for(es);
            if (pdlp()) es += eta;
        }
        // pageable source: the bytes are staged before the call returns
        CK(cudaMemcpyAsync(coef.p, coef_host.data(), sizeof(StepCoef<T>) * len,
                           cudaMemcpyHostToDevice, s));
        CK(cudaGraphLaunch(graph[cur], s));
        launches += (int64_t)len * step_launches();
        eta_sum = es;
        if (len & 1) cur ^= 1;
        advance_counters(len);
    }

    void run_single() {
        cudaStream_t s = h->stream;
        if (!coef1.p) coef1.alloc(1);
        StepCoef<T> k = coef_for(eta_sum);
        CK(cudaMemcpyAsync(coef1.p, &k, sizeof(k), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        enqueue_step(cur, coef1.p, s);
        launches += step_launches();
        cur ^= 1;
        if (pdlp()) eta_sum += eta;
        advance_counters(1);
    }

    void step(int64_t count) override {
        const int ce = prm.check_every > 0 ? prm.check_every : 100;
        while (count >= ce) {
            run_block(ce);
            count -= ce;
        }
        while (count-- > 0) run_single();
        CK(cudaStreamSynchronize(h->stream));
    }

    // KKT errors (errors.jl:65-109) of NV (1 or 4) (x, y) pairs in ONE
    // row-side and ONE column-side tile pass.  Four pairs are packed first
    // (x4[4j + p], y4[4i + p]: one request per nonzero gathers all four, and
    // the tile's indices and values are read once); a narrow matrix's pack
    // also applies D2 / D1, the scales its products need.  Each pass leaves
    // FP64 block partials (2 NV row-side, 3 NV column-side values per block);
    // a pair's sums do not depend on the other pairs of the pass.
    template <int NV>
    void enqueue_kkt(const T* const (&xs)[NV], const T* const (&ys)[NV]) {
        static_assert(NV == 1 || NV == 4, "one or four iterates per KKT pass");
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        const size_t nz = (size_t)std::max<int64_t>(P.n, 1), mz = (size_t)std::max<int64_t>(P.m, 1);
        const T* gx = xs[0];
        const T* gy = ys[0];
        if (NV == 4 || P.pm1) {
            if (!kx4.p) {
                kx4.alloc(4 * nz);
                ky4.alloc(4 * mz);
            }
            PackSrc<T, NV> px, py;
            for (int p = 0; p < NV; p++) {
                px.v[p] = xs[p];
                py.v[p] = ys[p];
            }
            k_pack<T, NV><<<red_grid(*h, std::max(P.m, P.n)), RED_THREADS, 0, s>>>(
                px, P.pm1 ? P.d2t.p : nullptr, P.n, kx4.p, py, P.pm1 ? P.d1t.p : nullptr, P.m,
                ky4.p);
            CK_LAUNCH();
            launches += 1;
            gx = kx4.p;
            gy = ky4.p;
        }
        if (P.pm1) kkt_impl<true, NV>(xs, ys, gx, gy, view_A_pm1(P), view_At_pm1(P));
        else kkt_impl<false, NV>(xs, ys, gx, gy, view_A(P), view_At(P));
    }
    template <bool SC, int NV, class VA, class VAt>
    void kkt_impl(const T* const (&xs)[NV], const T* const (&ys)[NV], const T* gx, const T* gy,
                  const VA& vA, const VAt& vAt) {
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        constexpr int W = kkt_warps<T>();
        const int64_t gA = NV == 4 ? side_blocks4(P, 0, W) : side_blocks(P, 0, W);
        const int64_t gAt = NV == 4 ? side_blocks4(P, 1, W) : side_blocks(P, 1, W);
        KktRowEpi<T, NV, SC, W> re;
        re.lc = P.lc.p; re.uc = P.uc.p; re.invD1 = P.invD1_T();
        for (int p = 0; p < NV; p++) re.y[p] = ys[p];
        re.block_out = P.red_rows.p;
        re.long_out = re.block_out + (size_t)gA * 2 * NV;
        re.dsc = SC ? P.d1t.p : nullptr;
        KktColEpi<T, NV, SC, W> ce;
        ce.c = P.c.p; ce.lv = P.lv.p; ce.uv = P.uv.p; ce.invD2 = P.invD2_T();
        for (int p = 0; p < NV; p++) ce.x[p] = xs[p];
        ce.block_out = P.red_cols.p;
        ce.long_out = ce.block_out + (size_t)gAt * 3 * NV;
        ce.dsc = SC ? P.d2t.p : nullptr;
        if constexpr (NV == 4) {
            launch_side4<W>(P, 0, vA, gx, re, s);
            launch_side4<W>(P, 1, vAt, gy, ce, s);
        } else {
            launch_side<W>(P, 0, vA, VecSet<T, 1>{{gx}}, re, s);
            launch_side<W>(P, 1, vAt, VecSet<T, 1>{{gy}}, ce, s);
        }
    }

    template <int NV>
    void kkt_multi(const T* const (&xs)[NV], const T* const (&ys)[NV], cpdlp_kkt_errors* out) {
        if (kkt_hook) {
            kkt_hook(NV, xs, ys, out);
            return;
        }
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        enqueue_kkt<NV>(xs, ys);
        reduce_partials(P.red_rows.p, NV == 4 ? P.rows_A_kkt4 : P.rows_A_kkt, 2 * NV,
                        P.red_out.p, s);
        reduce_partials(P.red_cols.p, NV == 4 ? P.rows_At_kkt4 : P.rows_At_kkt, 3 * NV,
                        P.red_out.p + 2 * NV, s);
        launches += tiles_launches(P.planA) + tiles_launches(P.planAt) + 2;
        double* pin = h->pinned_area(sizeof(double) * 64);
        CK(cudaMemcpyAsync(pin, P.red_out.p, sizeof(double) * 5 * NV, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int p = 0; p < NV; p++) {
            const double pr2 = pin[2 * p], pc = pin[2 * p + 1];
            const double du2 = pin[2 * NV + 3 * p], pv = pin[2 * NV + 3 * p + 1],
                         cx = pin[2 * NV + 3 * p + 2];
            cpdlp_kkt_errors& e = out[p];
            e.primal = std::sqrt(pr2);
            e.primal_scale = P.primal_scale;
            e.dual = std::sqrt(du2);
            e.dual_scale = P.dual_scale;
            e.gap = std::fabs((cx + pc) + pv);
            e.gap_scale = (1.0 + std::fabs(pc + pv)) + std::fabs(cx);
        }
    }

    void vec_of(int which, const T*& vx, const T*& vy) {
        switch (which) {
            case CPDLP_VEC_SOL_LAST: vx = x[cur ^ 1].p; vy = y[cur ^ 1].p; break;
            case CPDLP_VEC_SOL_AVG: vx = xa[cur].p; vy = ya[cur].p; break;
            case CPDLP_VEC_SOL_AVG_LAST: vx = xa[cur ^ 1].p; vy = ya[cur ^ 1].p; break;
            case CPDLP_VEC_SOL_RESTART: vx = xr.p; vy = yr.p; break;
            default: vx = x[cur].p; vy = y[cur].p; break;
        }
    }

    void kkt(int which, cpdlp_kkt_errors* e) override {
        const T *vx, *vy;
        vec_of(which, vx, vy);
        const T* const xs[1] = {vx};
        const T* const ys[1] = {vy};
        kkt_multi<1>(xs, ys, e);
    }

    // Tests the change of the iterates since the previous check as an
    // infeasibility certificate; returns PRIMAL_INFEASIBLE / DUAL_INFEASIBLE
    // (the ray replaces y / x of sol) or STILL_RUNNING.
    int32_t infeasibility_check() {
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        const int64_t m = P.m, n = P.n;
        const size_t nz = (size_t)std::max<int64_t>(n, 1), mz = (size_t)std::max<int64_t>(m, 1);
        if (!xprev.p) {
            xprev.alloc(nz); yprev.alloc(mz); rx.alloc(nz); ry.alloc(mz);
            if (P.pm1) { rxs.alloc(nz); rys.alloc(mz); }
            rpart_A.alloc((size_t)std::max(P.planA.npieces, 1));
            rpart_At.alloc((size_t)std::max(P.planAt.npieces, 1));
        }
        auto keep = [&] {
            CK(cudaMemcpyAsync(xprev.p, x[cur].p, sizeof(T) * nz, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(yprev.p, y[cur].p, sizeof(T) * mz, cudaMemcpyDeviceToDevice, s));
        };
        if (!have_prev) {
            keep();
            have_prev = true;
            return CPDLP_STILL_RUNNING;
        }
        k_ray<T><<<red_grid(*h, std::max(m, n)), RED_THREADS, 0, s>>>(
            x[cur].p, xprev.p, P.lv.p, P.uv.p, rx.p, P.pm1 ? rxs.p : nullptr, P.D2.p, n,
            y[cur].p, yprev.p, P.lc.p, P.uc.p, ry.p, P.pm1 ? rys.p : nullptr, P.D1.p, m);
        CK_LAUNCH();
        keep();
        const int64_t gA = side_blocks(P, 0, TILE_WARPS), gAt = side_blocks(P, 1, TILE_WARPS);
        double* const rblk = P.red_rows.p;
        double* const cblk = P.red_cols.p;
        if (P.pm1) {
            const CsrView<Pm1, double> A1{P.a_ptr.p, P.a_idx.p, nullptr, P.planA.tasks.p,
                                          P.planA.ntasks, P.planA.ltasks.p, P.planA.nltasks,
                                          P.planA.counters.p, rpart_A.p};
            const CsrView<Pm1, double> At1{P.at_ptr.p, P.at_idx.p, nullptr, P.planAt.tasks.p,
                                           P.planAt.ntasks, P.planAt.ltasks.p, P.planAt.nltasks,
                                           P.planAt.counters.p, rpart_At.p};
            launch_side(P, 0, A1, VecSet<double, 1>{{rxs.p}},
                            RayRowEpi<T, true>{P.lc.p, P.uc.p, ry.p, P.D1.p, rblk, rblk + (size_t)gA * 2}, s);
            launch_side(P, 1, At1, VecSet<double, 1>{{rys.p}},
                            RayColEpi<T, true>{P.c.p, P.lv.p, P.uv.p, rx.p, P.D2.p, cblk,
                                               cblk + (size_t)gAt * 3}, s);
        } else {
            const CsrView<T, double> A{P.a_ptr.p, P.a_idx.p, P.a_val.p, P.planA.tasks.p,
                                       P.planA.ntasks, P.planA.ltasks.p, P.planA.nltasks,
                                       P.planA.counters.p, rpart_A.p};
            const CsrView<T, double> At{P.at_ptr.p, P.at_idx.p, P.at_val.p, P.planAt.tasks.p,
                                        P.planAt.ntasks, P.planAt.ltasks.p, P.planAt.nltasks,
                                        P.planAt.counters.p, rpart_At.p};
            launch_side(P, 0, A, VecSet<double, 1>{{rx.p}},
                            RayRowEpi<T>{P.lc.p, P.uc.p, ry.p, nullptr, rblk, rblk + (size_t)gA * 2}, s);
            launch_side(P, 1, At, VecSet<double, 1>{{ry.p}},
                            RayColEpi<T>{P.c.p, P.lv.p, P.uv.p, rx.p, nullptr, cblk,
                                         cblk + (size_t)gAt * 3}, s);
        }
        reduce_partials(rblk, P.rows_A_partials, 2, P.red_out.p, s);
        reduce_partials(cblk, P.rows_At_partials, 3, P.red_out.p + 2, s);
        launches += 3 + tiles_launches(P.planA) + tiles_launches(P.planAt) + 2;
        double* pin = h->pinned_area(sizeof(double) * 64);
        CK(cudaMemcpyAsync(pin, P.red_out.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        const double ep = std::sqrt(pin[0]), yrow = pin[1], ed = std::sqrt(pin[2]),
                     ycol = pin[3], cx = pin[4];
        const double tol = prm.infeasibility_tol, bobj = yrow + ycol;
        if (bobj > 0.0 && ed <= tol * bobj) {
            if (m > 0) {
                k_narrow<T><<<grid_for(m, 256), 256, 0, s>>>(ry.p, y[cur].p, m);
                CK_LAUNCH();
            }
            return CPDLP_PRIMAL_INFEASIBLE;
        }
        if (cx < 0.0 && ep <= tol * (-cx)) {
            if (n > 0) {
                k_narrow<T><<<grid_for(n, 256), 256, 0, s>>>(rx.p, x[cur].p, n);
                CK_LAUNCH();
            }
            return CPDLP_DUAL_INFEASIBLE;
        }
        return CPDLP_STILL_RUNNING;
    }

    void push_history() {
        if (!prm.record_error_history) return;
        hist_passes.push_back(kkt_passes);
        hist_err.push_back(err);
    }

    static double relative(const cpdlp_kkt_errors& e) {
        return jl_max(jl_max(e.primal / e.primal_scale, e.dual / e.dual_scale), e.gap / e.gap_scale);
    }
    static double absolute(const cpdlp_kkt_errors& e, double w) {
        return std::sqrt((w * w) * (e.primal * e.primal) + (1.0 / (w * w)) * (e.dual * e.dual) +
                         e.gap * e.gap);
    }

    int32_t termination_status_now() const {
        if (relative(err) <= prm.termination_reltol) return CPDLP_OPTIMAL;
        if (time_elapsed >= prm.time_limit) return CPDLP_TIME_LIMIT;
        if (kkt_passes >= prm.max_kkt_passes) return CPDLP_ITERATION_LIMIT;
        return CPDLP_STILL_RUNNING;
    }

    // termination_check! (common.jl:218-231), given err of sol
    bool termination_check_with(const cpdlp_kkt_errors& e_sol) {
        time_elapsed = now_seconds() - starting_time;
        err = e_sol;
        push_history();
        status = termination_status_now();
        return status != CPDLP_STILL_RUNNING;
    }

    // restart_check! (pdlp.jl:138-170) with the four errors already evaluated
    bool restart_check(const cpdlp_kkt_errors (&e4)[4]) {
        const double w = omega;
        const cpdlp_kkt_errors &e = e4[0], &ea = e4[1], &el = e4[2], &eal = e4[3];
        if (absolute(e, w) < absolute(ea, w)) {
            restart_from_avg = 0;
            err_cand = e;
        } else {
            restart_from_avg = 1;
            err_cand = ea;
        }
        err_cand_last = (absolute(el, w) < absolute(eal, w)) ? el : eal;
        if (!err_restart_valid) {
            kkt(CPDLP_VEC_SOL_RESTART, &err_restart);
            err_restart_valid = true;
        }
        const double ac = absolute(err_cand, w), ar = absolute(err_restart, w),
                     acl = absolute(err_cand_last, w);
        const bool sufficient = ac <= prm.sufficient_decay * ar;
        const bool necessary = ac <= prm.necessary_decay * ar;
        const bool no_local_progress = ac > acl;
        const bool long_inner_loop = (double)inner >= prm.artificial_decay * (double)total;
        return sufficient || (necessary && no_local_progress) || long_inner_loop;
    }

    // restart! (pdlp.jl:172-196) + primal_weight_update! (step_size.jl:58-75)
    void restart() {
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        const T* cx = restart_from_avg ? xa[cur].p : x[cur].p;
        const T* cy = restart_from_avg ? ya[cur].p : y[cur].p;
        eta_sum = 0.0;
        const unsigned g = red_grid(*h, std::max(P.m, P.n));
        k_diff_norms<T><<<g, RED_THREADS, 0, s>>>(cx, xr.p, P.n, cy, yr.p, P.m, P.red_rows.p);
        CK_LAUNCH();
        launches += 2;
        double q[2];
        fetch_reduced(*h, P.red_rows.p, g, 2, P.red_out.p, q);
        const double dx = std::sqrt(q[0]), dy = std::sqrt(q[1]);
        const double th = prm.primal_weight_damping;
        if (dx > prm.zero_tol && dy > prm.zero_tol)
            omega = std::exp(th * std::log(dy / dx) + (1.0 - th) * std::log(omega));
        if (restart_from_avg) {
            CK(cudaMemcpyAsync(x[cur].p, xa[cur].p, sizeof(T) * P.n, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(y[cur].p, ya[cur].p, sizeof(T) * P.m, cudaMemcpyDeviceToDevice, s));
            if (P.pm1 && P.m > 0) {
                k_mul_vec<T><<<grid_for(P.m, 256), 256, 0, s>>>(y[cur].p, P.d1t.p, ys[cur].p, P.m);
                CK_LAUNCH();
                launches += 1;
            }
        }
        CK(cudaMemsetAsync(xa[cur].p, 0, sizeof(T) * P.n, s));
        CK(cudaMemsetAsync(ya[cur].p, 0, sizeof(T) * P.m, s));
        CK(cudaMemcpyAsync(xr.p, x[cur].p, sizeof(T) * P.n, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(yr.p, y[cur].p, sizeof(T) * P.m, cudaMemcpyDeviceToDevice, s));
        // the restart point now equals the candidate, whose errors are known
        err_restart = err_cand;
        err_restart_valid = true;
        outer += 1;
        inner = 0;
    }


    int32_t solve_blocks(int64_t max_blocks) override {
        const int ce = prm.check_every > 0 ? prm.check_every : 100;
        int64_t blocks = 0;
        if (!pdlp()) {
            for (;;) {
                if (blocks >= max_blocks) return status;
                run_block(ce);
                blocks++;
                cpdlp_kkt_errors e;
                kkt(CPDLP_VEC_SOL, &e);
                if (termination_check_with(e)) break;
                if (prm.infeasibility_tol > 0) {
                    const int32_t inf = infeasibility_check();
                    if (inf != CPDLP_STILL_RUNNING) { status = inf; break; }
                }
            }
            return status;
        }
        // The reference's nested loops (pdlp.jl:75-91) reduce to: block, check,
        // restart check; on termination the outer loop checks once more.
        for (;;) {
            if (blocks >= max_blocks) return status;
            run_block(ce);
            blocks++;
            cpdlp_kkt_errors e4[4];
            const T* const xs[4] = {x[cur].p, xa[cur].p, x[cur ^ 1].p, xa[cur ^ 1].p};
            const T* const ys[4] = {y[cur].p, ya[cur].p, y[cur ^ 1].p, ya[cur ^ 1].p};
            kkt_multi<4>(xs, ys, e4);
            err_avg = e4[1];
            restarted_at_check = false;
            if (termination_check_with(e4[0])) {
                // the outer loop's second termination_check! (pdlp.jl:88) re-evaluates sol
                termination_check_with(e4[0]);
                break;
            }
            if (prm.infeasibility_tol > 0) {
                const int32_t inf = infeasibility_check();
                if (inf != CPDLP_STILL_RUNNING) { status = inf; break; }
            }
            if (restart_check(e4)) {
                restart();
                restarted_at_check = true;
            }
        }
        return status;
    }

    void profile(int reps, double* ms) override {
        ProblemT<T>& P = *PT;
        cudaStream_t s = h->stream;
        const size_t nz = (size_t)std::max<int64_t>(P.n, 1), mz = (size_t)std::max<int64_t>(P.m, 1);
        DBuf<T> tx(nz), tb(nz), txa(nz), ty(mz), tya(mz), tys(P.pm1 ? mz : 1);
        if (!coef1.p) coef1.alloc(1);
        StepCoef<T> k = coef_for(eta_sum);
        CK(cudaMemcpyAsync(coef1.p, &k, sizeof(k), cudaMemcpyHostToDevice, s));
        const int o = cur;
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        auto timed = [&](auto&& launch) {
            launch();  // warm-up
            CK(cudaEventRecord(e0, s));
            for (int r = 0; r < reps; r++) launch();
            CK(cudaEventRecord(e1, s));
            CK(cudaEventSynchronize(e1));
            float t = 0;
            CK(cudaEventElapsedTime(&t, e0, e1));
            return (double)t / reps;
        };
        ms[0] = timed([&] {
            launch_primal(x[o].p, tx.p, tb.p, xa[o].p, txa.p, P.pm1 ? ys[o].p : y[o].p, coef1.p, s);
        });
        ms[1] = timed([&] {
            launch_dual(y[o].p, ty.p, P.pm1 ? tys.p : nullptr, ya[o].p, tya.p, xbar.p, coef1.p, s);
        });
        ms[2] = timed([&] {
            const T* const xs4[4] = {x[cur].p, xa[cur].p, x[cur ^ 1].p, xa[cur ^ 1].p};
            const T* const ys4[4] = {y[cur].p, ya[cur].p, y[cur ^ 1].p, ya[cur ^ 1].p};
            enqueue_kkt<4>(xs4, ys4);
        });
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }

    void kernel_bytes(double* bytes) const override {
        const ProblemT<T>& P = *PT;
        const double nnz = (double)P.nnz, m = (double)P.m, n = (double)P.n;
        const double sv = P.pm1 ? 0.0 : sizeof(T), si = sizeof(int32_t), sf = sizeof(T);
        const bool avg = prm.algorithm == CPDLP_ALGO_PDLP;
        // primal: A' values+indices, row pointer, gather y (m), read x c lv uv,
        // write x+ xbar (+ avg read/write); narrow: no values, read d2
        bytes[0] = nnz * (sv + si) + (n + 1) * si + sf * (m + (avg ? 8 : 6) * n) +
                   (P.pm1 ? sf * n : 0.0);
        // dual: A values+indices, row pointer, gather xbar (n), read y lc uc,
        // write y+ (+ avg read/write); narrow: no values, read d1, write D1 y+
        bytes[1] = nnz * (sv + si) + (m + 1) * si + sf * (n + (avg ? 6 : 4) * m) +
                   (P.pm1 ? 2 * sf * m : 0.0);
        // KKT of 4 pairs in one pass per side: both matrices once, the 4
        // gathered vectors per side (packed: counted once), bounds, the 4
        // epilogue vectors per side, D1/D2 inverses (in T); narrow: the row
        // scales and the column scales of the pack, once each.  The pack
        // itself (read 4 vectors, write them interleaved) is not counted.
        bytes[2] = 2 * nnz * (sv + si) + (m + n + 2) * si + sf * (4 * n + 4 * m) +
                   sf * (2 * m + 4 * m) + sf * (3 * n + 4 * n) + sf * (m + n) +
                   (P.pm1 ? sf * 2 * (m + n) : 0.0);
    }

    void early_exit_zero_problem() override {
        ProblemT<T>& P = *PT;
        k_proj_zero<T><<<grid_for(P.n, 256), 256, 0, h->stream>>>(x[cur].p, P.lv.p, P.uv.p, P.n);
        CK_LAUNCH();
        status = CPDLP_OPTIMAL;
        CK(cudaStreamSynchronize(h->stream));
    }

    void vectors(int which, double* hx, double* hy) override {
        ProblemT<T>& P = *PT;
        const T *vx, *vy;
        vec_of(which, vx, vy);
        DBuf<double> tmp((size_t)std::max<int64_t>(std::max(P.m, P.n), 1));
        cudaStream_t s = h->stream;
        if (hx && P.n > 0) {
            k_widen<T><<<grid_for(P.n, 256), 256, 0, s>>>(vx, tmp.p, P.n);
            CK_LAUNCH();
            order_to_user(P, 1, tmp.p, s);
            CK(cudaMemcpyAsync(hx, tmp.p, sizeof(double) * P.n, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
        if (hy && P.m > 0) {
            k_widen<T><<<grid_for(P.m, 256), 256, 0, s>>>(vy, tmp.p, P.m);
            CK_LAUNCH();
            order_to_user(P, 0, tmp.p, s);
            CK(cudaMemcpyAsync(hy, tmp.p, sizeof(double) * P.m, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
    }

    // get_solution (common.jl:233-235): unprecondition (preconditioning.jl:53-59)
    void solution(double* hx, double* hy) override {
        ProblemT<T>& P = *PT;
        DBuf<double> tx((size_t)std::max<int64_t>(P.n, 1)), ty((size_t)std::max<int64_t>(P.m, 1));
        cudaStream_t s = h->stream;
        if (P.n > 0) k_unscale<T><<<grid_for(P.n, 256), 256, 0, s>>>(x[cur].p, P.D2.p, tx.p, P.n);
        if (P.m > 0) k_unscale<T><<<grid_for(P.m, 256), 256, 0, s>>>(y[cur].p, P.D1.p, ty.p, P.m);
        CK_LAUNCH();
        order_to_user(P, 1, tx.p, s);
        order_to_user(P, 0, ty.p, s);
        if (hx && P.n > 0) CK(cudaMemcpyAsync(hx, tx.p, sizeof(double) * P.n, cudaMemcpyDeviceToHost, s));
        if (hy && P.m > 0) CK(cudaMemcpyAsync(hy, ty.p, sizeof(double) * P.m, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
};

template <class T>
StateBase* make_state(Handle& h, ProblemT<T>* P, const cpdlp_params* prm, const double* x0,
                      const double* y0, double eta0, double omega0) {
    double t0 = now_seconds();
    auto* S = new StateT<T>();
    std::unique_ptr<StateT<T>> guard(S);
    S->P = P;
    S->PT = P;
    S->h = &h;
    S->prm = *prm;
    S->starting_time = t0;
    cudaStream_t s = h.stream;
    const int64_t m = P->m, n = P->n;
    const size_t nz = (size_t)(n > 0 ? n : 1), mz = (size_t)(m > 0 ? m : 1);
    for (int b = 0; b < 2; b++) {
        S->x[b].alloc(nz); S->y[b].alloc(mz); S->xa[b].alloc(nz); S->ya[b].alloc(mz);
    }
    S->xr.alloc(nz); S->yr.alloc(mz); S->xbar.alloc(nz);
    // sol = precondition(sol_init): x ./ D2, y ./ D1 (preconditioning.jl:45-51)
    DBuf<double> tx(nz), ty(mz);
    if (x0 && n > 0) CK(cudaMemcpyAsync(tx.p, x0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    else CK(cudaMemsetAsync(tx.p, 0, sizeof(double) * nz, s));
    if (y0 && m > 0) CK(cudaMemcpyAsync(ty.p, y0, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    else CK(cudaMemsetAsync(ty.p, 0, sizeof(double) * mz, s));
    if (x0) order_to_internal(*P, 1, tx.p, s);
    if (y0) order_to_internal(*P, 0, ty.p, s);
    if (n > 0) k_prescale<T><<<grid_for(n, 256), 256, 0, s>>>(tx.p, P->D2.p, S->x[0].p, n);
    if (m > 0) k_prescale<T><<<grid_for(m, 256), 256, 0, s>>>(ty.p, P->D1.p, S->y[0].p, m);
    CK_LAUNCH();
    // sol_last = zero(sol), sol_avg = copy(sol), sol_avg_last = zero(sol), sol_restart = copy(sol)
    CK(cudaMemsetAsync(S->x[1].p, 0, sizeof(T) * nz, s));
    CK(cudaMemsetAsync(S->y[1].p, 0, sizeof(T) * mz, s));
    CK(cudaMemcpyAsync(S->xa[0].p, S->x[0].p, sizeof(T) * nz, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(S->ya[0].p, S->y[0].p, sizeof(T) * mz, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(S->xa[1].p, 0, sizeof(T) * nz, s));
    CK(cudaMemsetAsync(S->ya[1].p, 0, sizeof(T) * mz, s));
    CK(cudaMemcpyAsync(S->xr.p, S->x[0].p, sizeof(T) * nz, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(S->yr.p, S->y[0].p, sizeof(T) * mz, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(S->xbar.p, 0, sizeof(T) * nz, s));
    if (P->pm1) {
        for (int b = 0; b < 2; b++) S->ys[b].alloc(mz);
        CK(cudaMemsetAsync(S->ys[1].p, 0, sizeof(T) * mz, s));
        if (m > 0) {
            k_mul_vec<T><<<grid_for(m, 256), 256, 0, s>>>(S->y[0].p, P->d1t.p, S->ys[0].p, m);
            CK_LAUNCH();
        }
    }
    S->cur = 0;
    // fixed_stepsize (step_size.jl:22-27)
    if (eta0 > 0) {  // continuation of an earlier solve of the same LP
        S->eta = eta0;
        S->power_iterations = 0;
    } else {
        double sn = spectral_norm_T(h, *P, prm, &S->power_iterations, t0 + prm->time_limit);
        S->eta = prm->invnorm_scaling * (1.0 / sn);
    }
    // primal_weight_init (step_size.jl:29-40); PDHG: omega = 1 (pdhg.jl:48)
    if (prm->algorithm == CPDLP_ALGO_PDHG) {
        S->omega = 1.0;
    } else {
        unsigned g = red_grid(h, std::max(m, n));
        k_scales<T><<<g, RED_THREADS, 0, s>>>(P->lc.p, P->uc.p, P->invD1.p, m, P->c.p,
                                              P->invD2.p, n, P->red_rows.p);
        CK_LAUNCH();
        double q[4];
        fetch_reduced(h, P->red_rows.p, g, 4, P->red_out.p, q);
        const double c_norm = std::sqrt(q[3]), cb_norm = std::sqrt(q[1]);
        S->omega = (c_norm > prm->zero_tol && cb_norm > prm->zero_tol) ? c_norm / cb_norm : 1.0;
        if (omega0 > 0) S->omega = omega0;
    }
    S->eta_sum = 0.0;
    for (auto* e : {&S->err, &S->err_cand, &S->err_cand_last, &S->err_restart})
        e->primal = e->primal_scale = e->dual = e->dual_scale = e->gap = e->gap_scale = NAN;
    CK(cudaStreamSynchronize(s));
    if (trace_level() > 0)
        fprintf(stderr, "[cpdlp setup] %-28s %8.2f ms (%lld power iterations)\n",
                "state, power method", 1e3 * (now_seconds() - t0), (long long)S->power_iterations);
    S->setup_seconds = P->setup_seconds + (now_seconds() - t0);
    guard.release();
    return S;
}

// ---------------------------------------------------------------------------
// refinement on the residual LP (FP32 rounds, FP64 residuals)
// ---------------------------------------------------------------------------
// A round fixes a base point (x0, y0) of the scaled LP (FP64) and solves, with
// FP32 iterates, for the correction (dx, dy) of
//   min r'dx  s.t.  lc - A x0 <= A dx <= uc - A x0,  lv - x0 <= dx <= uv - x0,
// r = c - A'y0.  Its saddle function is the original one shifted by (x0, y0),
// so it has the same KKT errors; the dual step decides each row's activity on
// y0 + dy (DualEpi SHIFT).  The residual data are computed in FP64 and scaled
// by powers of two, dp on the primal side and dd on the dual side, so that the
// FP32 iterates resolve them.  After the round, x0 += dx/dp and y0 += dy/dd in
// FP64.
constexpr int REFINE_MAX_ROUNDS = 8;
// a round ends once the combined relative KKT error fell by this factor
constexpr double REFINE_ROUND_DECAY = 1e-4;
constexpr double REFINE_MAX_SCALE = 1099511627776.0;  // 2^40

// CPDLP_TRACE=1 in the environment prints one line per setup phase and per
// refinement round to stderr, CPDLP_TRACE=2 also one line per check
int trace_level() {
    static const int lvl = [] {
        const char* v = std::getenv("CPDLP_TRACE");
        return v ? std::atoi(v) : 0;
    }();
    return lvl;
}
bool trace_on() { return trace_level() > 0; }

__global__ void k_refine_rows(const double* __restrict__ lc, const double* __restrict__ uc,
                              const double* __restrict__ Ax0, const double* __restrict__ y0,
                              double dp, double dd, float* __restrict__ lco,
                              float* __restrict__ uco, double* __restrict__ yoff, int64_t m) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    lco[i] = (float)__dmul_rn(dp, __dsub_rn(lc[i], Ax0[i]));
    uco[i] = (float)__dmul_rn(dp, __dsub_rn(uc[i], Ax0[i]));
    yoff[i] = __dmul_rn(dd, y0[i]);
}
__global__ void k_refine_cols(const double* __restrict__ c, const double* __restrict__ lv,
                              const double* __restrict__ uv, const double* __restrict__ Aty0,
                              const double* __restrict__ x0, double dp, double dd,
                              float* __restrict__ co, float* __restrict__ lvo,
                              float* __restrict__ uvo, int64_t n) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    co[j] = (float)__dmul_rn(dd, __dsub_rn(c[j], Aty0[j]));
    lvo[j] = (float)__dmul_rn(dp, __dsub_rn(lv[j], x0[j]));
    uvo[j] = (float)__dmul_rn(dp, __dsub_rn(uv[j], x0[j]));
}
// combined iterate: x = proj(x0 + dx/dp, lv, uv); y = y0 + dy/dd restricted to
// the signs its row's bounds allow (>= 0 with only lc finite, <= 0 with only
// uc finite, 0 for a free row), as the dual step keeps them
template <class T>
__global__ void k_refine_combine(const double* x0, const T* __restrict__ dx, double inv_dp,
                                 const double* __restrict__ lv, const double* __restrict__ uv,
                                 double* xo, int64_t n, const double* y0,
                                 const T* __restrict__ dy, double inv_dd,
                                 const double* __restrict__ lc, const double* __restrict__ uc,
                                 double* yo, int64_t m) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
        xo[j] = proj_box(__dadd_rn(x0[j], __dmul_rn((double)dx[j], inv_dp)), lv[j], uv[j]);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double v = __dadd_rn(y0[i], __dmul_rn((double)dy[i], inv_dd));
        const bool lo = !isinf(lc[i]), up = !isinf(uc[i]);
        if (lo && !up) v = fmax(v, 0.0);
        else if (!lo && up) v = fmin(v, 0.0);
        else if (!lo && !up) v = 0.0;
        yo[i] = v;
    }
}

// Progress of an FP32 run, checked after every block: stalled once the error
// has not halved over `window` passes while at most `max_rel`, or over `long_window`
// passes at any level
struct StallWatch {
    double best = INFINITY;
    int64_t mark = 0;
    bool stalled(double rel, int64_t passes, int64_t window, int64_t long_window, double max_rel) {
        if (rel < 0.5 * best) {
            best = rel;
            mark = passes;
            return false;
        }
        const int64_t since = passes - mark;
        return (since >= window && best <= max_rel) || since >= long_window;
    }
};

double rel_err(const cpdlp_kkt_errors& e) {
    return jl_max(jl_max(e.primal / e.primal_scale, e.dual / e.dual_scale), e.gap / e.gap_scale);
}
// 2^k nearest below 1/v, within [1, 2^40]
double pow2_scale(double v) {
    if (!(v > 0.0)) return REFINE_MAX_SCALE;
    double sc = 1.0 / v;
    if (!(sc >= 1.0)) return 1.0;
    if (sc > REFINE_MAX_SCALE) return REFINE_MAX_SCALE;
    return std::exp2(std::floor(std::log2(sc)));
}

struct RefineResult {
    int32_t status = CPDLP_STILL_RUNNING;
    bool progress = true;  // false: a round did not halve the error (continue in FP64)
    int rounds = 0;
    int64_t passes = 0, launches = 0;
    int64_t first_gain = 0;  // passes the last round needed to first beat its base
    double omega = 1.0;    // primal weight in the original scaling
    cpdlp_kkt_errors err{};
    // the combined point's errors at every check of every round (original
    // units), passes counted from the start of the solve
    std::vector<int64_t> hist_passes;
    std::vector<cpdlp_kkt_errors> hist_err;
};

// Rounds from the base point (x0, y0) (FP64, scaled space) until refine_reltol,
// the pass or time limit, a round without progress or REFINE_MAX_ROUNDS.  P32's
// bound and cost vectors are overwritten with each round's residual data; S64
// is a state of P64 used for its FP64 KKT passes.
RefineResult refine_residual(Handle& h, ProblemT<float>& P32, ProblemT<double>& P64,
                             StateT<double>& S64, DBuf<double>& x0, DBuf<double>& y0,
                             const cpdlp_params& prm, double t0, double eta, double omega,
                             int64_t passes_left, int64_t passes_before) {
    RefineResult R;
    R.omega = omega;
    cudaStream_t s = h.stream;
    const int64_t m = P64.m, n = P64.n;
    const size_t nz = (size_t)std::max<int64_t>(n, 1), mz = (size_t)std::max<int64_t>(m, 1);
    DBuf<double> Ax0(mz), Aty0(nz), cx[4], cy[4];
    DBuf<double> yoff(mz);
    DBuf<float> bdx(nz), bdy(mz);  // the round's best correction
    for (int q = 0; q < 4; q++) {
        cx[q].alloc(nz);
        cy[q].alloc(mz);
    }
    const unsigned gc = red_grid(h, std::max(m, n));
    auto kkt_base = [&](cpdlp_kkt_errors* e) {
        const double* const xs[1] = {x0.p};
        const double* const ys[1] = {y0.p};
        S64.kkt_multi<1>(xs, ys, e);
    };
    cpdlp_kkt_errors e;
    kkt_base(&e);
    const int ce = prm.check_every > 0 ? prm.check_every : 100;
    for (;;) {
        R.err = e;
        const double r0 = rel_err(e);
        if (r0 <= prm.refine_reltol) { R.status = CPDLP_OPTIMAL; break; }
        if (now_seconds() - t0 >= prm.time_limit) { R.status = CPDLP_TIME_LIMIT; break; }
        if (passes_left <= 0) { R.status = CPDLP_ITERATION_LIMIT; break; }
        if (R.rounds >= REFINE_MAX_ROUNDS) { R.progress = false; break; }
        const double ep = e.primal / e.primal_scale, ed = e.dual / e.dual_scale,
                     eg = e.gap / e.gap_scale;
        const double dp = pow2_scale(jl_max(ep, eg)), dd = pow2_scale(jl_max(ed, eg));
        // the round's residual LP, in P32's vectors
        launch_side(P64, 0, view_A(P64), VecSet<double, 1>{{x0.p}}, StoreEpi<double>{Ax0.p}, s);
        launch_side(P64, 1, view_At(P64), VecSet<double, 1>{{y0.p}},
                        StoreEpi<double>{Aty0.p}, s);
        if (m > 0)
            k_refine_rows<<<grid_for(m, 256), 256, 0, s>>>(P64.lc.p, P64.uc.p, Ax0.p, y0.p, dp, dd,
                                                           P32.lc.p, P32.uc.p, yoff.p, m);
        if (n > 0)
            k_refine_cols<<<grid_for(n, 256), 256, 0, s>>>(P64.c.p, P64.lv.p, P64.uv.p, Aty0.p,
                                                           x0.p, dp, dd, P32.c.p, P32.lv.p,
                                                           P32.uv.p, n);
        CK_LAUNCH();
        R.launches += tiles_launches(P64.planA) + tiles_launches(P64.planAt) + 2;
        cpdlp_params pr = prm;
        pr.float_type = CPDLP_VAL_F32;
        pr.termination_reltol = 0.0;  // the rounds' own rule below decides
        pr.max_kkt_passes = passes_left;
        pr.infeasibility_tol = 0.0;   // rays of the residual LP would need its shifted cones
        std::unique_ptr<StateBase> SB(
            make_state<float>(h, &P32, &pr, nullptr, nullptr, eta, R.omega * dd / dp));
        auto& S = static_cast<StateT<float>&>(*SB);
        S.starting_time = t0;
        S.yoff = yoff.p;
        cpdlp_kkt_errors e_cur = e, e_avg = e;
        S.kkt_hook = [&](int nv, const float* const* xs, const float* const* ys,
                         cpdlp_kkt_errors* o) {
            for (int q = 0; q < nv; q++)
                k_refine_combine<float><<<gc, RED_THREADS, 0, s>>>(
                    x0.p, xs[q], 1.0 / dp, P64.lv.p, P64.uv.p, cx[q].p, n, y0.p, ys[q], 1.0 / dd,
                    P64.lc.p, P64.uc.p, cy[q].p, m);
            CK_LAUNCH();
            S.launches += nv;
            if (nv == 4) {
                const double* const X[4] = {cx[0].p, cx[1].p, cx[2].p, cx[3].p};
                const double* const Y[4] = {cy[0].p, cy[1].p, cy[2].p, cy[3].p};
                S64.kkt_multi<4>(X, Y, o);
                e_cur = o[0];  // the current iterate (checked after every block)
                e_avg = o[1];
            } else {
                const double* const X[1] = {cx[0].p};
                const double* const Y[1] = {cy[0].p};
                S64.kkt_multi<1>(X, Y, o);
                if (!S.pdlp()) e_cur = o[0];  // PDHG checks sol alone
            }
            // the residual LP's errors in its own (dp, dd) scaling, for the
            // restart rule and the primal weight
            for (int q = 0; q < nv; q++) {
                o[q].primal *= dp;
                o[q].dual *= dd;
                o[q].gap *= dp * dd;
            }
        };
        const double target = jl_max(prm.refine_reltol, REFINE_ROUND_DECAY * r0);
        // a round counts as stalled once it gained a factor 100 and stopped
        // halving, or after FP32_STALL_LONG windows without halving (a round
        // restarts PDLP cold, and its first halving can take 20,000 passes)
        StallWatch watch;
        const char* why = "limit";
        // the best correction seen at a check (sol or its average), kept so that
        // the base point never gets worse; the base itself (dx = 0) has r0
        double best_rel = r0;
        bool have_best = false;
        int64_t first_gain = -1;  // the round's passes when it first beat r0
        int64_t outer_before = S.outer;
        for (;;) {
            const int32_t st = S.solve_blocks(1);
            if (prm.record_error_history) {
                R.hist_passes.push_back(passes_before + R.passes + S.kkt_passes);
                R.hist_err.push_back(e_cur);
            }
            if (st != CPDLP_STILL_RUNNING) break;
            // candidates: sol and its average; a restart at the check moved the
            // chosen one (the average if restart_from_avg) into sol
            const bool restarted = S.outer != outer_before;
            outer_before = S.outer;
            const double r_sol = restarted && S.restart_from_avg ? rel_err(e_avg) : rel_err(e_cur);
            const double r_avg = (S.pdlp() && !restarted) ? rel_err(e_avg) : INFINITY;
            const bool use_avg = r_avg < r_sol;
            const double rc = jl_min(r_sol, r_avg);
            if (rc < best_rel) {
                if (first_gain < 0) first_gain = S.kkt_passes;
                best_rel = rc;
                have_best = true;
                CK(cudaMemcpyAsync(bdx.p, use_avg ? S.xa[S.cur].p : S.x[S.cur].p,
                                   sizeof(float) * nz, cudaMemcpyDeviceToDevice, s));
                CK(cudaMemcpyAsync(bdy.p, use_avg ? S.ya[S.cur].p : S.y[S.cur].p,
                                   sizeof(float) * mz, cudaMemcpyDeviceToDevice, s));
            }
            if (trace_level() > 1)
                fprintf(stderr, "[cpdlp refine]   %.3fs %lld: rel %.3e (p %.2e d %.2e g %.2e) omega %.3g\n",
                        now_seconds() - t0, (long long)S.kkt_passes, rc, e_cur.primal / e_cur.primal_scale,
                        e_cur.dual / e_cur.dual_scale, e_cur.gap / e_cur.gap_scale, S.omega);
            if (rc <= target) { why = "target"; break; }
            // a later round (the error already small) that has not improved at
            // all ends after 3 stall windows (90 checks), or after twice the
            // passes the previous round needed for its first gain if that is
            // longer (a cold PDLP start on a hard residual LP can take
            // thousands of checks to beat its base point)
            if (R.rounds > 0 && best_rel >= r0 &&
                S.kkt_passes >= std::max<int64_t>(3 * FP32_STALL_CHECKS * (int64_t)ce,
                                                  2 * R.first_gain)) {
                why = "no gain";
                break;
            }
            if (watch.stalled(rc, S.kkt_passes, FP32_STALL_CHECKS * (int64_t)ce,
                              FP32_STALL_LONG * FP32_STALL_CHECKS * (int64_t)ce, 1e-2 * r0)) {
                why = "stall";
                break;
            }
        }
        // the new base point: the best correction added in FP64 (none: the base
        // stays)
        if (have_best) {
            k_refine_combine<float><<<gc, RED_THREADS, 0, s>>>(x0.p, bdx.p, 1.0 / dp, P64.lv.p,
                                                              P64.uv.p, x0.p, n, y0.p, bdy.p,
                                                              1.0 / dd, P64.lc.p, P64.uc.p, y0.p, m);
            CK_LAUNCH();
        }
        R.launches += S.launches + 1;
        R.passes += S.kkt_passes;
        passes_left -= S.kkt_passes;
        R.first_gain = first_gain > 0 ? first_gain : 0;
        R.omega = S.omega * dp / dd;
        R.rounds++;
        kkt_base(&e);
        if (trace_on())
            fprintf(stderr,
                    "[cpdlp refine] %.2fs round %d: rel %.3e (p %.2e d %.2e g %.2e) dp %.3g dd %.3g "
                    "-> %.3e after %lld passes (%s, %lld restarts)\n",
                    now_seconds() - t0, R.rounds, r0, ep, ed, eg, dp, dd, rel_err(e), (long long)S.kkt_passes, why,
                    (long long)S.outer);
        if (!(rel_err(e) <= 0.5 * r0)) {
            R.err = e;
            R.progress = false;
            break;
        }
    }
    if (prm.record_error_history) {  // the final base point
        R.hist_passes.push_back(passes_before + R.passes);
        R.hist_err.push_back(R.err);
    }
    R.launches += S64.launches;
    return R;
}

}  // namespace

void StateBase::stats(cpdlp_stats* st) const {
    memset(st, 0, sizeof(*st));
    st->err = err;
    st->time_elapsed = time_elapsed;
    st->kkt_passes = kkt_passes;
    st->termination_status = status;
    st->restart_from_avg = restart_from_avg;
    st->outer = outer;
    st->inner = inner;
    st->total = total;
    st->eta = eta;
    st->eta_sum = eta_sum;
    st->omega = omega;
    st->history_length = (int64_t)hist_passes.size();
    st->power_iterations = power_iterations;
    st->refine_kkt_passes = refine_passes;
    st->setup_seconds = setup_seconds;
    st->kernel_launches = launches;
}

ProblemBase* problem_create(Handle& h, const cpdlp_lp* lp, const cpdlp_params* prm, bool plans) {
    if (!lp || !prm) fail(CPDLP_ERR_ARGUMENT, "null lp or params");
    if (lp->m < 0 || lp->n < 0) fail(CPDLP_ERR_DIMENSION, "negative problem size");
    if (prm->tile_flags & ~(CPDLP_TILE_NO_NARROW | CPDLP_TILE_DENSITY_ORDER | CPDLP_TILE_NO_DENSITY_ORDER))
        fail(CPDLP_ERR_ARGUMENT, "unknown tile_flags bits");
    if (prm->float_type == CPDLP_VAL_F32) return make_problem<float>(h, lp, prm, plans);
    if (prm->float_type == CPDLP_VAL_F64) return make_problem<double>(h, lp, prm, plans);
    fail(CPDLP_ERR_ARGUMENT, "float_type must be CPDLP_VAL_F64 or CPDLP_VAL_F32");
}

StateBase* state_create(Handle& h, ProblemBase* P, const cpdlp_params* prm, const double* x0,
                        const double* y0, double eta0, double omega0) {
    if (!P || !prm) fail(CPDLP_ERR_ARGUMENT, "null problem or params");
    if (prm->check_every <= 0) fail(CPDLP_ERR_ARGUMENT, "check_every must be positive");
    if (P->vt == CPDLP_VAL_F32)
        return make_state<float>(h, static_cast<ProblemT<float>*>(P), prm, x0, y0, eta0, omega0);
    return make_state<double>(h, static_cast<ProblemT<double>*>(P), prm, x0, y0, eta0, omega0);
}

double problem_spectral_norm(Handle& h, ProblemBase* P, const cpdlp_params* prm, int64_t* iters) {
    if (P->vt == CPDLP_VAL_F32)
        return spectral_norm_T<float>(h, *static_cast<ProblemT<float>*>(P), prm, iters);
    return spectral_norm_T<double>(h, *static_cast<ProblemT<double>*>(P), prm, iters);
}

void solve_full(Handle& h, const cpdlp_lp* lp, const cpdlp_params* params, const double* x0,
                const double* y0, double* x_out, double* y_out, cpdlp_stats* stats) {
    const double t0 = now_seconds();
    h.solve_hist_passes.clear();
    h.solve_hist_err.clear();
    // appends a state's history, its passes offset by `base`
    auto keep_history = [&h](const StateBase& S, int64_t base) {
        for (size_t t = 0; t < S.hist_passes.size(); t++) {
            h.solve_hist_passes.push_back(base + S.hist_passes[t]);
            h.solve_hist_err.push_back(S.hist_err[t]);
        }
    };
    std::unique_ptr<ProblemBase> P(problem_create(h, lp, params));
    std::unique_ptr<StateBase> S(state_create(h, P.get(), params, x0, y0));
    S->starting_time = t0;
    const bool mixed = params->float_type == CPDLP_VAL_F32 && params->refine_reltol > 0;
    bool stalled = false;
    double fp32_best = INFINITY;      // mixed: the FP32 phase's best point
    DBuf<float> best_x, best_y;
    if (P->m == 0 && P->zero_cost) {
        S->early_exit_zero_problem();  // common.jl:194-198
    } else if (mixed) {
        // FP32 phase, one check at a time, until a stall or the tighter of the
        // two tolerances (FP32 iterates often get well below termination_reltol)
        StallWatch watch;
        S->prm.termination_reltol = std::min(params->termination_reltol,
                                             params->refine_reltol > 0 ? params->refine_reltol
                                                                       : INFINITY);
        const int64_t win = FP32_STALL_CHECKS * (int64_t)params->check_every;
        auto& S32 = static_cast<StateT<float>&>(*S);
        const size_t nz1 = (size_t)std::max<int64_t>(P->n, 1), mz1 = (size_t)std::max<int64_t>(P->m, 1);
        while (S->solve_blocks(1) == CPDLP_STILL_RUNNING) {
            const cpdlp_kkt_errors& e = S->err;
            // candidates: sol and its average (the current iterate's error is
            // noisy); a restart at the check moved the chosen one into sol
            const bool rs = S32.restarted_at_check;
            const double r_sol = rs && S32.restart_from_avg ? rel_err(S32.err_avg) : rel_err(e);
            const double r_avg = (S32.pdlp() && !rs) ? rel_err(S32.err_avg) : INFINITY;
            const double rel = jl_min(r_sol, r_avg);
            if (rel < fp32_best) {  // the refinement starts from the best point
                fp32_best = rel;
                if (!best_x.p) {
                    best_x.alloc(nz1);
                    best_y.alloc(mz1);
                }
                const bool ua = r_avg < r_sol;
                CK(cudaMemcpyAsync(best_x.p, ua ? S32.xa[S32.cur].p : S32.x[S32.cur].p,
                                   sizeof(float) * nz1, cudaMemcpyDeviceToDevice, h.stream));
                CK(cudaMemcpyAsync(best_y.p, ua ? S32.ya[S32.cur].p : S32.y[S32.cur].p,
                                   sizeof(float) * mz1, cudaMemcpyDeviceToDevice, h.stream));
            }
            if (trace_level() > 1)
                fprintf(stderr, "[cpdlp refine]   %.3fs FP32 %lld: rel %.3e (p %.2e d %.2e g %.2e)\n",
                        now_seconds() - t0, (long long)S->kkt_passes, rel, e.primal / e.primal_scale,
                        e.dual / e.dual_scale, e.gap / e.gap_scale);
            if (watch.stalled(rel, S->kkt_passes, win, FP32_STALL_LONG * win, FP32_STALL_REL)) {
                stalled = true;
                break;
            }
        }
    } else {
        const double ts = now_seconds();
        S->solve();
        if (trace_on())
            fprintf(stderr, "[cpdlp setup] %-28s %8.2f ms (%lld passes)\n", "solve", 1e3 * (now_seconds() - ts),
                    (long long)S->kkt_passes);
    }
    if (mixed && trace_on())
        fprintf(stderr, "[cpdlp refine] %.2fs FP32 phase: rel %.3e (best %.3e) after %lld passes%s\n",
                now_seconds() - t0, rel_err(S->err), fp32_best, (long long)S->kkt_passes,
                stalled ? " (stalled)" : "");
    // refinement: the FP32 iterates stalled before the tolerance
    const bool refine = mixed && stalled;
    keep_history(*S, 0);
    if (!refine) {
        const double ts = now_seconds();
        S->solution(x_out, y_out);
        if (trace_on())
            fprintf(stderr, "[cpdlp setup] %-28s %8.2f ms\n", "solution to the host", 1e3 * (now_seconds() - ts));
        if (stats) {
            S->stats(stats);
            stats->history_length = (int64_t)h.solve_hist_passes.size();
        }
        return;
    }
    // Refinement on the residual LP: FP32 rounds from the FP32 solution, with
    // the residuals, the combination and the KKT errors in FP64 (the step size
    // is a property of A and carries over, and the rounds start from the FP32
    // run's primal weight)
    cpdlp_stats st32;
    S->stats(&st32);
    const double eta32 = S->eta, omega32 = S->omega;
    auto& P32 = static_cast<ProblemT<float>&>(*P);
    const int64_t m = P->m, n = P->n;
    const size_t nz = (size_t)std::max<int64_t>(n, 1), mz = (size_t)std::max<int64_t>(m, 1);
    DBuf<double> bx(nz), by(mz);
    {
        // the base point: the FP32 phase's best point at a check
        auto& S32 = static_cast<StateT<float>&>(*S);
        const float* xb = best_x.p ? best_x.p : S32.x[S32.cur].p;
        const float* yb = best_y.p ? best_y.p : S32.y[S32.cur].p;
        if (n > 0) k_widen<float><<<grid_for(n, 256), 256, 0, h.stream>>>(xb, bx.p, n);
        if (m > 0) k_widen<float><<<grid_for(m, 256), 256, 0, h.stream>>>(yb, by.p, m);
        CK_LAUNCH();
    }
    S.reset();
    cpdlp_params p64 = *params;
    p64.float_type = CPDLP_VAL_F64;
    p64.termination_reltol = params->refine_reltol;
    // the FP64 copy takes the FP32 problem's order (the rounds combine their
    // vectors elementwise)
    p64.tile_flags = (p64.tile_flags & ~(CPDLP_TILE_DENSITY_ORDER | CPDLP_TILE_NO_DENSITY_ORDER)) |
                     (P->ordered ? CPDLP_TILE_DENSITY_ORDER : CPDLP_TILE_NO_DENSITY_ORDER);
    std::unique_ptr<ProblemBase> P64(problem_create(h, lp, &p64));
    auto& Q64 = static_cast<ProblemT<double>&>(*P64);
    std::unique_ptr<StateBase> S64(state_create(h, P64.get(), &p64, nullptr, nullptr, eta32, omega32));
    auto& T64 = static_cast<StateT<double>&>(*S64);
    const RefineResult R = refine_residual(h, P32, Q64, T64, bx, by, *params, t0, eta32, omega32,
                                           params->max_kkt_passes - st32.kkt_passes,
                                           st32.kkt_passes);
    h.solve_hist_passes.insert(h.solve_hist_passes.end(), R.hist_passes.begin(),
                               R.hist_passes.end());
    h.solve_hist_err.insert(h.solve_hist_err.end(), R.hist_err.begin(), R.hist_err.end());
    int64_t passes = st32.kkt_passes + R.passes;
    int64_t launches = st32.kernel_launches + R.launches;
    if (R.progress || R.status != CPDLP_STILL_RUNNING) {
        if (n > 0) k_unscale<double><<<grid_for(n, 256), 256, 0, h.stream>>>(bx.p, Q64.D2.p, T64.xr.p, n);
        if (m > 0) k_unscale<double><<<grid_for(m, 256), 256, 0, h.stream>>>(by.p, Q64.D1.p, T64.yr.p, m);
        CK_LAUNCH();
        order_to_user(Q64, 1, T64.xr.p, h.stream);
        order_to_user(Q64, 0, T64.yr.p, h.stream);
        if (x_out && n > 0)
            CK(cudaMemcpyAsync(x_out, T64.xr.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h.stream));
        if (y_out && m > 0)
            CK(cudaMemcpyAsync(y_out, T64.yr.p, sizeof(double) * m, cudaMemcpyDeviceToHost, h.stream));
        CK(cudaStreamSynchronize(h.stream));
        if (stats) {
            *stats = st32;
            stats->err = R.err;
            stats->termination_status = R.status;
            stats->kkt_passes = passes;
            stats->refine_kkt_passes = R.passes;
            stats->omega = R.omega;
            stats->time_elapsed = now_seconds() - t0;
            stats->kernel_launches = launches;
            stats->history_length = (int64_t)h.solve_hist_passes.size();
        }
        return;
    }
    // a round made no progress: continue in FP64 from the refined point
    if (trace_on())
        fprintf(stderr, "[cpdlp refine] %.2fs no progress after %d rounds: FP64 continuation\n",
                now_seconds() - t0, R.rounds);
    std::vector<double> xs(nz), ys(mz);
    if (n > 0) k_unscale<double><<<grid_for(n, 256), 256, 0, h.stream>>>(bx.p, Q64.D2.p, T64.xr.p, n);
    if (m > 0) k_unscale<double><<<grid_for(m, 256), 256, 0, h.stream>>>(by.p, Q64.D1.p, T64.yr.p, m);
    CK_LAUNCH();
    // in the caller's order: the continuation's state takes them as a start
    order_to_user(Q64, 1, T64.xr.p, h.stream);
    order_to_user(Q64, 0, T64.yr.p, h.stream);
    if (n > 0) CK(cudaMemcpyAsync(xs.data(), T64.xr.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h.stream));
    if (m > 0) CK(cudaMemcpyAsync(ys.data(), T64.yr.p, sizeof(double) * m, cudaMemcpyDeviceToHost, h.stream));
    CK(cudaStreamSynchronize(h.stream));
    S64.reset();
    P.reset();
    p64.max_kkt_passes = std::max<int64_t>(params->max_kkt_passes - passes, 1);
    // the primal weight continues from the rounds'
    std::unique_ptr<StateBase> C64(
        state_create(h, P64.get(), &p64, xs.data(), ys.data(), eta32, R.omega));
    C64->starting_time = t0;
    C64->solve();
    keep_history(*C64, passes);
    // the continuation can end at a limit with a worse current iterate than
    // the refined point it started from (PDLP's iterate error is not
    // monotone): the refined point is returned then
    const bool keep_base = C64->status != CPDLP_OPTIMAL && !(rel_err(C64->err) <= rel_err(R.err));
    if (keep_base) {
        if (x_out && n > 0) memcpy(x_out, xs.data(), sizeof(double) * n);
        if (y_out && m > 0) memcpy(y_out, ys.data(), sizeof(double) * m);
        if (params->record_error_history) {  // the returned point's errors close the history
            h.solve_hist_passes.push_back(passes + C64->kkt_passes);
            h.solve_hist_err.push_back(R.err);
        }
    } else {
        C64->solution(x_out, y_out);
    }
    if (stats) {
        C64->stats(stats);
        if (keep_base) stats->err = R.err;
        stats->refine_kkt_passes = R.passes + C64->kkt_passes;
        stats->kkt_passes = passes + C64->kkt_passes;
        stats->kernel_launches += launches;
        stats->history_length = (int64_t)h.solve_hist_passes.size();
    }
    if (trace_on())
        fprintf(stderr, "[cpdlp refine] %.2fs FP64 continuation: rel %.3e after %lld passes%s\n",
                now_seconds() - t0, rel_err(C64->err), (long long)C64->kkt_passes,
                keep_base ? " (worse than the refined point, which is returned)" : "");
}

void problem_scaling(Handle& h, ProblemBase* P, double* d1, double* d2) {
    for (int sd = 0; sd < 2; sd++) {
        double* out = sd == 0 ? d1 : d2;
        const int64_t len = sd == 0 ? P->m : P->n;
        if (!out || len <= 0) continue;
        DBuf<double> t((size_t)len);
        CK(cudaMemcpyAsync(t.p, (sd == 0 ? P->D1 : P->D2).p, sizeof(double) * len,
                           cudaMemcpyDeviceToDevice, h.stream));
        order_to_user(*P, sd, t.p, h.stream);
        CK(cudaMemcpyAsync(out, t.p, sizeof(double) * len, cudaMemcpyDeviceToHost, h.stream));
        CK(cudaStreamSynchronize(h.stream));
    }
}

}  // namespace cpdlp
