// epilogues.cuh -- the fused per-row epilogues of the tile SpMV engine:
// PDHG steps (pdlp.jl:108-117, :126-136), KKT error terms (errors.jl:65-109),
// the power method (linalg.jl:60-96) and a plain store.
//
// Epilogue interface (per row r, per input vector p):
//   struct Pre;                      inputs of one row, loaded before the gathers
//   Pre pre_global(int r) const;     loads them
//   void row(int p, int r, T s, const Pre&, Acc&)   rows of short tiles
//   void row_long(int p, int r, T s, int lid, Acc&)  long rows (one lane)
//   void init(Acc&); void finish(Acc&);             block reductions
// Every load of a vector that a kernel may itself have written earlier (the
// in-kernel step loop of the batched solver) is a coherent load.
#pragma once

#include "cpdlp_common.cuh"
#include "solver.cuh"
#include "tiles.cuh"

namespace cpdlp {

struct NoAcc {};

template <class T>
struct StoreEpi {  // out = s (mul! with alpha = true, beta = false)
    T* out;
    using Acc = NoAcc;
    struct Pre {};
    __device__ Pre pre_global(int) const { return Pre{}; }
    __device__ void init(Acc&) {}
    __device__ void row(int, int r, T s, const Pre&, Acc&) { out[r] = s; }
    __device__ void row_long(int, int r, T s, int, Acc&) { out[r] = s; }
    __device__ void finish(Acc&) {}
};

// out_i = d_i * (d_i * s): the power method's first product over a Pm1 matrix
// (s = (S D2 x)_i, so d1_i s is (A x)_i and the next product gathers d1 .* (A x))
template <class T>
struct ScaledStoreEpi {
    T* out;
    const T* __restrict__ dsc;
    using Acc = NoAcc;
    struct Pre {};
    __device__ Pre pre_global(int) const { return Pre{}; }
    __device__ void init(Acc&) {}
    __device__ void row(int, int r, T s, const Pre&, Acc&) {
        const T d = dsc[r];
        out[r] = mul_rn(d, mul_rn(d, s));
    }
    __device__ void row_long(int p, int r, T s, int, Acc& a) { row(p, r, s, Pre{}, a); }
    __device__ void finish(Acc&) {}
};

// Step coefficients tau, sigma, 1/sigma and the averaging weights: read from
// device memory written before the launch (graph-captured step kernels), or
// carried by value (the batched kernel, which changes them between steps
// inside one launch).
template <class T, bool BYVAL>
struct CoefSrc;
template <class T>
struct CoefSrc<T, false> {
    const StepCoef<T>* __restrict__ coef;
    __device__ __forceinline__ const StepCoef<T>& get() const { return *coef; }
};
template <class T>
struct CoefSrc<T, true> {
    StepCoef<T> k;
    __device__ __forceinline__ const StepCoef<T>& get() const { return k; }
};

// SCALED (the +-1 storage of Pm1 matrices): the stored matrix is the sign
// pattern S of A, the scaled matrix is D1 S D2, so the product gathers the
// pre-scaled vector (D1 y here), the row sum is multiplied by this row's scale
// (d2_j), and xbar receives the pre-scaled D2 xbar that the dual product
// gathers (the extrapolated point itself is needed nowhere else).
template <class T, bool BYVAL = false, bool SCALED = false>
struct PrimalEpi {
    const T* __restrict__ x;
    const T* __restrict__ c;
    const T* __restrict__ lv;
    const T* __restrict__ uv;
    T* __restrict__ xn;
    T* __restrict__ xbar;
    const T* __restrict__ xa_old;
    T* __restrict__ xa_new;
    CoefSrc<T, BYVAL> coef;
    int avg;
    const T* __restrict__ dsc;  // SCALED: d2
    using Acc = NoAcc;
    struct Pre { T x, c, lv, uv, xa, d; };
    __device__ __forceinline__ Pre pre_global(int j) const {
        return Pre{ld_stream(x + j), ld_stream(c + j), ld_stream(lv + j), ld_stream(uv + j),
                   avg ? ld_stream(xa_old + j) : T(0), SCALED ? ld_stream(dsc + j) : T(0)};
    }
    __device__ void init(Acc&) {}
    __device__ __forceinline__ void row(int, int j, T s, const Pre& q, Acc&) {
        const StepCoef<T>& k = coef.get();
        if (SCALED) s = mul_rn(q.d, s);
        const T xp = proj_box(sub_rn(q.x, mul_rn(k.tau, sub_rn(q.c, s))), q.lv, q.uv);
        __stcs(xn + j, xp);
        const T xb = sub_rn(mul_rn(T(2), xp), q.x);
        xbar[j] = SCALED ? mul_rn(q.d, xb) : xb;
        if (avg) __stcs(xa_new + j, add_rn(mul_rn(xp, k.a), mul_rn(q.xa, k.b)));
    }
    __device__ void row_long(int p, int j, T s, int, Acc& a) { row(p, j, s, pre_global(j), a); }
    __device__ void finish(Acc&) {}
};

// SCALED: the product gathers D2 xbar, the row sum is multiplied by d1_i, and
// the epilogue also writes d1 .* y+ for the next primal product.
// SHIFT (a refinement round on the residual LP, whose multipliers are the
// corrections dy to base multipliers y0): the projection that decides each
// row's activity sees the whole multiplier, (yoff_i + dy_i)/sigma - s, with
// yoff the scaled base multipliers; the rest of the step acts on dy.  yoff is
// FP64 and so is this row's arithmetic: yoff can exceed dy by many orders of
// magnitude, and the activity decision needs dy's precision.
template <class T, bool BYVAL = false, bool SCALED = false, bool SHIFT = false>
struct DualEpi {
    const T* __restrict__ y;
    const T* __restrict__ lc;
    const T* __restrict__ uc;
    T* __restrict__ yn;
    const T* __restrict__ ya_old;
    T* __restrict__ ya_new;
    CoefSrc<T, BYVAL> coef;
    int avg;
    const T* __restrict__ dsc;   // SCALED: d1
    T* __restrict__ ysn;         // SCALED: d1 .* y+
    const double* __restrict__ yoff;  // SHIFT: scaled base multipliers
    using Acc = NoAcc;
    struct Pre { T y, lc, uc, ya, d; };
    __device__ __forceinline__ Pre pre_global(int i) const {
        return Pre{ld_stream(y + i), ld_stream(lc + i), ld_stream(uc + i),
                   avg ? ld_stream(ya_old + i) : T(0), SCALED ? ld_stream(dsc + i) : T(0)};
    }
    __device__ void init(Acc&) {}
    __device__ __forceinline__ void row(int, int i, T s, const Pre& q, Acc&) {
        const StepCoef<T>& k = coef.get();
        if (SCALED) s = mul_rn(q.d, s);
        const T sigma = k.sigma;
        T yp;
        if constexpr (SHIFT) {
            // read here, not prefetched with the row's other inputs: an FP64
            // value per prefetched row doubled the kernel's registers
            const double yo = ld_stream(yoff + i);
            const double sd = (double)s, sg = (double)sigma;
            const double t4 = __dsub_rn(__dmul_rn((double)k.inv_sigma, __dadd_rn(yo, (double)q.y)), sd);
            const double pr = proj_box(t4, -(double)q.uc, -(double)q.lc);
            yp = (T)__dsub_rn(__dsub_rn((double)q.y, __dmul_rn(sg, sd)), __dmul_rn(sg, pr));
        } else {
            const T t2 = sub_rn(q.y, mul_rn(sigma, s));
            const T t4 = sub_rn(mul_rn(k.inv_sigma, q.y), s);
            const T pr = proj_box(t4, -q.uc, -q.lc);
            yp = sub_rn(t2, mul_rn(sigma, pr));
        }
        yn[i] = yp;
        if (SCALED) ysn[i] = mul_rn(q.d, yp);
        if (avg) __stcs(ya_new + i, add_rn(mul_rn(yp, k.a), mul_rn(q.ya, k.b)));
    }
    __device__ void row_long(int p, int i, T s, int, Acc& a) { row(p, i, s, pre_global(i), a); }
    __device__ void finish(Acc&) {}
};

// The KKT pass evaluates NV (1 or 4) iterates (x_p, y_p) in one launch per
// side (four: packed gathers, short_tile4, whose iterate index is a constant
// at every epilogue call, so the accumulators stay in registers).  A block of
// W warps reduces its threads' FP64 sums in a fixed order; an iterate's sums
// do not depend on the other iterates of the launch.
// Each row's terms are computed in the iterate type T (FP64 arithmetic is
// scarce on GB300, and a term's own rounding is relative to that term) and
// accumulated in FP64: the squares from the T value widened, so they cannot
// overflow.  With T = double this is the FP64 evaluation of errors.jl.
// KKT row side (errors.jl:73-80, 87-89): s = (A x_p)_i (SCALED: the product
// gathered D2 x_p and s is multiplied by d1_i)
template <class T, int NV, bool SCALED = false, int W = TILE_WARPS>
struct KktRowEpi {
    const T* __restrict__ lc;
    const T* __restrict__ uc;
    const T* __restrict__ invD1;   // 1 ./ D1 in T
    const T* y[NV];
    double* block_out;
    double* long_out;
    const T* __restrict__ dsc = nullptr;
    struct Acc { double v[2 * NV]; };
    // inputs are read when the row is reduced (no prefetch): four iterates
    // per row would cost too many registers
    struct Pre {};
    __device__ void init(Acc& a) {
#pragma unroll
        for (int q = 0; q < 2 * NV; q++) a.v[q] = 0.0;
    }
    __device__ __forceinline__ Pre pre_global(int) const { return Pre{}; }
    __device__ __forceinline__ void terms(int p, int i, T s, double& pr2, double& pc) const {
        if (SCALED) s = mul_rn(dsc[i], s);
        const T l = lc[i], u = uc[i];
        const double d = (double)mul_rn(invD1[i], sub_rn(s, proj_box(s, l, u)));
        pr2 = __dmul_rn(d, d);
        const T yy = pick(y, p)[i];  // y[] is not restrict: a coherent load
        pc = (double)sub_rn(safeprod_left(u, pos_part(-yy)), safeprod_left(l, neg_part(-yy)));
    }
    __device__ __forceinline__ void row(int p, int i, T s, const Pre&, Acc& a) {
        double pr2, pc;
        terms(p, i, s, pr2, pc);
        a.v[2 * p] += pr2;
        a.v[2 * p + 1] += pc;
    }
    __device__ void row_long(int p, int i, T s, int lid, Acc&) {
        double pr2, pc;
        terms(p, i, s, pr2, pc);
        long_out[(size_t)lid * 2 * NV + 2 * p] = pr2;
        long_out[(size_t)lid * 2 * NV + 2 * p + 1] = pc;
    }
    __device__ void finish(Acc& a) { block_reduce_store<2 * NV, W>(a.v, block_out); }
};

// KKT column side (errors.jl:74-75, 82-95): s = (A' y_p)_j (SCALED: the
// product gathered D1 y_p and s is multiplied by d2_j)
template <class T, int NV, bool SCALED = false, int W = TILE_WARPS>
struct KktColEpi {
    const T* __restrict__ c;
    const T* __restrict__ lv;
    const T* __restrict__ uv;
    const T* __restrict__ invD2;   // 1 ./ D2 in T
    const T* x[NV];
    double* block_out;
    double* long_out;
    const T* __restrict__ dsc = nullptr;
    struct Acc { double v[3 * NV]; };
    struct Pre {};
    __device__ void init(Acc& a) {
#pragma unroll
        for (int q = 0; q < 3 * NV; q++) a.v[q] = 0.0;
    }
    __device__ __forceinline__ Pre pre_global(int) const { return Pre{}; }
    __device__ __forceinline__ void terms(int p, int j, T s, double& du2, double& pv,
                                          double& cx) const {
        if (SCALED) s = mul_rn(dsc[j], s);
        const T cj = c[j], l = lv[j], u = uv[j];
        const T g = sub_rn(cj, s);
        const T r = proj_multiplier(g, l, u);
        const double d = (double)mul_rn(invD2[j], sub_rn(g, r));
        du2 = __dmul_rn(d, d);
        pv = (double)sub_rn(safeprod_left(u, pos_part(-r)), safeprod_left(l, neg_part(-r)));
        cx = (double)mul_rn(cj, pick(x, p)[j]);
    }
    __device__ __forceinline__ void row(int p, int j, T s, const Pre&, Acc& a) {
        double du2, pv, cx;
        terms(p, j, s, du2, pv, cx);
        a.v[3 * p] += du2;
        a.v[3 * p + 1] += pv;
        a.v[3 * p + 2] += cx;
    }
    __device__ void row_long(int p, int j, T s, int lid, Acc&) {
        double du2, pv, cx;
        terms(p, j, s, du2, pv, cx);
        double* o = long_out + (size_t)lid * 3 * NV + 3 * p;
        o[0] = du2;
        o[1] = pv;
        o[2] = cx;
    }
    __device__ void finish(Acc& a) { block_reduce_store<3 * NV, W>(a.v, block_out); }
};

// Infeasibility certificates (an extension; the reference has no detection).
// Row side, primal ray x: s = (A x)_i (SCALED: the product gathered D2 x and s
// is multiplied by d1_i); accumulates the squared distance of s to the
// recession cone of [lc_i, uc_i] and the dual ray y's row objective
// (lc_i y_i for y_i > 0, uc_i y_i for y_i < 0; y's signs are already those
// the bounds allow).
template <class T, bool SCALED = false>
struct RayRowEpi {
    const T* __restrict__ lc;
    const T* __restrict__ uc;
    const double* __restrict__ ry;
    const double* __restrict__ dsc;
    double* block_out;
    double* long_out;
    struct Acc { double v[2]; };
    struct Pre {};
    __device__ void init(Acc& a) { a.v[0] = a.v[1] = 0.0; }
    __device__ __forceinline__ Pre pre_global(int) const { return Pre{}; }
    __device__ __forceinline__ void terms(int i, double s, double& r2, double& ob) const {
        if (SCALED) s = __dmul_rn(dsc[i], s);
        const double l = (double)lc[i], u = (double)uc[i];
        const bool lo = !isinf(l), up = !isinf(u);
        const double res = (lo && up) ? s : lo ? fmin(s, 0.0) : up ? fmax(s, 0.0) : 0.0;
        r2 = __dmul_rn(res, res);
        const double y = ry[i];
        ob = y > 0.0 ? __dmul_rn(l, y) : (y < 0.0 ? __dmul_rn(u, y) : 0.0);
    }
    __device__ __forceinline__ void row(int, int i, double s, const Pre&, Acc& a) {
        double r2, ob;
        terms(i, s, r2, ob);
        a.v[0] += r2;
        a.v[1] += ob;
    }
    __device__ void row_long(int, int i, double s, int lid, Acc&) {
        double r2, ob;
        terms(i, s, r2, ob);
        long_out[(size_t)lid * 2] = r2;
        long_out[(size_t)lid * 2 + 1] = ob;
    }
    __device__ void finish(Acc& a) { block_reduce_store<2>(a.v, block_out); }
};

// Column side, dual ray y: g = -(A' y)_j (SCALED: gathered D1 y, times d2_j),
// r = the part of g the variable bounds allow (proj_multiplier); accumulates
// |g - r|^2, the ray objective of r (lv_j r for r > 0, uv_j r for r < 0) and
// c'x of the primal ray
template <class T, bool SCALED = false>
struct RayColEpi {
    const T* __restrict__ c;
    const T* __restrict__ lv;
    const T* __restrict__ uv;
    const double* __restrict__ rx;
    const double* __restrict__ dsc;
    double* block_out;
    double* long_out;
    struct Acc { double v[3]; };
    struct Pre {};
    __device__ void init(Acc& a) { a.v[0] = a.v[1] = a.v[2] = 0.0; }
    __device__ __forceinline__ Pre pre_global(int) const { return Pre{}; }
    __device__ __forceinline__ void terms(int j, double s, double& r2, double& ob,
                                          double& cx) const {
        if (SCALED) s = __dmul_rn(dsc[j], s);
        const double l = (double)lv[j], u = (double)uv[j];
        const double g = -s;
        const double r = proj_multiplier(g, l, u);
        const double res = __dsub_rn(g, r);
        r2 = __dmul_rn(res, res);
        ob = r > 0.0 ? __dmul_rn(l, r) : (r < 0.0 ? __dmul_rn(u, r) : 0.0);
        cx = __dmul_rn((double)c[j], rx[j]);
    }
    __device__ __forceinline__ void row(int, int j, double s, const Pre&, Acc& a) {
        double r2, ob, cx;
        terms(j, s, r2, ob, cx);
        a.v[0] += r2;
        a.v[1] += ob;
        a.v[2] += cx;
    }
    __device__ void row_long(int, int j, double s, int lid, Acc&) {
        double r2, ob, cx;
        terms(j, s, r2, ob, cx);
        double* o = long_out + (size_t)lid * 3;
        o[0] = r2;
        o[1] = ob;
        o[2] = cx;
    }
    __device__ void finish(Acc& a) { block_reduce_store<3>(a.v, block_out); }
};

// power method, second product: Ax_j = (A' s)_j; accumulates x.Ax and Ax.Ax
// (SCALED: the product gathered D1 s and Ax_j is the row sum times d2_j)
template <class T, bool SCALED = false>
struct PowerEpi {
    const T* __restrict__ x;
    T* __restrict__ out;
    double* block_out;
    double* long_out;
    const T* __restrict__ dsc = nullptr;
    struct Acc { double v[2]; };
    struct Pre { T x; };
    __device__ Pre pre_global(int j) const { return Pre{ld_stream(x + j)}; }
    __device__ void init(Acc& a) { a.v[0] = a.v[1] = 0.0; }
    __device__ __forceinline__ void row(int, int j, T s, const Pre& q, Acc& a) {
        if (SCALED) s = mul_rn(dsc[j], s);
        out[j] = s;
        a.v[0] += (double)q.x * (double)s;
        a.v[1] += (double)s * (double)s;
    }
    __device__ void row_long(int, int j, T s, int lid, Acc&) {
        if (SCALED) s = mul_rn(dsc[j], s);
        out[j] = s;
        long_out[(size_t)lid * 2] = (double)ld_stream(x + j) * (double)s;
        long_out[(size_t)lid * 2 + 1] = (double)s * (double)s;
    }
    __device__ void finish(Acc& a) { block_reduce_store<2>(a.v, block_out); }
};

}  // namespace cpdlp
