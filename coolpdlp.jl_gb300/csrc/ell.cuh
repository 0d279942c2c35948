// ell.cuh -- the ELL product engine of the solver (GPUSparseMatrixELL,
// src/utils/mat_ell.jl:72-89): one thread per row over column-major slabs,
// with the same fused per-row epilogues as the CSR tile engine.
//
// Layout: idx / val are rows x width, column-major (entry k of row r at
// r + k*rows), rows left-aligned in CSR order; the row pointer gives each
// row's length, so the padding is never read.  Consecutive threads read
// consecutive addresses of a slab (coalesced).  A row's sum runs in its
// column order, sequentially, like the reference's spmv_ell! loop, so every
// row reproduces a sequential CPU sum exactly (in the CSR tile engine only
// rows of at most LONG_ROW nonzeros do).  Narrow +-1 storage carries the sign
// in the index (~col for -1) and has no value slab.
#pragma once

#include "tiles.cuh"

namespace cpdlp {

template <class V, class T>
struct EllView {
    const int32_t* __restrict__ ptr;  // CSR row pointer (0-based, rows + 1)
    const int32_t* __restrict__ idx;  // rows x width, column-major, 0-based
    const V* __restrict__ val;        // rows x width, column-major (null for Pm1)
    int64_t rows;
};

// one row: sum_k val[k] * x[idx[k]] in k order, four entries' loads and
// gathers issued together
template <class V, class T>
__device__ __forceinline__ T ell_row(const EllView<V, T>& A, int64_t r, int len,
                                     const T* __restrict__ xv) {
    T sum = T(0);
    int k = 0;
    for (; k + 4 <= len; k += 4) {
        int c[4];
        T v[4], g[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            c[u] = __ldcs(A.idx + r + (int64_t)(k + u) * A.rows);
            if constexpr (!is_pm1<V>::value) v[u] = load1v<V, T>(A.val + r + (int64_t)(k + u) * A.rows);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) g[u] = gather<false>(xv + (is_pm1<V>::value ? pm1_col(c[u]) : c[u]));
#pragma unroll
        for (int u = 0; u < 4; u++)
            sum = add_rn(sum, is_pm1<V>::value ? pm1_apply(c[u], g[u]) : mul_rn(v[u], g[u]));
    }
    for (; k < len; k++) {
        const int c = __ldcs(A.idx + r + (int64_t)k * A.rows);
        const T g = gather<false>(xv + (is_pm1<V>::value ? pm1_col(c) : c));
        if constexpr (is_pm1<V>::value) sum = add_rn(sum, pm1_apply(c, g));
        else sum = add_rn(sum, mul_rn(load1v<V, T>(A.val + r + (int64_t)k * A.rows), g));
    }
    return sum;
}

template <int WARPS, int NVEC, class V, class T, class Epi>
__global__ void __launch_bounds__(WARPS * 32)
    k_ell(EllView<V, T> A, VecSet<T, NVEC> xs, Epi epi) {
    const int64_t r = (int64_t)blockIdx.x * (WARPS * 32) + threadIdx.x;
    typename Epi::Acc acc;
    epi.init(acc);
    if (r < A.rows) {
        const int a = ld_keep(A.ptr + r);
        const int len = ld_keep(A.ptr + r + 1) - a;
        const typename Epi::Pre pre = epi.pre_global((int)r);
#pragma unroll 1
        for (int p = 0; p < NVEC; p++) epi.row(p, (int)r, ell_row(A, r, len, pick(xs.v, p)), pre, acc);
    }
    epi.finish(acc);
}

// four packed iterates (x4[4*col + p], see short_tile4): one 16-byte gather
// (two for FP64) per entry, four sums side by side, each in column order
template <int WARPS, class V, class T, class Epi>
__global__ void __launch_bounds__(WARPS * 32)
    k_ell4(EllView<V, T> A, const T* __restrict__ x4, Epi epi) {
    typename Epi::Acc acc;
    epi.init(acc);
    // a capped grid (ell4_grid) strides over the rows
    for (int64_t r = (int64_t)blockIdx.x * (WARPS * 32) + threadIdx.x; r < A.rows;
         r += (int64_t)gridDim.x * (WARPS * 32)) {
        const int a = ld_keep(A.ptr + r);
        const int len = ld_keep(A.ptr + r + 1) - a;
        T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
        int k = 0;
        for (; k + 2 <= len; k += 2) {
            int c[2];
            T v[2], g[2][4];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                c[u] = __ldcs(A.idx + r + (int64_t)(k + u) * A.rows);
                if constexpr (!is_pm1<V>::value) v[u] = load1v<V, T>(A.val + r + (int64_t)(k + u) * A.rows);
            }
#pragma unroll
            for (int u = 0; u < 2; u++)
                gather4(x4 + 4 * (size_t)(is_pm1<V>::value ? pm1_col(c[u]) : c[u]), g[u]);
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if constexpr (is_pm1<V>::value) {
                    s0 = add_rn(s0, pm1_apply(c[u], g[u][0]));
                    s1 = add_rn(s1, pm1_apply(c[u], g[u][1]));
                    s2 = add_rn(s2, pm1_apply(c[u], g[u][2]));
                    s3 = add_rn(s3, pm1_apply(c[u], g[u][3]));
                } else {
                    s0 = add_rn(s0, mul_rn(v[u], g[u][0]));
                    s1 = add_rn(s1, mul_rn(v[u], g[u][1]));
                    s2 = add_rn(s2, mul_rn(v[u], g[u][2]));
                    s3 = add_rn(s3, mul_rn(v[u], g[u][3]));
                }
            }
        }
        for (; k < len; k++) {
            const int c = __ldcs(A.idx + r + (int64_t)k * A.rows);
            T g[4];
            gather4(x4 + 4 * (size_t)(is_pm1<V>::value ? pm1_col(c) : c), g);
            if constexpr (is_pm1<V>::value) {
                s0 = add_rn(s0, pm1_apply(c, g[0]));
                s1 = add_rn(s1, pm1_apply(c, g[1]));
                s2 = add_rn(s2, pm1_apply(c, g[2]));
                s3 = add_rn(s3, pm1_apply(c, g[3]));
            } else {
                const T v = load1v<V, T>(A.val + r + (int64_t)k * A.rows);
                s0 = add_rn(s0, mul_rn(v, g[0]));
                s1 = add_rn(s1, mul_rn(v, g[1]));
                s2 = add_rn(s2, mul_rn(v, g[2]));
                s3 = add_rn(s3, mul_rn(v, g[3]));
            }
        }
        const typename Epi::Pre pre{};
        epi.row(0, (int)r, s0, pre, acc);
        epi.row(1, (int)r, s1, pre, acc);
        epi.row(2, (int)r, s2, pre, acc);
        epi.row(3, (int)r, s3, pre, acc);
    }
    epi.finish(acc);
}

// blocks (= block-partial rows of a reducing epilogue) of an ELL launch
inline unsigned ell_grid(int64_t rows, int warps) {
    const int64_t g = (rows + warps * 32 - 1) / (warps * 32);
    return (unsigned)(g > 0 ? g : 1);
}
// the same for the four-iterate pass, at most max_blocks (0: no cap)
inline unsigned ell4_grid(int64_t rows, int warps, int64_t max_blocks) {
    const unsigned g = ell_grid(rows, warps);
    return (max_blocks > 0 && g > max_blocks) ? (unsigned)max_blocks : g;
}

template <int WARPS, int NVEC, class V, class T, class Epi>
void launch_ell(const EllView<V, T>& A, const VecSet<T, NVEC>& xs, const Epi& epi, cudaStream_t s) {
    if (A.rows == 0 || tiles_dry_run()) return;
    k_ell<WARPS, NVEC, V, T, Epi><<<ell_grid(A.rows, WARPS), WARPS * 32, 0, s>>>(A, xs, epi);
    CK_LAUNCH();
}
template <int WARPS, class V, class T, class Epi>
void launch_ell4(const EllView<V, T>& A, const T* x4, const Epi& epi, int64_t max_blocks,
                 cudaStream_t s) {
    if (A.rows == 0 || tiles_dry_run()) return;
    k_ell4<WARPS, V, T, Epi><<<ell4_grid(A.rows, WARPS, max_blocks), WARPS * 32, 0, s>>>(A, x4, epi);
    CK_LAUNCH();
}

}  // namespace cpdlp
