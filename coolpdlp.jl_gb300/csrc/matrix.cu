// matrix.cu -- the pluggable sparse matrix types (src/utils/mat_csr.jl,
// mat_ell.jl, mat_coo.jl): device builds, export and mul!.
#include <algorithm>
#include <cmath>
#include <memory>
#include <type_traits>

#include "matrix.cuh"

namespace cpdlp {

namespace {

template <class T>
struct MulEpi {  // c[i] = alpha*s + beta*c[i]; beta == 0 does not read c (mat_csr.jl:74)
    T* out;
    T alpha, beta;
    int use_beta;
    struct Acc {};
    struct Pre { T c; };
    __device__ Pre pre_global(int r) const { return Pre{use_beta ? out[r] : T(0)}; }
    __device__ void init(Acc&) {}
    __device__ __forceinline__ void row(int, int r, T s, const Pre& q, Acc&) {
        T v = mul_rn(alpha, s);
        if (use_beta) v = add_rn(v, mul_rn(beta, q.c));
        out[r] = v;
    }
    __device__ void row_long(int p, int r, T s, int, Acc& a) { row(p, r, s, pre_global(r), a); }
    __device__ void finish(Acc&) {}
};

// spmv_ell! (mat_ell.jl:72-89): one thread per row, column-major slabs,
// 1-based column indices with 0 as padding.
template <class T>
__global__ void k_spmv_ell(const int32_t* __restrict__ col1, const T* __restrict__ val, int64_t m,
                           int64_t d, const T* __restrict__ b, T* __restrict__ c, T alpha, T beta,
                           int use_beta) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    T s = T(0);
    for (int64_t k = 0; k < d; k++) {
        const int32_t j = col1[i + k * m];
        if (j != 0) s = add_rn(s, mul_rn(val[i + k * m], b[j - 1]));
    }
    T v = mul_rn(alpha, s);
    if (use_beta) v = add_rn(v, mul_rn(beta, c[i]));
    c[i] = v;
}

// mul! for COO (mat_coo.jl:68-80): c .*= beta, then atomic c[i] += alpha*v*b[j]
template <class T>
__global__ void k_scale_or_zero(T* __restrict__ c, int64_t m, T beta, int use_beta) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) c[i] = use_beta ? mul_rn(c[i], beta) : T(0);
}
template <class T>
__global__ void k_spmv_coo(const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                           const T* __restrict__ val, int64_t nnz, const T* __restrict__ b,
                           T* __restrict__ c, T alpha) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) atomicAdd(c + row[k], mul_rn(mul_rn(alpha, val[k]), b[col[k]]));
}

// GPUSparseMatrixELL(A) (mat_ell.jl:54-70) from the device CSR
template <class T>
__global__ void k_build_ell(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const T* __restrict__ v, int64_t m, int64_t d,
                            int32_t* __restrict__ ecol, T* __restrict__ eval) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int a = ptr[i], b = ptr[i + 1];
    for (int64_t k = 0; k < d; k++) {
        const int64_t e = a + k;
        const bool in = e < b;
        ecol[i + k * m] = in ? idx[e] + 1 : 0;
        eval[i + k * m] = in ? v[e] : T(0);
    }
}

__global__ void k_to_i64_plus(const int32_t* __restrict__ in, int64_t* __restrict__ out, int64_t len,
                              int64_t add) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = (int64_t)in[i] + add;
}
template <class T>
__global__ void k_to_f64(const T* __restrict__ in, double* __restrict__ out, int64_t len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len) out[i] = (double)in[i];
}
// narrow +-1 CSR (CPDLP_VAL_PM1): the stored index is col for +1, ~col for -1
__global__ void k_pm1_encode(int32_t* __restrict__ idx, const double* __restrict__ v, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz && v[k] < 0.0) idx[k] = ~idx[k];
}
__global__ void k_pm1_decode(const int32_t* __restrict__ idx, int64_t* __restrict__ col1,
                             double* __restrict__ val, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    const int32_t c = idx[k];
    if (col1) col1[k] = (int64_t)pm1_col(c) + 1;
    if (val) val[k] = c < 0 ? -1.0 : 1.0;
}

template <class T>
DBuf<T>& vals_of(Matrix& M);
template <>
DBuf<double>& vals_of<double>(Matrix& M) { return M.vd; }
template <>
DBuf<float>& vals_of<float>(Matrix& M) { return M.vf; }

template <class T>
void build_T(Handle& h, Matrix& M, CscPair& S) {
    cudaStream_t s = h.stream;
    const int64_t m = M.m, nnz = M.nnz;
    const size_t zn = (size_t)(nnz > 0 ? nnz : 1);
    if (M.format == CPDLP_FMT_COO) {
        M.ptr = std::move(S.idx1);   // rowval (0-based), findnz order
        M.idx = std::move(S.col1);   // colval (0-based)
        vals_of<T>(M).alloc(zn);
        if (nnz > 0) {
            if (std::is_same<T, double>::value)
                CK(cudaMemcpyAsync(vals_of<T>(M).p, S.val1.p, sizeof(double) * nnz,
                                   cudaMemcpyDeviceToDevice, s));
            else {
                DBuf<int32_t> iota(zn);
                std::vector<int32_t> hi((size_t)nnz);
                for (int64_t k = 0; k < nnz; k++) hi[(size_t)k] = (int32_t)k;
                CK(cudaMemcpyAsync(iota.p, hi.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s));
                gather_values<T, double>(S.val1.p, iota.p, vals_of<T>(M).p, nnz, s);
                CK(cudaStreamSynchronize(s));
            }
        }
        CK(cudaStreamSynchronize(s));
        return;
    }
    // CSR of A: S2 structure with A's values permuted into it (padded for the
    // aligned 128-bit tile loads)
    DBuf<T> v2(zn + PAD_ELEMS);
    CK(cudaMemsetAsync(v2.p, 0, sizeof(T) * (zn + PAD_ELEMS), s));
    gather_values<T, double>(S.val1.p, S.p21.p, v2.p, nnz, s);
    std::vector<int32_t> hp((size_t)m + 1);
    CK(cudaMemcpyAsync(hp.data(), S.ptr2.p, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (M.format == CPDLP_FMT_CSR) {
        M.ptr = std::move(S.ptr2);
        M.idx = std::move(S.idx2);
        vals_of<T>(M) = std::move(v2);
        build_tile_plan(hp, (int32_t)m, choose_items(nnz, m, 0), M.plan, s);
        M.part.alloc((size_t)(M.plan.npieces > 0 ? M.plan.npieces : 1) * sizeof(double));
        return;
    }
    // ELL: width d = maximum(diff(rowptr)) (mat_ell.jl:57)
    int64_t d = 0;
    for (int64_t i = 0; i < m; i++) d = std::max<int64_t>(d, hp[(size_t)i + 1] - hp[(size_t)i]);
    M.width = d;
    const double bytes = (double)m * (double)d * (double)(sizeof(int32_t) + sizeof(T));
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > 0.9 * (double)free_b) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "ELL storage needs %.3g GB (m=%lld x width d=%lld) but %.3g GB are free", bytes / 1e9,
                 (long long)m, (long long)d, (double)free_b / 1e9);
        fail(CPDLP_ERR_OUT_OF_MEMORY, buf);
    }
    const size_t md = (size_t)(m * d > 0 ? m * d : 1);
    M.idx.alloc(md);
    vals_of<T>(M).alloc(md);
    if (m > 0) {
        k_build_ell<T><<<grid_for(m, 256), 256, 0, s>>>(S.ptr2.p, S.idx2.p, v2.p, m, d, M.idx.p,
                                                        vals_of<T>(M).p);
        CK_LAUNCH();
    }
    CK(cudaStreamSynchronize(s));
}

template <class T>
void spmv_T(Handle& h, const Matrix& M, const T* b, T* c, double alpha, double beta) {
    cudaStream_t s = h.stream;
    const T a = (T)alpha, bb = (T)beta;
    const int ub = beta != 0.0;
    const DBuf<T>& vals = vals_of<T>(const_cast<Matrix&>(M));
    if (M.format == CPDLP_FMT_CSR) {
        CsrView<T, T> v{M.ptr.p, M.idx.p, vals.p, M.plan.tasks.p, M.plan.ntasks,
                        M.plan.ltasks.p, M.plan.nltasks, M.plan.counters.p,
                        reinterpret_cast<T*>(M.part.p)};
        MulEpi<T> e{c, a, bb, ub};
        launch_tiles<1>(M.plan, v, VecSet<T, 1>{{b}}, e, s);
    } else if (M.format == CPDLP_FMT_ELL) {
        if (M.m > 0)
            k_spmv_ell<T><<<grid_for(M.m, 256), 256, 0, s>>>(M.idx.p, vals.p, M.m, M.width, b, c, a,
                                                             bb, ub);
        CK_LAUNCH();
    } else {
        if (M.m > 0) k_scale_or_zero<T><<<grid_for(M.m, 256), 256, 0, s>>>(c, M.m, bb, ub);
        if (M.nnz > 0)
            k_spmv_coo<T><<<grid_for(M.nnz, 256), 256, 0, s>>>(M.ptr.p, M.idx.p, vals.p, M.nnz, b, c, a);
        CK_LAUNCH();
    }
}

template <class T>
void export_T(Handle& h, const Matrix& M, int64_t* ptr, int64_t* idx, double* val) {
    cudaStream_t s = h.stream;
    const DBuf<T>& vals = vals_of<T>(const_cast<Matrix&>(M));
    auto copy_idx = [&](const int32_t* src, int64_t len, int64_t add, int64_t* dst) {
        if (!dst || len <= 0) return;
        DBuf<int64_t> t((size_t)len);
        k_to_i64_plus<<<grid_for(len, 256), 256, 0, s>>>(src, t.p, len, add);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(dst, t.p, sizeof(int64_t) * len, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    };
    auto copy_val = [&](int64_t len) {
        if (!val || len <= 0) return;
        DBuf<double> t((size_t)len);
        k_to_f64<T><<<grid_for(len, 256), 256, 0, s>>>(vals.p, t.p, len);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(val, t.p, sizeof(double) * len, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    };
    if (M.format == CPDLP_FMT_CSR) {
        copy_idx(M.ptr.p, M.m + 1, 1, ptr);
        copy_idx(M.idx.p, M.nnz, 1, idx);
        copy_val(M.nnz);
    } else if (M.format == CPDLP_FMT_ELL) {
        copy_idx(M.idx.p, M.m * M.width, 0, idx);
        copy_val(M.m * M.width);
    } else {
        copy_idx(M.ptr.p, M.nnz, 1, ptr);
        copy_idx(M.idx.p, M.nnz, 1, idx);
        copy_val(M.nnz);
    }
}

// CPDLP_VAL_PM1: CSR of A with the signs in the column indices, no values
void build_pm1(Handle& h, Matrix& M, CscPair& S) {
    cudaStream_t s = h.stream;
    const int64_t m = M.m, nnz = M.nnz;
    DBuf<double> v2((size_t)(nnz > 0 ? nnz : 1));
    gather_values<double, double>(S.val1.p, S.p21.p, v2.p, nnz, s);
    if (nnz > 0) {
        k_pm1_encode<<<grid_for(nnz, 256), 256, 0, s>>>(S.idx2.p, v2.p, nnz);
        CK_LAUNCH();
    }
    std::vector<int32_t> hp((size_t)m + 1);
    CK(cudaMemcpyAsync(hp.data(), S.ptr2.p, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    M.ptr = std::move(S.ptr2);
    M.idx = std::move(S.idx2);
    build_tile_plan(hp, (int32_t)m, choose_items(nnz, m, 0), M.plan, s);
    M.part.alloc((size_t)(M.plan.npieces > 0 ? M.plan.npieces : 1) * sizeof(double));
}

void spmv_pm1(Handle& h, const Matrix& M, const float* b, float* c, double alpha, double beta) {
    CsrView<Pm1, float> v{M.ptr.p, M.idx.p, nullptr, M.plan.tasks.p, M.plan.ntasks,
                          M.plan.ltasks.p, M.plan.nltasks, M.plan.counters.p,
                          reinterpret_cast<float*>(M.part.p)};
    MulEpi<float> e{c, (float)alpha, (float)beta, beta != 0.0};
    launch_tiles<1>(M.plan, v, VecSet<float, 1>{{b}}, e, h.stream);
}

void export_pm1(Handle& h, const Matrix& M, int64_t* ptr, int64_t* idx, double* val) {
    cudaStream_t s = h.stream;
    if (ptr && M.m + 1 > 0) {
        DBuf<int64_t> t((size_t)(M.m + 1));
        k_to_i64_plus<<<grid_for(M.m + 1, 256), 256, 0, s>>>(M.ptr.p, t.p, M.m + 1, 1);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(ptr, t.p, sizeof(int64_t) * (M.m + 1), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    if ((idx || val) && M.nnz > 0) {
        DBuf<int64_t> ti((size_t)M.nnz);
        DBuf<double> tv((size_t)M.nnz);
        k_pm1_decode<<<grid_for(M.nnz, 256), 256, 0, s>>>(M.idx.p, idx ? ti.p : nullptr,
                                                          val ? tv.p : nullptr, M.nnz);
        CK_LAUNCH();
        if (idx) CK(cudaMemcpyAsync(idx, ti.p, sizeof(int64_t) * M.nnz, cudaMemcpyDeviceToHost, s));
        if (val) CK(cudaMemcpyAsync(val, tv.p, sizeof(double) * M.nnz, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
}

}  // namespace

Matrix* matrix_from_csc(Handle& h, int64_t m, int64_t n, int64_t nnz, const int64_t* colptr,
                        const int64_t* rowval, const double* nzval, int32_t format, int32_t vt) {
    if (format != CPDLP_FMT_CSR && format != CPDLP_FMT_ELL && format != CPDLP_FMT_COO)
        fail(CPDLP_ERR_ARGUMENT, "unknown matrix format");
    if (vt != CPDLP_VAL_F64 && vt != CPDLP_VAL_F32 && vt != CPDLP_VAL_PM1)
        fail(CPDLP_ERR_ARGUMENT, "matrix value type must be CPDLP_VAL_F64, F32 or PM1");
    if (vt == CPDLP_VAL_PM1) {
        if (format != CPDLP_FMT_CSR)
            fail(CPDLP_ERR_UNSUPPORTED, "CPDLP_VAL_PM1 storage is CSR only");
        if (nnz > 0 && !nzval) fail(CPDLP_ERR_ARGUMENT, "null nzval");
        for (int64_t k = 0; k < nnz; k++)
            if (std::fabs(nzval[k]) != 1.0)
                fail(CPDLP_ERR_ARGUMENT, "CPDLP_VAL_PM1 needs every value to be exactly +1 or -1");
    }
    auto M = std::make_unique<Matrix>();
    M->h = &h;
    M->format = format;
    M->vt = vt;
    M->m = m; M->n = n; M->nnz = nnz;
    CscPair S;
    build_csc_pair(h, m, n, nnz, colptr, rowval, nzval, S);
    if (vt == CPDLP_VAL_F64) build_T<double>(h, *M, S);
    else if (vt == CPDLP_VAL_PM1) build_pm1(h, *M, S);
    else build_T<float>(h, *M, S);
    return M.release();
}

void matrix_spmv(Handle& h, const Matrix& M, const void* b, void* c, double alpha, double beta) {
    if ((!b && M.n > 0) || (!c && M.m > 0)) fail(CPDLP_ERR_ARGUMENT, "null vector pointer");
    if (M.vt == CPDLP_VAL_F64)
        spmv_T<double>(h, M, static_cast<const double*>(b), static_cast<double*>(c), alpha, beta);
    else if (M.vt == CPDLP_VAL_PM1)
        spmv_pm1(h, M, static_cast<const float*>(b), static_cast<float*>(c), alpha, beta);
    else
        spmv_T<float>(h, M, static_cast<const float*>(b), static_cast<float*>(c), alpha, beta);
}

void matrix_export(Handle& h, const Matrix& M, int64_t* ptr, int64_t* idx, double* val) {
    if (M.vt == CPDLP_VAL_F64) export_T<double>(h, M, ptr, idx, val);
    else if (M.vt == CPDLP_VAL_PM1) export_pm1(h, M, ptr, idx, val);
    else export_T<float>(h, M, ptr, idx, val);
}

}  // namespace cpdlp
