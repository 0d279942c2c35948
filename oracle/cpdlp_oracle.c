/*
 * cpdlp_oracle.c -- CPU ORACLE (test infrastructure only).
 *
 * A plain-C, Float64 restatement of CoolPDLP.jl's solve path, used by the test
 * suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker for libcoolpdlp_cuda.  It is never linked into, loaded by or called
 * from the product.  Each function cites the reference file:line it follows
 * (paths relative to the CoolPDLP.jl source tree).
 *
 * Parity status.  The reference is Julia and cannot run in this build's
 * environment (no julia), and it ships no golden vectors.  This restatement
 * is pinned against the known answers its test suite holds (projections,
 * `combine`, the KKT closed forms and their invariance under
 * preconditioning, the Ruiz fixed point, the 2-variable LP with objective
 * 205, the "termination check not skipped" LP, SpMV = alpha*A*b + beta*c for
 * the three formats) and against scipy's HiGHS objective.  The trajectory
 * is NOT pinned bit-for-bit to Julia: the power-method start vector comes
 * from StableRNG(0) + Julia's ziggurat randn! in the reference and from a
 * SplitMix64 + Box-Muller stream here, and Julia's BLAS-backed reductions
 * (norm/dot/sum for length >= 32) use a summation order this code does not
 * reproduce.  Everything else (SpMV order, scaling order, projections,
 * restart logic) follows the reference operation by operation.
 *
 * Third-party arithmetic restated here:
 *  - SparseArrays (Julia stdlib >= 1.10): CSC mul! and sparse(transpose(A)).
 *  - IterativeSolvers 0.9.4 powm!: Rayleigh-quotient power method with
 *    tol = eps(T) * size(B,2)^3 (Int64 power, which wraps on overflow exactly
 *    as Julia's Int does) and maxiter = size(B,1); the start vector is NOT
 *    normalised (CoolPDLP passes randn! output directly, linalg.jl:91-94).
 *
 * Build: see oracle/build_oracle.sh (gcc -O2 -ffp-contract=off, so that no
 * multiply-add is fused: Julia does not contract a*b+c either).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../include/coolpdlp_cuda.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* scalar helpers: src/utils/linalg.jl:1-53                                  */
/* ------------------------------------------------------------------------ */

/* Base.max / Base.min on floats: NaN propagates and -0.0 < +0.0. */
static inline double jl_max(double x, double y) {
    int sx = signbit(x) != 0, sy = signbit(y) != 0;
    if ((y > x) || (sy < sx)) return isnan(x) ? x : y;
    return isnan(y) ? y : x;
}
static inline double jl_min(double x, double y) {
    int sx = signbit(x) != 0, sy = signbit(y) != 0;
    if ((y < x) || (sy > sx)) return isnan(x) ? x : y;
    return isnan(y) ? y : x;
}
/* positive_part / negative_part (linalg.jl:4-5) */
static inline double pos_part(double a) { return jl_max(a, 0.0); }
static inline double neg_part(double a) { return -jl_min(a, 0.0); }
/* safeprod_left (linalg.jl:17): returns r, not 0, when l is infinite */
static inline double safeprod_left(double l, double r) { return isinf(l) ? r : l * r; }
/* proj_box (linalg.jl:19) */
static inline double proj_box(double x, double l, double u) { return jl_min(u, jl_max(l, x)); }
/* proj_multiplier (linalg.jl:26-42) */
static inline double proj_multiplier(double lam, double l, double u) {
    int lmin = (l == -INFINITY), umax = (u == INFINITY);
    if (lmin) return umax ? 0.0 : -neg_part(lam);
    return umax ? pos_part(lam) : lam;
}
/* combine (linalg.jl:49-53) */
static inline double combine(double l, double u) {
    double ls = isfinite(l) ? fabs(l) : 0.0;
    double us = isfinite(u) ? fabs(u) : 0.0;
    return jl_max(jl_max(0.0, ls), us);
}

ORC_EXPORT double orc_proj_box(double x, double l, double u) { return proj_box(x, l, u); }
ORC_EXPORT double orc_proj_multiplier(double x, double l, double u) { return proj_multiplier(x, l, u); }
ORC_EXPORT double orc_combine(double l, double u) { return combine(l, u); }
ORC_EXPORT double orc_safeprod_left(double l, double r) { return safeprod_left(l, r); }
ORC_EXPORT double orc_positive_part(double a) { return pos_part(a); }
ORC_EXPORT double orc_negative_part(double a) { return neg_part(a); }

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------ */
/* Gaussian stream: SplitMix64 (Steele, Lea & Flood, 2014) + Box-Muller.      */
/* Element i uses counters 2i and 2i+1 of the stream, so it can be produced   */
/* independently.  Stands in for randn!(StableRNG(0), x0) (linalg.jl:92).     */
/* ------------------------------------------------------------------------ */
static inline uint64_t splitmix64_at(uint64_t seed, uint64_t counter) {
    uint64_t z = seed + (counter + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline double unit_open0(uint64_t bits) { /* (0, 1] */
    return (double)((bits >> 11) + 1) * (1.0 / 9007199254740992.0);
}
ORC_EXPORT void orc_gaussian_vector(uint64_t seed, int64_t len, double* out) {
    for (int64_t i = 0; i < len; i++) {
        double u1 = unit_open0(splitmix64_at(seed, 2 * (uint64_t)i));
        double u2 = unit_open0(splitmix64_at(seed, 2 * (uint64_t)i + 1));
        out[i] = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
}

/* ------------------------------------------------------------------------ */
/* Sparse formats: src/utils/mat_csr.jl, mat_ell.jl, mat_coo.jl              */
/* All index arrays in this section are 0-based; the Python wrapper adds 1.  */
/* ------------------------------------------------------------------------ */

/* sparse(transpose(A)) of an m x n CSC (SparseArrays halfperm!): a counting
 * sort that keeps the column order inside each output column.  With CSC
 * input this yields the CSR arrays of GPUSparseMatrixCSR (mat_csr.jl:58-61):
 * rowptr (m+1), colval ascending inside each row.  perm[k_out] = k_in. */
ORC_EXPORT void orc_csc_transpose(int64_t m, int64_t n, const int64_t* colptr,
                                  const int64_t* rowval, const double* nzval,
                                  int64_t* tptr, int64_t* tidx, double* tval, int64_t* perm) {
    int64_t nnz = colptr[n];
    for (int64_t i = 0; i <= m; i++) tptr[i] = 0;
    for (int64_t k = 0; k < nnz; k++) tptr[rowval[k] + 1]++;
    for (int64_t i = 0; i < m; i++) tptr[i + 1] += tptr[i];
    int64_t* cursor = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    for (int64_t i = 0; i < m; i++) cursor[i] = tptr[i];
    for (int64_t j = 0; j < n; j++) {
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) {
            int64_t p = cursor[rowval[k]]++;
            tidx[p] = j;
            if (tval) tval[p] = nzval[k];
            if (perm) perm[p] = k;
        }
    }
    free(cursor);
}

/* ELL width d = maximum(diff(rowptr)) (mat_ell.jl:57); 0 for m == 0. */
ORC_EXPORT int64_t orc_ell_width(int64_t m, const int64_t* rowptr) {
    int64_t d = 0;
    for (int64_t i = 0; i < m; i++) {
        int64_t len = rowptr[i + 1] - rowptr[i];
        if (len > d) d = len;
    }
    return d;
}

/* GPUSparseMatrixELL(A) (mat_ell.jl:54-70): m x d column-major colval (1-based,
 * 0 = padding) and nzval (0 padding), from the CSR arrays. */
ORC_EXPORT void orc_ell_from_csr(int64_t m, int64_t d, const int64_t* rowptr,
                                 const int64_t* colval, const double* nzval,
                                 int64_t* ell_col1, double* ell_val) {
    for (int64_t t = 0; t < m * d; t++) { ell_col1[t] = 0; ell_val[t] = 0.0; }
    for (int64_t i = 0; i < m; i++) {
        int64_t k1 = rowptr[i], k2 = rowptr[i + 1];
        for (int64_t k = k1; k < k2; k++) {
            ell_col1[i + (k - k1) * m] = colval[k] + 1;
            ell_val[i + (k - k1) * m] = nzval[k];
        }
    }
}

/* GPUSparseMatrixCOO(A) = findnz(A) (mat_coo.jl:50-53): column-major order. */
ORC_EXPORT void orc_coo_from_csc(int64_t n, const int64_t* colptr, const int64_t* rowval,
                                 const double* nzval, int64_t* coo_row, int64_t* coo_col,
                                 double* coo_val) {
    for (int64_t j = 0; j < n; j++) {
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) {
            coo_row[k] = rowval[k];
            coo_col[k] = j;
            coo_val[k] = nzval[k];
        }
    }
}

/* SparseArrays mul!(C, A::SparseMatrixCSC, B, alpha, beta): C is filled (beta
 * == 0) or scaled, then each column scatters nzval*(B[j]*alpha). */
ORC_EXPORT void orc_spmv_csc(int64_t m, int64_t n, const int64_t* colptr, const int64_t* rowval,
                             const double* nzval, const double* b, double* c, double alpha,
                             double beta) {
    if (beta == 0.0) {
        for (int64_t i = 0; i < m; i++) c[i] = 0.0;
    } else if (beta != 1.0) {
        for (int64_t i = 0; i < m; i++) c[i] *= beta;
    }
    for (int64_t j = 0; j < n; j++) {
        double axj = b[j] * alpha;
        for (int64_t k = colptr[j]; k < colptr[j + 1]; k++) c[rowval[k]] += nzval[k] * axj;
    }
}

/* spmv_csr! (mat_csr.jl:63-79): c[i] = alpha*s + beta*c[i]; beta == 0 is a
 * strong zero (beta = false in the reference), so c is not read. */
ORC_EXPORT void orc_spmv_csr(int64_t m, const int64_t* rowptr, const int64_t* colval,
                             const double* nzval, const double* b, double* c, double alpha,
                             double beta) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (m > 4096)
#endif
    for (int64_t i = 0; i < m; i++) {
        double s = 0.0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) s += nzval[k] * b[colval[k]];
        c[i] = (beta == 0.0) ? alpha * s : alpha * s + beta * c[i];
    }
}

/* spmv_ell! (mat_ell.jl:72-89): skips the 0 padding sentinel (1-based colval). */
ORC_EXPORT void orc_spmv_ell(int64_t m, int64_t d, const int64_t* ell_col1, const double* ell_val,
                             const double* b, double* c, double alpha, double beta) {
    for (int64_t i = 0; i < m; i++) {
        double s = 0.0;
        for (int64_t k = 0; k < d; k++) {
            int64_t j = ell_col1[i + k * m];
            if (j != 0) s += ell_val[i + k * m] * b[j - 1];
        }
        c[i] = (beta == 0.0) ? alpha * s : alpha * s + beta * c[i];
    }
}

/* spmv_coo! + mul! (mat_coo.jl:55-80): c .*= beta, then c[i] += alpha*v*b[j]
 * per stored entry (the reference uses atomics; here the order is k). */
ORC_EXPORT void orc_spmv_coo(int64_t m, int64_t nnz, const int64_t* row, const int64_t* col,
                             const double* val, const double* b, double* c, double alpha,
                             double beta) {
    for (int64_t i = 0; i < m; i++) c[i] = (beta == 0.0) ? 0.0 : c[i] * beta;
    for (int64_t k = 0; k < nnz; k++) c[row[k]] += alpha * val[k] * b[col[k]];
}

/* ------------------------------------------------------------------------ */
/* MILP in the oracle (src/problems/milp.jl:20-115)                          */
/*                                                                            */
/* The reference keeps A (m x n) and At (n x m) as two CSC matrices whose    */
/* values are scaled separately (and so can differ in the last bit).  Here:   */
/*   S1 = CSC(A)  = CSR(At): ptr1 (n+1), idx1 (row of A)                      */
/*   S2 = CSC(At) = CSR(A) : ptr2 (m+1), idx2 (column of A)                   */
/*   vA  : A's values in S1 order,  vAt : At's values in S2 order             */
/*   p21[k2] = position in S1 of the same (i, j) as S2 position k2.           */
/* A*x is a gather over S2 rows with vA (identical, operation by operation,   */
/* to the reference's CSC scatter: both add a_ij*x_j into row i in ascending  */
/* j starting from 0.0), At*y a gather over S1 rows with vAt.                 */
/* ------------------------------------------------------------------------ */
typedef struct orc_milp {
    int64_t m, n, nnz;
    int64_t *ptr1, *idx1, *ptr2, *idx2, *p21, *p12;
    double *vA, *vAt;          /* CSC layouts (preconditioning)  */
    double *gA, *gAt;          /* gather layouts (solve)         */
    double *c, *lv, *uv, *lc, *uc, *D1, *D2;
} orc_milp;

static void milp_free(orc_milp* P) {
    free(P->ptr1); free(P->idx1); free(P->ptr2); free(P->idx2); free(P->p21); free(P->p12);
    free(P->vA); free(P->vAt); free(P->gA); free(P->gAt);
    free(P->c); free(P->lv); free(P->uv); free(P->lc); free(P->uc); free(P->D1); free(P->D2);
    memset(P, 0, sizeof(*P));
}

static double* dup_vec(const double* v, int64_t len) {
    double* o = (double*)malloc(sizeof(double) * (size_t)(len > 0 ? len : 1));
    if (v) memcpy(o, v, sizeof(double) * (size_t)len);
    return o;
}

/* MILP(; c, lv, uv, A, lc, uc) with At = convert(typeof(A), transpose(A))
 * (milp.jl:60) and D1, D2 = I (milp.jl:63-64). Input is 1-based CSC. */
static int milp_from_lp(const cpdlp_lp* lp, orc_milp* P) {
    memset(P, 0, sizeof(*P));
    int64_t m = lp->m, n = lp->n, nnz = lp->nnz;
    P->m = m; P->n = n; P->nnz = nnz;
    size_t zn = (size_t)(nnz > 0 ? nnz : 1);
    P->ptr1 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    P->idx1 = (int64_t*)malloc(sizeof(int64_t) * zn);
    P->ptr2 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
    P->idx2 = (int64_t*)malloc(sizeof(int64_t) * zn);
    P->p21 = (int64_t*)malloc(sizeof(int64_t) * zn);
    P->p12 = (int64_t*)malloc(sizeof(int64_t) * zn);
    P->vA = (double*)malloc(sizeof(double) * zn);
    P->vAt = (double*)malloc(sizeof(double) * zn);
    P->gA = (double*)malloc(sizeof(double) * zn);
    P->gAt = (double*)malloc(sizeof(double) * zn);
    for (int64_t j = 0; j <= n; j++) P->ptr1[j] = lp->colptr[j] - 1;
    for (int64_t k = 0; k < nnz; k++) { P->idx1[k] = lp->rowval[k] - 1; P->vA[k] = lp->nzval[k]; }
    orc_csc_transpose(m, n, P->ptr1, P->idx1, P->vA, P->ptr2, P->idx2, P->vAt, P->p21);
    for (int64_t k2 = 0; k2 < nnz; k2++) P->p12[P->p21[k2]] = k2;
    P->c = dup_vec(lp->c, n); P->lv = dup_vec(lp->lv, n); P->uv = dup_vec(lp->uv, n);
    P->lc = dup_vec(lp->lc, m); P->uc = dup_vec(lp->uc, m);
    P->D1 = dup_vec(NULL, m); P->D2 = dup_vec(NULL, n);
    for (int64_t i = 0; i < m; i++) P->D1[i] = 1.0;
    for (int64_t j = 0; j < n; j++) P->D2[j] = 1.0;
    return 0;
}

static void milp_build_gather(orc_milp* P) {
    for (int64_t k2 = 0; k2 < P->nnz; k2++) P->gA[k2] = P->vA[P->p21[k2]];
    for (int64_t k1 = 0; k1 < P->nnz; k1++) P->gAt[k1] = P->vAt[P->p12[k1]];
}

/* A*x (m) and At*y (n) on the scaled problem. */
static void milp_Ax(const orc_milp* P, const double* x, double* out) {
    orc_spmv_csr(P->m, P->ptr2, P->idx2, P->gA, x, out, 1.0, 0.0);
}
static void milp_Aty(const orc_milp* P, const double* y, double* out) {
    orc_spmv_csr(P->n, P->ptr1, P->idx1, P->gAt, y, out, 1.0, 0.0);
}

/* ------------------------------------------------------------------------ */
/* Preconditioning: src/components/preconditioning.jl                        */
/* ------------------------------------------------------------------------ */

/* norm(view(nonzeros(A), nzrange(A, j)), p) (linalg.jl:98-99) */
static double seg_norm(const double* v, int64_t a, int64_t b, double p) {
    if (b <= a) return 0.0;
    if (isinf(p) && p > 0) {
        double mx = 0.0;
        for (int64_t k = a; k < b; k++) mx = jl_max(mx, fabs(v[k]));
        return mx;
    }
    if (p == 1.0) {
        double s = 0.0;
        for (int64_t k = a; k < b; k++) s += fabs(v[k]);
        return s;
    }
    if (p == 2.0) {
        double s = 0.0;
        for (int64_t k = a; k < b; k++) s += v[k] * v[k];
        return sqrt(s);
    }
    if (p == 0.0) {
        double s = 0.0;
        for (int64_t k = a; k < b; k++) s += (v[k] != 0.0) ? 1.0 : 0.0;
        return s;
    }
    double s = 0.0;
    for (int64_t k = a; k < b; k++) s += pow(fabs(v[k]), p);
    return pow(s, 1.0 / p);
}

/* diagonal_norm_preconditioner (preconditioning.jl:102-111): column norms of A
 * from A's CSC values, row norms from At's CSC values; d = 1/sqrt(norm), or 1
 * when the norm is zero. */
static void diagonal_norm_prec(const orc_milp* P, const double* vA, const double* vAt,
                               double p_row, double p_col, double* d1, double* d2) {
    for (int64_t j = 0; j < P->n; j++) {
        double cn = seg_norm(vA, P->ptr1[j], P->ptr1[j + 1], p_col);
        d2[j] = (cn == 0.0) ? 1.0 : 1.0 / sqrt(cn);
    }
    for (int64_t i = 0; i < P->m; i++) {
        double rn = seg_norm(vAt, P->ptr2[i], P->ptr2[i + 1], p_row);
        d1[i] = (rn == 0.0) ? 1.0 : 1.0 / sqrt(rn);
    }
}

/* precondition(cons, prec) (preconditioning.jl:37-43):
 * A_p = D1*A*D2 -> (d1_i*a_ij)*d2_j ; At_p = D2*At*D1 -> (d2_j*a_ij)*d1_i. */
static void scale_cons(const orc_milp* P, const double* vA_in, const double* vAt_in,
                       const double* d1, const double* d2, double* vA_out, double* vAt_out) {
    for (int64_t j = 0; j < P->n; j++)
        for (int64_t k = P->ptr1[j]; k < P->ptr1[j + 1]; k++)
            vA_out[k] = (d1[P->idx1[k]] * vA_in[k]) * d2[j];
    for (int64_t i = 0; i < P->m; i++)
        for (int64_t k = P->ptr2[i]; k < P->ptr2[i + 1]; k++)
            vAt_out[k] = (d2[P->idx2[k]] * vAt_in[k]) * d1[i];
}

/* pdlp_preconditioner (preconditioning.jl:146-155) = ruiz (:117-125) then
 * chambolle_pock (:113-115) on the Ruiz-scaled constraints; returns the
 * product D1 = d1_r .* d1_cp, D2 = d2_cp .* d2_r. */
ORC_EXPORT void orc_pdlp_preconditioner_milp(const orc_milp* P, int32_t ruiz_iter, double alpha,
                                             double* D1, double* D2) {
    int64_t m = P->m, n = P->n, nnz = P->nnz;
    size_t zn = (size_t)(nnz > 0 ? nnz : 1);
    double* wA = (double*)malloc(sizeof(double) * zn);
    double* wAt = (double*)malloc(sizeof(double) * zn);
    double* tA = (double*)malloc(sizeof(double) * zn);
    double* tAt = (double*)malloc(sizeof(double) * zn);
    double* d1 = dup_vec(NULL, m);
    double* d2 = dup_vec(NULL, n);
    double* r1 = dup_vec(NULL, m);
    double* r2 = dup_vec(NULL, n);
    memcpy(wA, P->vA, sizeof(double) * (size_t)nnz);
    memcpy(wAt, P->vAt, sizeof(double) * (size_t)nnz);
    for (int64_t i = 0; i < m; i++) r1[i] = 1.0;  /* identity_preconditioner (:95-100) */
    for (int64_t j = 0; j < n; j++) r2[j] = 1.0;
    for (int32_t it = 0; it < ruiz_iter; it++) {
        diagonal_norm_prec(P, wA, wAt, INFINITY, INFINITY, d1, d2);
        scale_cons(P, wA, wAt, d1, d2, tA, tAt);
        memcpy(wA, tA, sizeof(double) * (size_t)nnz);
        memcpy(wAt, tAt, sizeof(double) * (size_t)nnz);
        /* prec = prec_next * prec: D1 = d1_next .* D1, D2 = D2 .* d2_next (:24-26) */
        for (int64_t i = 0; i < m; i++) r1[i] = d1[i] * r1[i];
        for (int64_t j = 0; j < n; j++) r2[j] = r2[j] * d2[j];
    }
    /* cons_r = precondition(cons, prec_r): the accumulated diagonals applied to
     * the ORIGINAL matrix, not the iterated one (:153) */
    scale_cons(P, P->vA, P->vAt, r1, r2, tA, tAt);
    diagonal_norm_prec(P, tA, tAt, 2.0 - alpha, alpha, d1, d2);
    for (int64_t i = 0; i < m; i++) D1[i] = r1[i] * d1[i];
    for (int64_t j = 0; j < n; j++) D2[j] = d2[j] * r2[j];
    free(wA); free(wAt); free(tA); free(tAt); free(d1); free(d2); free(r1); free(r2);
}

/* ruiz_preconditioner (preconditioning.jl:117-125) alone (with_cp = 0) or
 * pdlp_preconditioner (:146-155) (with_cp = 1) of an LP's matrix. */
ORC_EXPORT void orc_lp_preconditioner(const cpdlp_lp* lp, int32_t ruiz_iter, double alpha,
                                      int32_t with_cp, double* D1, double* D2) {
    orc_milp P;
    milp_from_lp(lp, &P);
    if (with_cp) {
        orc_pdlp_preconditioner_milp(&P, ruiz_iter, alpha, D1, D2);
    } else {
        int64_t nnz = P.nnz;
        size_t zn = (size_t)(nnz > 0 ? nnz : 1);
        double* wA = (double*)malloc(sizeof(double) * zn);
        double* wAt = (double*)malloc(sizeof(double) * zn);
        double* tA = (double*)malloc(sizeof(double) * zn);
        double* tAt = (double*)malloc(sizeof(double) * zn);
        double* d1 = dup_vec(NULL, P.m);
        double* d2 = dup_vec(NULL, P.n);
        memcpy(wA, P.vA, sizeof(double) * (size_t)nnz);
        memcpy(wAt, P.vAt, sizeof(double) * (size_t)nnz);
        for (int64_t i = 0; i < P.m; i++) D1[i] = 1.0;
        for (int64_t j = 0; j < P.n; j++) D2[j] = 1.0;
        for (int32_t it = 0; it < ruiz_iter; it++) {
            diagonal_norm_prec(&P, wA, wAt, INFINITY, INFINITY, d1, d2);
            scale_cons(&P, wA, wAt, d1, d2, tA, tAt);
            memcpy(wA, tA, sizeof(double) * (size_t)nnz);
            memcpy(wAt, tAt, sizeof(double) * (size_t)nnz);
            for (int64_t i = 0; i < P.m; i++) D1[i] = d1[i] * D1[i];
            for (int64_t j = 0; j < P.n; j++) D2[j] = D2[j] * d2[j];
        }
        free(wA); free(wAt); free(tA); free(tAt); free(d1); free(d2);
    }
    milp_free(&P);
}

/* precondition(milp, prec) (preconditioning.jl:61-91), in place on P. */
static void precondition_milp(orc_milp* P, const double* D1, const double* D2) {
    int64_t nnz = P->nnz;
    size_t zn = (size_t)(nnz > 0 ? nnz : 1);
    double* tA = (double*)malloc(sizeof(double) * zn);
    double* tAt = (double*)malloc(sizeof(double) * zn);
    scale_cons(P, P->vA, P->vAt, D1, D2, tA, tAt);
    memcpy(P->vA, tA, sizeof(double) * (size_t)nnz);
    memcpy(P->vAt, tAt, sizeof(double) * (size_t)nnz);
    free(tA); free(tAt);
    for (int64_t j = 0; j < P->n; j++) {
        P->c[j] = D2[j] * P->c[j];
        P->lv[j] = P->lv[j] / D2[j];
        P->uv[j] = P->uv[j] / D2[j];
        P->D2[j] = P->D2[j] * D2[j];  /* new_prec = prec * Preconditioner(milp) */
    }
    for (int64_t i = 0; i < P->m; i++) {
        P->lc[i] = D1[i] * P->lc[i];
        P->uc[i] = D1[i] * P->uc[i];
        P->D1[i] = D1[i] * P->D1[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Step size: src/components/step_size.jl, src/utils/linalg.jl:60-96          */
/* ------------------------------------------------------------------------ */
static double dotv(const double* a, const double* b, int64_t len) {
    double s = 0.0;
    for (int64_t i = 0; i < len; i++) s += a[i] * b[i];
    return s;
}
static double norm2v(const double* a, int64_t len) { return sqrt(dotv(a, a, len)); }

/* IterativeSolvers 0.9.4 default tol = eps(T) * size(B,2)^3 with Julia Int64
 * arithmetic (wraps modulo 2^64). */
ORC_EXPORT double orc_powm_default_tol(int64_t n, int32_t is_f32) {
    uint64_t un = (uint64_t)n;
    int64_t n3 = (int64_t)(un * un * un);
    double eps = is_f32 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
    return eps * (double)n3;
}

/* spectral_norm(K, K') (linalg.jl:86-96) through powm! on Symmetrized(K, K')
 * (linalg.jl:60-79): per iteration Ax = K'(K x), theta = x'Ax,
 * r = Ax - theta*x, residual = ||r||, x = Ax * (1/||Ax||); stops when
 * iteration > maxiter or residual <= tol; returns sqrt(theta). */
static double spectral_norm(const orc_milp* P, uint64_t seed, double tol, int64_t maxiter,
                            int64_t* iters_out) {
    int64_t m = P->m, n = P->n;
    double* x = dup_vec(NULL, n);
    double* Ax = dup_vec(NULL, n);
    double* r = dup_vec(NULL, n);
    double* s = dup_vec(NULL, m);
    orc_gaussian_vector(seed, n, x);
    double theta = 0.0, residual = INFINITY;
    int64_t it = 0;
    while (!(it > maxiter || residual <= tol)) {
        milp_Ax(P, x, s);
        milp_Aty(P, s, Ax);
        theta = dotv(x, Ax, n);
        for (int64_t j = 0; j < n; j++) r[j] = (-theta) * x[j] + Ax[j];
        residual = norm2v(r, n);
        double inv = 1.0 / norm2v(Ax, n);
        for (int64_t j = 0; j < n; j++) x[j] = Ax[j] * inv;
        it++;
    }
    if (iters_out) *iters_out = it;
    free(x); free(Ax); free(r); free(s);
    return sqrt(theta);
}

/* ------------------------------------------------------------------------ */
/* KKT errors: src/components/errors.jl:55-109                               */
/* ------------------------------------------------------------------------ */
typedef struct orc_work { double *sx, *sy, *sr; } orc_work;

static void kkt_errors(const orc_milp* P, orc_work* W, const double* x, const double* y,
                       cpdlp_kkt_errors* e) {
    int64_t m = P->m, n = P->n;
    double* Ax = W->sy;
    double* Aty = W->sx;
    milp_Ax(P, x, Ax);
    milp_Aty(P, y, Aty);
    double primal_sq = 0.0, pscale_sq = 0.0, pc_sum = 0.0;
    for (int64_t i = 0; i < m; i++) {
        double inv1 = 1.0 / P->D1[i];
        double d = inv1 * (Ax[i] - proj_box(Ax[i], P->lc[i], P->uc[i]));
        primal_sq += d * d;
        double cb = inv1 * combine(P->lc[i], P->uc[i]);
        pscale_sq += cb * cb;
        pc_sum += safeprod_left(P->uc[i], pos_part(-y[i])) - safeprod_left(P->lc[i], neg_part(-y[i]));
    }
    double dual_sq = 0.0, dscale_sq = 0.0, pv_sum = 0.0, cx = 0.0;
    for (int64_t j = 0; j < n; j++) {
        double rj = proj_multiplier(P->c[j] - Aty[j], P->lv[j], P->uv[j]);
        double inv2 = 1.0 / P->D2[j];
        double d = inv2 * ((P->c[j] - Aty[j]) - rj);
        dual_sq += d * d;
        double co = inv2 * P->c[j];
        dscale_sq += co * co;
        pv_sum += safeprod_left(P->uv[j], pos_part(-rj)) - safeprod_left(P->lv[j], neg_part(-rj));
        cx += P->c[j] * x[j];
    }
    e->primal = sqrt(primal_sq);
    e->primal_scale = 1.0 + sqrt(pscale_sq);
    e->dual = sqrt(dual_sq);
    e->dual_scale = 1.0 + sqrt(dscale_sq);
    e->gap = fabs((cx + pc_sum) + pv_sum);
    e->gap_scale = (1.0 + fabs(pc_sum + pv_sum)) + fabs(cx);
}

/* relative / absolute (errors.jl:55-63) */
static double err_relative(const cpdlp_kkt_errors* e) {
    return jl_max(jl_max(e->primal / e->primal_scale, e->dual / e->dual_scale), e->gap / e->gap_scale);
}
static double err_absolute(const cpdlp_kkt_errors* e, double w) {
    return sqrt((w * w) * (e->primal * e->primal) + (1.0 / (w * w)) * (e->dual * e->dual) +
                e->gap * e->gap);
}
ORC_EXPORT double orc_err_relative(const cpdlp_kkt_errors* e) { return err_relative(e); }
ORC_EXPORT double orc_err_absolute(const cpdlp_kkt_errors* e, double w) { return err_absolute(e, w); }

/* ------------------------------------------------------------------------ */
/* Solver state: src/algorithms/pdlp.jl:20-67, pdhg.jl:25-54                 */
/* ------------------------------------------------------------------------ */
typedef struct orc_state {
    orc_milp P;
    cpdlp_params prm;
    int64_t m, n;
    /* sol / sol_last are swapped by pointer every step (pdlp.jl:101) */
    double *x, *y, *x_last, *y_last;
    double *xa, *ya, *xa_last, *ya_last;   /* sol_avg, sol_avg_last */
    double *xr, *yr;                       /* sol_restart */
    orc_work W;
    double eta, eta_sum, omega;
    int64_t outer, inner, total, kkt_passes;
    int32_t status, restart_from_avg;
    cpdlp_kkt_errors err, err_cand, err_cand_last, err_restart;
    double starting_time, time_elapsed, setup_seconds;
    int64_t power_iterations;
    int64_t hist_len, hist_cap;
    int64_t* hist_passes;
    cpdlp_kkt_errors* hist_err;
} orc_state;

static void push_history(orc_state* S) {
    if (!S->prm.record_error_history) return;
    if (S->hist_len == S->hist_cap) {
        S->hist_cap = S->hist_cap ? 2 * S->hist_cap : 64;
        S->hist_passes = (int64_t*)realloc(S->hist_passes, sizeof(int64_t) * (size_t)S->hist_cap);
        S->hist_err = (cpdlp_kkt_errors*)realloc(S->hist_err, sizeof(cpdlp_kkt_errors) * (size_t)S->hist_cap);
    }
    S->hist_passes[S->hist_len] = S->kkt_passes;
    S->hist_err[S->hist_len] = S->err;
    S->hist_len++;
}

static void nan_errors(cpdlp_kkt_errors* e) {
    e->primal = e->primal_scale = e->dual = e->dual_scale = e->gap = e->gap_scale = NAN;
}

/* preprocess (common.jl:154-169) + initialize (pdlp.jl:45-67 / pdhg.jl:40-54).
 * Starting point x0/y0 in original units (NULL = zeros). */
ORC_EXPORT orc_state* orc_state_create(const cpdlp_lp* lp, const cpdlp_params* prm,
                                       const double* x0, const double* y0) {
    double t0 = now_seconds();
    orc_state* S = (orc_state*)calloc(1, sizeof(orc_state));
    S->prm = *prm;
    S->starting_time = t0;
    milp_from_lp(lp, &S->P);
    orc_milp* P = &S->P;
    int64_t m = lp->m, n = lp->n;
    S->m = m; S->n = n;
    double* D1 = dup_vec(NULL, m);
    double* D2 = dup_vec(NULL, n);
    orc_pdlp_preconditioner_milp(P, prm->ruiz_iter, prm->chambolle_pock_alpha, D1, D2);
    precondition_milp(P, D1, D2);
    milp_build_gather(P);
    S->x = dup_vec(NULL, n); S->y = dup_vec(NULL, m);
    /* precondition(sol, prec) (preconditioning.jl:45-51): x ./ D2, y ./ D1 */
    for (int64_t j = 0; j < n; j++) S->x[j] = (x0 ? x0[j] : 0.0) / D2[j];
    for (int64_t i = 0; i < m; i++) S->y[i] = (y0 ? y0[i] : 0.0) / D1[i];
    free(D1); free(D2);
    S->x_last = dup_vec(NULL, n); S->y_last = dup_vec(NULL, m);
    S->xa = dup_vec(S->x, n); S->ya = dup_vec(S->y, m);
    S->xa_last = dup_vec(NULL, n); S->ya_last = dup_vec(NULL, m);
    S->xr = dup_vec(S->x, n); S->yr = dup_vec(S->y, m);
    memset(S->x_last, 0, sizeof(double) * (size_t)n);
    memset(S->y_last, 0, sizeof(double) * (size_t)m);
    memset(S->xa_last, 0, sizeof(double) * (size_t)n);
    memset(S->ya_last, 0, sizeof(double) * (size_t)m);
    S->W.sx = dup_vec(NULL, n); S->W.sy = dup_vec(NULL, m); S->W.sr = dup_vec(NULL, n);
    /* fixed_stepsize (step_size.jl:22-27) */
    double tol = prm->power_tol_override > 0 ? prm->power_tol_override : orc_powm_default_tol(n, 0);
    int64_t maxiter = prm->power_maxiter_override > 0 ? prm->power_maxiter_override : n;
    double sn = spectral_norm(P, prm->power_seed, tol, maxiter, &S->power_iterations);
    S->eta = prm->invnorm_scaling * (1.0 / sn);
    /* primal_weight_init (step_size.jl:29-40); PDHG fixes omega = 1 (pdhg.jl:48) */
    if (prm->algorithm == CPDLP_ALGO_PDHG) {
        S->omega = 1.0;
    } else {
        double c_norm = norm2v(P->c, n);
        double cb = 0.0;
        for (int64_t i = 0; i < m; i++) { double v = combine(P->lc[i], P->uc[i]); cb += v * v; }
        double cb_norm = sqrt(cb);
        S->omega = (c_norm > prm->zero_tol && cb_norm > prm->zero_tol) ? c_norm / cb_norm : 1.0;
    }
    S->eta_sum = 0.0;
    S->status = CPDLP_STILL_RUNNING;
    nan_errors(&S->err); nan_errors(&S->err_cand); nan_errors(&S->err_cand_last); nan_errors(&S->err_restart);
    S->setup_seconds = now_seconds() - t0;
    return S;
}

ORC_EXPORT void orc_state_destroy(orc_state* S) {
    if (!S) return;
    milp_free(&S->P);
    free(S->x); free(S->y); free(S->x_last); free(S->y_last);
    free(S->xa); free(S->ya); free(S->xa_last); free(S->ya_last);
    free(S->xr); free(S->yr);
    free(S->W.sx); free(S->W.sy); free(S->W.sr);
    free(S->hist_passes); free(S->hist_err);
    free(S);
}

/* step! (pdlp.jl:96-124, pdhg.jl:76-102) */
static void step(orc_state* S) {
    orc_milp* P = &S->P;
    int64_t m = S->m, n = S->n;
    double* t;
    /* switch pointers (pdlp.jl:101) */
    t = S->x; S->x = S->x_last; S->x_last = t;
    t = S->y; S->y = S->y_last; S->y_last = t;
    const double *x = S->x_last, *y = S->y_last;
    double *xp = S->x, *yp = S->y;
    double tau = S->eta / S->omega, sigma = S->eta * S->omega;
    double* Aty = S->W.sx;
    milp_Aty(P, y, Aty);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (n > 16384)
#endif
    for (int64_t j = 0; j < n; j++) {
        xp[j] = proj_box(x[j] - tau * (P->c[j] - Aty[j]), P->lv[j], P->uv[j]);
        Aty[j] = 2.0 * xp[j] - x[j];   /* xdiff overwrites scratch.x (pdlp.jl:113) */
    }
    double* Axd = S->W.sy;
    milp_Ax(P, Aty, Axd);
    double inv_sigma = 1.0 / sigma;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (m > 16384)
#endif
    for (int64_t i = 0; i < m; i++) {
        yp[i] = (y[i] - sigma * Axd[i]) - sigma * proj_box(inv_sigma * y[i] - Axd[i], -P->uc[i], -P->lc[i]);
    }
    S->kkt_passes += 1;
    if (S->prm.algorithm == CPDLP_ALGO_PDLP) {
        /* update_average! (pdlp.jl:126-136): copy!(avg_last, avg) then
         * axpby!(eta/(eta+eta_sum), sol, eta_sum/(eta+eta_sum), avg) */
        double a = S->eta / (S->eta + S->eta_sum);
        double b = S->eta_sum / (S->eta + S->eta_sum);
        t = S->xa_last; S->xa_last = S->xa; S->xa = t;
        t = S->ya_last; S->ya_last = S->ya; S->ya = t;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (n > 16384)
#endif
        for (int64_t j = 0; j < n; j++) S->xa[j] = xp[j] * a + S->xa_last[j] * b;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (m > 16384)
#endif
        for (int64_t i = 0; i < m; i++) S->ya[i] = yp[i] * a + S->ya_last[i] * b;
        S->eta_sum += S->eta;
        /* add_inner! (iteration.jl:7-11) */
        S->inner += 1;
        S->total += 1;
    }
}

ORC_EXPORT void orc_state_step(orc_state* S, int64_t count) {
    for (int64_t k = 0; k < count; k++) step(S);
}

/* termination_status (termination.jl:89-101) */
static int32_t termination_status(const orc_state* S) {
    if (err_relative(&S->err) <= S->prm.termination_reltol) return CPDLP_OPTIMAL;
    if (S->time_elapsed >= S->prm.time_limit) return CPDLP_TIME_LIMIT;
    if (S->kkt_passes >= S->prm.max_kkt_passes) return CPDLP_ITERATION_LIMIT;
    return CPDLP_STILL_RUNNING;
}

/* termination_check! (common.jl:218-231) */
static int termination_check(orc_state* S) {
    S->time_elapsed = now_seconds() - S->starting_time;
    kkt_errors(&S->P, &S->W, S->x, S->y, &S->err);
    push_history(S);
    S->status = termination_status(S);
    return S->status != CPDLP_STILL_RUNNING;
}

/* restart_check! (pdlp.jl:138-170) + should_restart (restart.jl:40-57) */
static int restart_check(orc_state* S) {
    double w = S->omega;
    cpdlp_kkt_errors e, ea, el, eal;
    kkt_errors(&S->P, &S->W, S->x, S->y, &e);
    kkt_errors(&S->P, &S->W, S->xa, S->ya, &ea);
    if (err_absolute(&e, w) < err_absolute(&ea, w)) {
        S->restart_from_avg = 0;
        S->err_cand = e;
    } else {
        S->restart_from_avg = 1;
        S->err_cand = ea;
    }
    kkt_errors(&S->P, &S->W, S->x_last, S->y_last, &el);
    kkt_errors(&S->P, &S->W, S->xa_last, S->ya_last, &eal);
    S->err_cand_last = (err_absolute(&el, w) < err_absolute(&eal, w)) ? el : eal;
    kkt_errors(&S->P, &S->W, S->xr, S->yr, &S->err_restart);
    double ac = err_absolute(&S->err_cand, w);
    double ar = err_absolute(&S->err_restart, w);
    double acl = err_absolute(&S->err_cand_last, w);
    int sufficient = ac <= S->prm.sufficient_decay * ar;
    int necessary = ac <= S->prm.necessary_decay * ar;
    int no_local_progress = ac > acl;
    int long_inner_loop = (double)S->inner >= S->prm.artificial_decay * (double)S->total;
    return sufficient || (necessary && no_local_progress) || long_inner_loop;
}

/* restart! (pdlp.jl:172-196) + primal_weight_update! (step_size.jl:58-75) */
static void restart(orc_state* S) {
    int64_t m = S->m, n = S->n;
    const double* cx = S->restart_from_avg ? S->xa : S->x;
    const double* cy = S->restart_from_avg ? S->ya : S->y;
    S->eta_sum = 0.0;
    double dx = 0.0, dy = 0.0;
    for (int64_t j = 0; j < n; j++) { double d = cx[j] - S->xr[j]; dx += d * d; }
    for (int64_t i = 0; i < m; i++) { double d = cy[i] - S->yr[i]; dy += d * d; }
    dx = sqrt(dx); dy = sqrt(dy);
    double th = S->prm.primal_weight_damping;
    if (dx > S->prm.zero_tol && dy > S->prm.zero_tol)
        S->omega = exp(th * log(dy / dx) + (1.0 - th) * log(S->omega));
    if (S->restart_from_avg) {
        memcpy(S->x, S->xa, sizeof(double) * (size_t)n);
        memcpy(S->y, S->ya, sizeof(double) * (size_t)m);
    }
    memset(S->xa, 0, sizeof(double) * (size_t)n);
    memset(S->ya, 0, sizeof(double) * (size_t)m);
    memcpy(S->xr, S->x, sizeof(double) * (size_t)n);
    memcpy(S->yr, S->y, sizeof(double) * (size_t)m);
    S->outer += 1;   /* add_outer! (iteration.jl:13-17) */
    S->inner = 0;
}

/* solve! (pdlp.jl:69-94, pdhg.jl:56-74) with a budget of `max_blocks` rounds
 * of (check_every steps + checks); the reference's nested loops reduce to:
 * block, termination check, restart check, and on termination one more
 * termination check (pdlp.jl:88).  Returns STILL_RUNNING if the budget ends. */
ORC_EXPORT int32_t orc_state_solve_blocks(orc_state* S, int64_t max_blocks) {
    int32_t ce = S->prm.check_every;
    int64_t blocks = 0;
    if (S->prm.algorithm == CPDLP_ALGO_PDHG) {
        for (;;) {
            if (blocks >= max_blocks) return S->status;
            for (int32_t k = 0; k < ce; k++) step(S);
            blocks++;
            if (termination_check(S)) break;
        }
        return S->status;
    }
    for (;;) {
        if (blocks >= max_blocks) return S->status;
        for (int32_t k = 0; k < ce; k++) step(S);
        blocks++;
        if (termination_check(S)) {
            termination_check(S);
            break;
        }
        if (restart_check(S)) restart(S);
    }
    return S->status;
}

ORC_EXPORT int32_t orc_state_solve(orc_state* S) { return orc_state_solve_blocks(S, INT64_MAX); }

ORC_EXPORT void orc_state_stats(const orc_state* S, cpdlp_stats* st) {
    memset(st, 0, sizeof(*st));
    st->err = S->err;
    st->time_elapsed = S->time_elapsed;
    st->kkt_passes = S->kkt_passes;
    st->termination_status = S->status;
    st->restart_from_avg = S->restart_from_avg;
    st->outer = S->outer; st->inner = S->inner; st->total = S->total;
    st->eta = S->eta; st->eta_sum = S->eta_sum; st->omega = S->omega;
    st->history_length = S->hist_len;
    st->power_iterations = S->power_iterations;
    st->setup_seconds = S->setup_seconds;
}

/* which: CPDLP_VEC_* ; scaled units */
ORC_EXPORT void orc_state_vectors(const orc_state* S, int32_t which, double* x, double* y) {
    const double *sx = S->x, *sy = S->y;
    switch (which) {
        case CPDLP_VEC_SOL_LAST: sx = S->x_last; sy = S->y_last; break;
        case CPDLP_VEC_SOL_AVG: sx = S->xa; sy = S->ya; break;
        case CPDLP_VEC_SOL_AVG_LAST: sx = S->xa_last; sy = S->ya_last; break;
        case CPDLP_VEC_SOL_RESTART: sx = S->xr; sy = S->yr; break;
        default: break;
    }
    if (x) memcpy(x, sx, sizeof(double) * (size_t)S->n);
    if (y) memcpy(y, sy, sizeof(double) * (size_t)S->m);
}

ORC_EXPORT void orc_state_kkt(orc_state* S, int32_t which, cpdlp_kkt_errors* e) {
    double* x = (double*)malloc(sizeof(double) * (size_t)(S->n > 0 ? S->n : 1));
    double* y = (double*)malloc(sizeof(double) * (size_t)(S->m > 0 ? S->m : 1));
    orc_state_vectors(S, which, x, y);
    kkt_errors(&S->P, &S->W, x, y, e);
    free(x); free(y);
}

/* get_solution (common.jl:233-235) + unprecondition (preconditioning.jl:53-59) */
ORC_EXPORT void orc_state_solution(const orc_state* S, double* x, double* y) {
    for (int64_t j = 0; j < S->n; j++) x[j] = S->P.D2[j] * S->x[j];
    for (int64_t i = 0; i < S->m; i++) y[i] = S->P.D1[i] * S->y[i];
}

ORC_EXPORT int64_t orc_state_history(const orc_state* S, int64_t* passes, cpdlp_kkt_errors* errs,
                                     int64_t cap) {
    int64_t k = S->hist_len < cap ? S->hist_len : cap;
    for (int64_t t = 0; t < k; t++) { passes[t] = S->hist_passes[t]; errs[t] = S->hist_err[t]; }
    return S->hist_len;
}

/* The scaled problem of a state: D1, D2, scaled vectors and the gather-layout
 * values (S2 order for A, S1 order for At), for scaling parity tests. */
ORC_EXPORT void orc_state_scaled(const orc_state* S, double* D1, double* D2, double* c, double* lv,
                                 double* uv, double* lc, double* uc, double* gA, double* gAt) {
    const orc_milp* P = &S->P;
    if (D1) memcpy(D1, P->D1, sizeof(double) * (size_t)P->m);
    if (D2) memcpy(D2, P->D2, sizeof(double) * (size_t)P->n);
    if (c) memcpy(c, P->c, sizeof(double) * (size_t)P->n);
    if (lv) memcpy(lv, P->lv, sizeof(double) * (size_t)P->n);
    if (uv) memcpy(uv, P->uv, sizeof(double) * (size_t)P->n);
    if (lc) memcpy(lc, P->lc, sizeof(double) * (size_t)P->m);
    if (uc) memcpy(uc, P->uc, sizeof(double) * (size_t)P->m);
    if (gA) memcpy(gA, P->gA, sizeof(double) * (size_t)P->nnz);
    if (gAt) memcpy(gAt, P->gAt, sizeof(double) * (size_t)P->nnz);
}

/* KKT errors of an arbitrary (x, y) in scaled units on the state's problem. */
ORC_EXPORT void orc_state_kkt_of(orc_state* S, const double* x, const double* y, cpdlp_kkt_errors* e) {
    kkt_errors(&S->P, &S->W, x, y, e);
}

/* solve(milp, sol, algo) (common.jl:186-209), including the early exit for a
 * problem without constraints and with zero cost (:194-198). */
ORC_EXPORT int32_t orc_solve(const cpdlp_lp* lp, const cpdlp_params* prm, const double* x0,
                             const double* y0, double* x_out, double* y_out, cpdlp_stats* st,
                             orc_state** keep) {
    orc_state* S = orc_state_create(lp, prm, x0, y0);
    int zero_c = 1;
    for (int64_t j = 0; j < S->n; j++) if (S->P.c[j] != 0.0) { zero_c = 0; break; }
    if (S->m == 0 && zero_c) {
        for (int64_t j = 0; j < S->n; j++) S->x[j] = proj_box(0.0, S->P.lv[j], S->P.uv[j]);
        S->status = CPDLP_OPTIMAL;
    } else {
        orc_state_solve(S);
    }
    if (x_out && y_out) orc_state_solution(S, x_out, y_out);
    if (st) orc_state_stats(S, st);
    int32_t status = S->status;
    if (keep) *keep = S; else orc_state_destroy(S);
    return status;
}

/* Thread count of the OpenMP row loops (the CPU baselines time 1 thread, as
 * the reference's single-threaded CPU path, and all host threads). */
ORC_EXPORT void orc_set_num_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

ORC_EXPORT int32_t orc_num_threads(void) {
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}
