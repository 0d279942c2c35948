// abi.cu -- the extern "C" entry points of libcoolpdlp_cuda (include/coolpdlp_cuda.h).
// Each converts cpdlp::Error / std::exception into a status code and stores
// the message in the handle.
#include <memory>
#include <new>
#include <vector>

#include "batch.cuh"
#include "duals.cuh"
#include "tiles.cuh"
#include "matrix.cuh"
#include "noalloc.cuh"
#include "permutation.cuh"
#include "solver.cuh"

using namespace cpdlp;

struct cpdlp_handle : Handle {};

namespace {

inline Handle* H(cpdlp_handle* h) { return static_cast<Handle*>(h); }

template <class F>
int guarded(cpdlp_handle* h, F&& f) {
    try {
        if (h) CK(cudaSetDevice(h->device));
        AllocScope scope(h ? h->stream : nullptr);
        f();
        if (h) h->last_error.clear();
        return CPDLP_OK;
    } catch (const Error& e) {
        if (h) h->last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        if (h) h->last_error = "host allocation failed";
        return CPDLP_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        if (h) h->last_error = e.what();
        return CPDLP_ERR_CUDA;
    }
}

#define NEED(h) \
    if (!(h)) return CPDLP_ERR_ARGUMENT

}  // namespace

extern "C" {

int cpdlp_abi_version(void) { return CPDLP_ABI_VERSION; }

void cpdlp_params_default(cpdlp_params* p, int32_t algorithm) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    const bool pdhg = algorithm == CPDLP_ALGO_PDHG;
    p->algorithm = pdhg ? CPDLP_ALGO_PDHG : CPDLP_ALGO_PDLP;
    p->float_type = CPDLP_VAL_F64;
    p->chambolle_pock_alpha = 1.0;
    p->ruiz_iter = pdhg ? 0 : 10;
    p->invnorm_scaling = 0.9;
    p->primal_weight_damping = pdhg ? NAN : 0.5;
    p->zero_tol = 1e-8;
    p->sufficient_decay = pdhg ? NAN : 0.2;
    p->necessary_decay = pdhg ? NAN : 0.8;
    p->artificial_decay = pdhg ? NAN : 0.36;
    p->show_progress = 0;
    p->check_every = 100;
    p->record_error_history = 1;
    p->termination_reltol = 1e-4;
    p->max_kkt_passes = 100000;
    p->time_limit = 100.0;
    p->power_tol_override = 0.0;
    p->power_maxiter_override = 0;
    p->power_seed = 0;
    p->refine_reltol = 0.0;
    p->tile_nnz = 0;
    p->infeasibility_tol = 0.0;
    p->matrix_type = CPDLP_FMT_AUTO;
}

int cpdlp_create(int32_t device, cpdlp_handle** out) {
    if (!out) return CPDLP_ERR_ARGUMENT;
    *out = nullptr;
    cpdlp_handle* h = new (std::nothrow) cpdlp_handle();
    if (!h) return CPDLP_ERR_OUT_OF_MEMORY;
    h->device = device;
    int rc = guarded(h, [&] {
        int count = 0;
        CK(cudaGetDeviceCount(&count));
        if (device < 0 || device >= count) fail(CPDLP_ERR_ARGUMENT, "no such CUDA device");
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device));
        // keep up to 16 GiB of freed stream-ordered memory in this process's
        // pool instead of returning it to the driver at every synchronisation
        cudaMemPool_t pool;
        CK(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t keep = 16ull << 30;
        CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    });
    if (rc != CPDLP_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return CPDLP_OK;
}

int cpdlp_destroy(cpdlp_handle* h) {
    NEED(h);
    cudaSetDevice(h->device);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    if (h->pinned) cudaFreeHost(h->pinned);
    h->host_release_all();
    delete h;
    return CPDLP_OK;
}

const char* cpdlp_last_error(const cpdlp_handle* h) {
    if (!h) return "null handle";
    return h->last_error.c_str();
}

int cpdlp_synchronize(cpdlp_handle* h) {
    NEED(h);
    return guarded(h, [&] { CK(cudaStreamSynchronize(h->stream)); });
}

void* cpdlp_stream(cpdlp_handle* h) { return h ? (void*)h->stream : nullptr; }

// ---- matrices ----
int cpdlp_matrix_from_csc(cpdlp_handle* h, int64_t m, int64_t n, int64_t nnz,
                          const int64_t* colptr, const int64_t* rowval, const double* nzval,
                          int32_t format, int32_t value_type, cpdlp_matrix** out) {
    NEED(h);
    if (!out) return CPDLP_ERR_ARGUMENT;
    *out = nullptr;
    return guarded(h, [&] {
        Matrix* M = matrix_from_csc(*H(h), m, n, nnz, colptr, rowval, nzval, format, value_type);
        *out = reinterpret_cast<cpdlp_matrix*>(M);
    });
}

int cpdlp_matrix_destroy(cpdlp_matrix* A) {
    if (!A) return CPDLP_ERR_ARGUMENT;
    Matrix* M = reinterpret_cast<Matrix*>(A);
    cudaSetDevice(M->h->device);
    cudaStreamSynchronize(M->h->stream);
    delete M;
    return CPDLP_OK;
}

int cpdlp_matrix_shape(const cpdlp_matrix* A, int64_t* m, int64_t* n, int64_t* nnz,
                       int64_t* width) {
    if (!A) return CPDLP_ERR_ARGUMENT;
    const Matrix* M = reinterpret_cast<const Matrix*>(A);
    if (m) *m = M->m;
    if (n) *n = M->n;
    if (nnz) *nnz = M->nnz;
    if (width) *width = M->width;
    return CPDLP_OK;
}

int cpdlp_matrix_export(cpdlp_handle* h, const cpdlp_matrix* A, int64_t* ptr, int64_t* idx,
                        double* val) {
    NEED(h);
    if (!A) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { matrix_export(*H(h), *reinterpret_cast<const Matrix*>(A), ptr, idx, val); });
}

int cpdlp_spmv(cpdlp_handle* h, const cpdlp_matrix* A, const void* b, void* c, double alpha,
               double beta) {
    NEED(h);
    if (!A) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        matrix_spmv(*H(h), *reinterpret_cast<const Matrix*>(A), b, c, alpha, beta);
        CK(cudaStreamSynchronize(h->stream));
    });
}

int cpdlp_spmv_csr_noalloc(cpdlp_handle* h, int64_t m, int64_t n, int64_t nnz,
                           const int32_t* rowptr, const int32_t* colval, const void* nzval,
                           int32_t value_type, const void* b, void* c, double alpha,
                           double beta) {
    NEED(h);
    return guarded(h, [&] {
        spmv_csr_noalloc(*H(h), m, n, nnz, rowptr, colval, nzval, value_type, b, c, alpha, beta);
    });
}

int cpdlp_sort_rows_columns(cpdlp_handle* h, const cpdlp_lp* lp, int64_t* perm_var,
                            int64_t* perm_cons, int64_t* colptr, int64_t* rowval, double* nzval,
                            double* c, double* lv, double* uv, double* lc, double* uc) {
    if (!lp) {
        if (h) h->last_error = "null LP";
        return CPDLP_ERR_ARGUMENT;
    }
    return guarded(h, [&] {
        sort_rows_columns(*lp, perm_var, perm_cons, colptr, rowval, nzval, c, lv, uv, lc, uc);
    });
}

// ---- solve path ----
int cpdlp_problem_create(cpdlp_handle* h, const cpdlp_lp* lp, const cpdlp_params* params,
                         cpdlp_problem** out) {
    NEED(h);
    if (!out) return CPDLP_ERR_ARGUMENT;
    *out = nullptr;
    return guarded(h, [&] {
        *out = reinterpret_cast<cpdlp_problem*>(problem_create(*H(h), lp, params));
    });
}

int cpdlp_problem_destroy(cpdlp_problem* p) {
    if (!p) return CPDLP_ERR_ARGUMENT;
    ProblemBase* P = reinterpret_cast<ProblemBase*>(p);
    cudaSetDevice(P->h->device);
    cudaStreamSynchronize(P->h->stream);
    delete P;
    return CPDLP_OK;
}

int cpdlp_problem_scaling(cpdlp_handle* h, const cpdlp_problem* p, double* d1, double* d2) {
    NEED(h);
    if (!p) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        problem_scaling(*H(h), const_cast<ProblemBase*>(reinterpret_cast<const ProblemBase*>(p)), d1, d2);
    });
}

int cpdlp_problem_spectral_norm(cpdlp_handle* h, cpdlp_problem* p, const cpdlp_params* params,
                                double* norm, int64_t* iterations) {
    NEED(h);
    if (!p || !params) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        double v = problem_spectral_norm(*H(h), reinterpret_cast<ProblemBase*>(p), params, iterations);
        if (norm) *norm = v;
    });
}

int cpdlp_state_create(cpdlp_handle* h, cpdlp_problem* p, const cpdlp_params* params,
                       const double* x0, const double* y0, cpdlp_state** out) {
    NEED(h);
    if (!out) return CPDLP_ERR_ARGUMENT;
    *out = nullptr;
    return guarded(h, [&] {
        *out = reinterpret_cast<cpdlp_state*>(
            state_create(*H(h), reinterpret_cast<ProblemBase*>(p), params, x0, y0));
    });
}

int cpdlp_state_destroy(cpdlp_state* s) {
    if (!s) return CPDLP_ERR_ARGUMENT;
    StateBase* S = reinterpret_cast<StateBase*>(s);
    cudaSetDevice(S->P->h->device);
    cudaStreamSynchronize(S->P->h->stream);
    delete S;
    return CPDLP_OK;
}

int cpdlp_state_solve(cpdlp_handle* h, cpdlp_state* s, cpdlp_stats* stats) {
    NEED(h);
    if (!s) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        StateBase* S = reinterpret_cast<StateBase*>(s);
        S->solve();
        if (stats) S->stats(stats);
    });
}

int cpdlp_state_solve_blocks(cpdlp_handle* h, cpdlp_state* s, int64_t max_blocks,
                             cpdlp_stats* stats) {
    NEED(h);
    if (!s || max_blocks < 0) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        StateBase* S = reinterpret_cast<StateBase*>(s);
        S->solve_blocks(max_blocks);
        if (stats) S->stats(stats);
    });
}

int cpdlp_state_profile(cpdlp_handle* h, cpdlp_state* s, int32_t reps, double* ms) {
    NEED(h);
    if (!s || !ms || reps <= 0) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { reinterpret_cast<StateBase*>(s)->profile(reps, ms); });
}

int cpdlp_state_kernel_bytes(const cpdlp_state* s, double* bytes) {
    if (!s || !bytes) return CPDLP_ERR_ARGUMENT;
    reinterpret_cast<const StateBase*>(s)->kernel_bytes(bytes);
    return CPDLP_OK;
}

int cpdlp_state_step(cpdlp_handle* h, cpdlp_state* s, int64_t count) {
    NEED(h);
    if (!s || count < 0) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { reinterpret_cast<StateBase*>(s)->step(count); });
}

int cpdlp_state_kkt(cpdlp_handle* h, cpdlp_state* s, int32_t which, cpdlp_kkt_errors* err) {
    NEED(h);
    if (!s || !err || which < 0 || which > CPDLP_VEC_SOL_RESTART) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { reinterpret_cast<StateBase*>(s)->kkt(which, err); });
}

int cpdlp_state_vectors(cpdlp_handle* h, const cpdlp_state* s, int32_t which, double* x,
                        double* y) {
    NEED(h);
    if (!s || which < 0 || which > CPDLP_VEC_SOL_RESTART) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        const_cast<StateBase*>(reinterpret_cast<const StateBase*>(s))->vectors(which, x, y);
    });
}

int cpdlp_state_solution(cpdlp_handle* h, const cpdlp_state* s, double* x, double* y) {
    NEED(h);
    if (!s) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] {
        const_cast<StateBase*>(reinterpret_cast<const StateBase*>(s))->solution(x, y);
    });
}

int cpdlp_state_stats(cpdlp_handle* h, const cpdlp_state* s, cpdlp_stats* stats) {
    NEED(h);
    if (!s || !stats) return CPDLP_ERR_ARGUMENT;
    reinterpret_cast<const StateBase*>(s)->stats(stats);
    return CPDLP_OK;
}

int cpdlp_state_history(const cpdlp_state* s, int64_t* kkt_passes, cpdlp_kkt_errors* errs,
                        int64_t capacity, int64_t* count) {
    if (!s) return CPDLP_ERR_ARGUMENT;
    const StateBase* S = reinterpret_cast<const StateBase*>(s);
    const int64_t len = (int64_t)S->hist_passes.size();
    const int64_t k = capacity < len ? capacity : len;
    for (int64_t t = 0; t < k; t++) {
        if (kkt_passes) kkt_passes[t] = S->hist_passes[(size_t)t];
        if (errs) errs[t] = S->hist_err[(size_t)t];
    }
    if (count) *count = len;
    return CPDLP_OK;
}

int cpdlp_reduced_costs(cpdlp_handle* h, const cpdlp_lp* lp, const double* y, double* z_out,
                        double* dual_objective) {
    NEED(h);
    return guarded(h, [&] { reduced_costs(*H(h), lp, y, z_out, dual_objective); });
}

int cpdlp_problem_layout(const cpdlp_problem* p, int32_t* format, int32_t* tile_nnz,
                         int64_t* width) {
    if (!p) return CPDLP_ERR_ARGUMENT;
    const ProblemBase* P = reinterpret_cast<const ProblemBase*>(p);
    for (int sd = 0; sd < 2; sd++) {
        const bool ell = P->fmt[sd] == CPDLP_FMT_ELL;
        if (format) format[sd] = P->fmt[sd];
        if (tile_nnz) tile_nnz[sd] = ell ? 0 : (sd == 0 ? P->planA : P->planAt).tile_nnz();
        if (width) width[sd] = ell ? P->ell_width[sd] : 0;
    }
    return CPDLP_OK;
}

int cpdlp_problem_order(cpdlp_handle* h, const cpdlp_problem* p, int32_t* ordered,
                        int64_t* order_row, int64_t* order_col) {
    NEED(h);
    if (!p) return CPDLP_ERR_ARGUMENT;
    const ProblemBase* P = reinterpret_cast<const ProblemBase*>(p);
    if (ordered) *ordered = P->ordered ? 1 : 0;
    if (!P->ordered) return CPDLP_OK;
    return guarded(h, [&] {
        for (int sd = 0; sd < 2; sd++) {
            int64_t* out = sd == 0 ? order_row : order_col;
            const int64_t len = sd == 0 ? P->m : P->n;
            if (!out || len <= 0) continue;
            std::vector<int32_t> o((size_t)len);
            CK(cudaMemcpyAsync(o.data(), (sd == 0 ? P->order_row : P->order_col).p,
                               sizeof(int32_t) * len, cudaMemcpyDeviceToHost, H(h)->stream));
            CK(cudaStreamSynchronize(H(h)->stream));
            for (int64_t k = 0; k < len; k++) out[k] = (int64_t)o[(size_t)k] + 1;
        }
    });
}

int cpdlp_solve_history(const cpdlp_handle* h, int64_t* kkt_passes, cpdlp_kkt_errors* errs,
                        int64_t capacity, int64_t* count) {
    if (!h) return CPDLP_ERR_ARGUMENT;
    const Handle& H0 = *static_cast<const Handle*>(h);
    const int64_t len = (int64_t)H0.solve_hist_passes.size();
    const int64_t k = capacity < len ? capacity : len;
    for (int64_t t = 0; t < k; t++) {
        if (kkt_passes) kkt_passes[t] = H0.solve_hist_passes[(size_t)t];
        if (errs) errs[t] = H0.solve_hist_err[(size_t)t];
    }
    if (count) *count = len;
    return CPDLP_OK;
}

int cpdlp_solve(cpdlp_handle* h, const cpdlp_lp* lp, const cpdlp_params* params,
                const double* x0, const double* y0, double* x_out, double* y_out,
                cpdlp_stats* stats) {
    NEED(h);
    return guarded(h, [&] { solve_full(*H(h), lp, params, x0, y0, x_out, y_out, stats); });
}

int cpdlp_batch_solve(cpdlp_handle* h, int64_t count, const cpdlp_lp* lps,
                      const cpdlp_params* params, double* const* x_out, double* const* y_out,
                      cpdlp_stats* stats) {
    NEED(h);
    if (count < 0 || (count > 0 && (!lps || !params))) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { batch_solve(*H(h), count, lps, params, x_out, y_out, stats); });
}

int cpdlp_submit(cpdlp_handle* h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 const double* reltol, const double* const* x0, const double* const* y0,
                 int64_t max_ctas, cpdlp_job** out) {
    NEED(h);
    if (!out) return CPDLP_ERR_ARGUMENT;
    *out = nullptr;
    return guarded(h, [&] {
        *out = reinterpret_cast<cpdlp_job*>(
            job_submit(*H(h), count, lps, params, reltol, x0, y0, max_ctas));
    });
}

int cpdlp_poll(cpdlp_handle* h, cpdlp_job* job, int32_t* done) {
    NEED(h);
    if (!job || !done) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { *done = job_poll(reinterpret_cast<Job*>(job)) ? 1 : 0; });
}

int cpdlp_wait(cpdlp_handle* h, cpdlp_job* job) {
    NEED(h);
    if (!job) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { job_wait(reinterpret_cast<Job*>(job)); });
}

int cpdlp_cancel(cpdlp_handle* h, cpdlp_job* job) {
    NEED(h);
    if (!job) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { job_cancel(reinterpret_cast<Job*>(job)); });
}

int cpdlp_collect(cpdlp_handle* h, cpdlp_job* job, double* const* x_out, double* const* y_out,
                  cpdlp_stats* stats) {
    NEED(h);
    if (!job) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { job_collect(reinterpret_cast<Job*>(job), x_out, y_out, stats); });
}

int cpdlp_job_ready(cpdlp_handle* h, const cpdlp_job* job, int32_t* ready) {
    NEED(h);
    if (!job || !ready) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { job_ready(reinterpret_cast<const Job*>(job), ready); });
}

int cpdlp_collect_lp(cpdlp_handle* h, cpdlp_job* job, int64_t k, double* x_out, double* y_out,
                     cpdlp_stats* stats) {
    NEED(h);
    if (!job) return CPDLP_ERR_ARGUMENT;
    return guarded(h, [&] { job_collect_lp(reinterpret_cast<Job*>(job), k, x_out, y_out, stats); });
}

int64_t cpdlp_job_count(const cpdlp_job* job) {
    return job ? job_count(reinterpret_cast<const Job*>(job)) : -1;
}

int cpdlp_job_destroy(cpdlp_job* job) {
    if (!job) return CPDLP_ERR_ARGUMENT;
    job_destroy(reinterpret_cast<Job*>(job));
    return CPDLP_OK;
}

int64_t cpdlp_batch_footprint(int64_t count, const cpdlp_lp* lps, const cpdlp_params* params) {
    if (count < 0 || (count > 0 && !lps)) return -1;
    return batch_footprint(count, lps, params);
}

}  // extern "C"
