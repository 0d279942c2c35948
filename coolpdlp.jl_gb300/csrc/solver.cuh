// solver.cuh -- single-LP PDLP / PDHG on the device.
#pragma once

#include <type_traits>

#include "cpdlp_common.cuh"
#include "sparse_build.cuh"
#include "tiles.cuh"

namespace cpdlp {

// Scalars of one step, in the iterate type T (pdlp.jl:108, :126-136).
// FP32 iterates whose relative KKT error has not halved over this many checks
// continue in FP64 (cpdlp_solve with refine_reltol > 0, and the batched solver)
constexpr int64_t FP32_STALL_CHECKS = 30;
// The single-LP rule also asks that the error be at most this (PDLP's error
// is noisy and can plateau for thousands of iterations far from a solution,
// where FP32 rounding is not what holds it back; FP32 iterates commonly reach
// 1e-6 to 1e-7), or that no halving came for FP32_STALL_LONG times as many
// checks
constexpr double FP32_STALL_REL = 1e-5;
constexpr int64_t FP32_STALL_LONG = 10;
// With FP32 iterates the power method also stops once its residual is below
// this fraction of theta.  The Rayleigh quotient's error is at most about the
// residual (eigenvalues clustered within it) and usually its square, and the
// step size 0.9/|A| leaves a 10% margin, so 1% is safe for PDHG's step rule.
constexpr double POWER_RTOL_F32 = 1e-2;

template <class T>
struct StepCoef {
    T tau, sigma, inv_sigma, a, b;
};

// A preprocessed LP resident on the device (the MILP after preprocess,
// common.jl:154-169).  The CSR of A (rows of A) and of A' (rows of A') hold
// A's and A''s scaled values respectively, as the reference scales its two
// CSC copies separately (preconditioning.jl:37-43).
struct ProblemBase {
    virtual ~ProblemBase() = default;
    Handle* h = nullptr;
    int32_t vt = CPDLP_VAL_F64;   // iterate / matrix value type
    int64_t m = 0, n = 0, nnz = 0;
    DBuf<int32_t> a_ptr, a_idx, at_ptr, at_idx;
    TilePlan planA, planAt;
    // product format per matrix ([0]: rows of A, [1]: rows of A'): CSR tiles
    // or ELL (ell_idx rows x width column-major, 0-based; the values in
    // ProblemT::ell_val; the CSR row pointer gives the row lengths)
    int32_t fmt[2] = {CPDLP_FMT_CSR, CPDLP_FMT_CSR};
    int64_t ell_width[2] = {0, 0};
    DBuf<int32_t> ell_idx[2];
    DBuf<double> D1, D2, invD1, invD2;
    double primal_scale = 0, dual_scale = 0;
    bool zero_cost = false;
    cpdlp_params prm{};
    double setup_seconds = 0;
    // reduction scratch (FP64 block partials) sized for NVEC = 4
    DBuf<double> red_rows, red_cols, red_out;
    int64_t rows_A_partials = 0, rows_At_partials = 0;
    // block-partial rows of the KKT pass (kkt_warps<T>() per block): one
    // iterate, and four packed iterates (grid capped at kkt4_cap blocks)
    int64_t rows_A_kkt = 0, rows_At_kkt = 0;
    int64_t kkt4_cap = 0, rows_A_kkt4 = 0, rows_At_kkt4 = 0;
    // density order (CPDLP_TILE_DENSITY_ORDER or the autotuner's choice):
    // internal row i is the caller's row order_row[i], internal column j the
    // caller's column order_col[j]; vectors cross the C ABI in the caller's
    // order (order_to_internal / order_to_user)
    bool ordered = false;
    DBuf<int32_t> order_row, order_col;
};

void order_to_internal(const ProblemBase& P, int side, double* v, cudaStream_t s);
void order_to_user(const ProblemBase& P, int side, double* v, cudaStream_t s);

template <class T>
struct ProblemT : ProblemBase {
    DBuf<T> a_val, at_val;
    DBuf<T> ell_val[2];   // ELL values of a matrix whose fmt is CPDLP_FMT_ELL
    DBuf<T> c, lv, uv, lc, uc;
    DBuf<T> partA, partAt;   // long-row piece partials, NVEC = 4
    // narrow +-1 storage: the index arrays carry the signs of A (Pm1), the
    // value arrays are empty, and the products apply d1 / d2 (as T)
    bool pm1 = false;
    DBuf<T> d1t, d2t;
    // 1 ./ D1 and 1 ./ D2 in T for the KKT terms (FP32 problems keep a copy;
    // FP64 problems use invD1 / invD2 themselves)
    DBuf<T> invD1t, invD2t;
    const T* invD1_T() const {
        if constexpr (std::is_same<T, double>::value) return invD1.p;
        else return invD1t.p;
    }
    const T* invD2_T() const {
        if constexpr (std::is_same<T, double>::value) return invD2.p;
        else return invD2t.p;
    }
};

struct StateBase {
    virtual ~StateBase() = default;
    ProblemBase* P = nullptr;
    cpdlp_params prm{};
    double eta = 0, eta_sum = 0, omega = 1;
    int64_t outer = 0, inner = 0, total = 0, kkt_passes = 0;
    int32_t status = CPDLP_STILL_RUNNING;
    int32_t restart_from_avg = 0;
    cpdlp_kkt_errors err{}, err_cand{}, err_cand_last{}, err_restart{};
    // PDLP: errors of the average at the last check, and whether that check
    // restarted (which moved the chosen candidate into sol and reset the average)
    cpdlp_kkt_errors err_avg{};
    bool restarted_at_check = false;
    bool err_restart_valid = false;
    double starting_time = 0, time_elapsed = 0, setup_seconds = 0;
    int64_t power_iterations = 0;
    int64_t refine_passes = 0;
    int64_t launches = 0;  // kernels of this library launched by the state
    std::vector<int64_t> hist_passes;
    std::vector<cpdlp_kkt_errors> hist_err;
    virtual void step(int64_t count) = 0;
    // solve! (pdlp.jl:69-94) with at most `max_blocks` rounds of check_every
    // steps + checks; returns STILL_RUNNING when the budget runs out.
    virtual int32_t solve_blocks(int64_t max_blocks) = 0;
    int32_t solve() { return solve_blocks(INT64_MAX); }
    // mean ms per launch of the primal step, dual step and 4-vector KKT kernels
    virtual void profile(int reps, double* ms) = 0;
    // algorithmic bytes per launch of the same three kernels
    virtual void kernel_bytes(double* bytes) const = 0;
    virtual void kkt(int which, cpdlp_kkt_errors* e) = 0;
    virtual void vectors(int which, double* x, double* y) = 0;
    virtual void solution(double* x, double* y) = 0;
    virtual void early_exit_zero_problem() = 0;
    void stats(cpdlp_stats* st) const;
};

// plans = false: scaling and device arrays only, no tile plans, reduction
// scratch or constant scales (the batched solver builds its own plans)
ProblemBase* problem_create(Handle& h, const cpdlp_lp* lp, const cpdlp_params* prm,
                            bool plans = true);
// eta0 > 0 / omega0 > 0 continue an earlier solve of the same LP: the step size
// (no power method) and the primal weight start from these values
StateBase* state_create(Handle& h, ProblemBase* P, const cpdlp_params* prm, const double* x0,
                        const double* y0, double eta0 = 0.0, double omega0 = 0.0);
double problem_spectral_norm(Handle& h, ProblemBase* P, const cpdlp_params* prm, int64_t* iters);

// solve(milp, sol, algo) (common.jl:186-209) on the device, plus mixed
// precision: with FP32 iterates and 0 < refine_reltol < termination_reltol the
// FP32 phase runs on towards refine_reltol until its error stalls; from there
// (or from an FP32 phase that stalls above termination_reltol) refinement
// rounds solve the residual LP of the FP64 point with FP32 iterates and add
// the correction in FP64, and PDLP continues in FP64 if a round makes no
// progress.  x_out (n) / y_out (m) may be null.
void solve_full(Handle& h, const cpdlp_lp* lp, const cpdlp_params* params, const double* x0,
                const double* y0, double* x_out, double* y_out, cpdlp_stats* stats);
void problem_scaling(Handle& h, ProblemBase* P, double* d1, double* d2);

}  // namespace cpdlp
