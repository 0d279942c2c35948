/*
 * coolpdlp_cuda.h -- C ABI of libcoolpdlp_cuda, the GB300 (sm_103a) PDLP/PDHG solver.
 *
 * Every entry point is plain C: pointers, sizes and status codes, no C++ or
 * torch types.  A Julia package binds it with `ccall`, Python with `ctypes`.
 * Each declaration names the CoolPDLP.jl interface it replaces (paths are
 * relative to the CoolPDLP.jl source tree).
 *
 * Conventions
 *  - Every call returns an int status: CPDLP_OK (0) or a CPDLP_ERR_* code.
 *    The message of the last failure on a handle is cpdlp_last_error(h).
 *    CPDLP_ERR_DIMENSION maps to Julia's DimensionMismatch, CPDLP_ERR_ARGUMENT
 *    to ArgumentError (src/problems/milp.jl:72-90, src/utils/device.jl:9).
 *  - Solver outcomes (OPTIMAL, TIME_LIMIT, ITERATION_LIMIT) are statuses in
 *    cpdlp_stats, never errors (src/components/termination.jl:13).
 *  - Index arrays cross the ABI 1-based, in Julia's SparseMatrixCSC layout, so
 *    that exported CSR/ELL/COO indices compare bit-for-bit with the Julia ones.
 *  - Host arrays belong to the caller and are copied in.  Device buffers made
 *    by the library belong to the handle (or the object) and are freed by the
 *    matching *_destroy call.  Pointers documented as "device" are CUDA device
 *    pointers owned by the caller.
 *  - A handle owns one CUDA stream; use one handle per host thread.
 *  - Missing bounds are +-INFINITY, as in the reference.
 */
#ifndef COOLPDLP_CUDA_H
#define COOLPDLP_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPDLP_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    CPDLP_OK = 0,
    CPDLP_ERR_ARGUMENT = 1,      /* ArgumentError: bad pointer, bad CSC, bad enum */
    CPDLP_ERR_DIMENSION = 2,     /* DimensionMismatch */
    CPDLP_ERR_CUDA = 3,          /* a CUDA runtime call failed */
    CPDLP_ERR_OUT_OF_MEMORY = 4, /* device allocation failed or admission refused */
    CPDLP_ERR_TIMEOUT = 5,       /* a bounded device wait ran out */
    CPDLP_ERR_NOT_FOUND = 6,     /* unknown ticket / object */
    CPDLP_ERR_UNSUPPORTED = 7    /* size or feature outside what this build handles */
};

/* ---- enums mirrored from the reference ---------------------------------- */
/* TerminationStatus, same order as src/components/termination.jl:13 */
enum {
    CPDLP_OPTIMAL = 0,
    CPDLP_TIME_LIMIT = 1,
    CPDLP_ITERATION_LIMIT = 2,
    CPDLP_STILL_RUNNING = 3,
    /* EXT (infeasibility_tol > 0; the reference has no detection): */
    CPDLP_PRIMAL_INFEASIBLE = 4, /* a dual ray certifies that no x is feasible */
    CPDLP_DUAL_INFEASIBLE = 5    /* a primal ray certifies that the objective is unbounded */
};

/* Algorithm{:PDLP} / Algorithm{:PDHG} (src/algorithms/pdlp.jl:6-11, pdhg.jl:6-16) */
enum { CPDLP_ALGO_PDLP = 0, CPDLP_ALGO_PDHG = 1 };

/* float_type of ConversionParameters (src/components/conversion.jl:14-30).
 * CPDLP_VAL_PM1 (matrices only): values that are all exactly +-1, stored as
 * the signs of the column indices (no value array, FP32 vectors, CSR). */
enum { CPDLP_VAL_F64 = 0, CPDLP_VAL_F32 = 1, CPDLP_VAL_PM1 = 2 };

/* matrix_type: GPUSparseMatrixCSR / ELL / COO (src/utils/mat_*.jl).
 * CPDLP_FMT_AUTO (solver parameter only, EXT): the autotuner picks the
 * product format of each matrix of the solve by timing. */
enum { CPDLP_FMT_AUTO = -1, CPDLP_FMT_CSR = 0, CPDLP_FMT_ELL = 1, CPDLP_FMT_COO = 2 };

/* which iterate to read back from a solver state (src/algorithms/pdlp.jl:20-43) */
enum {
    CPDLP_VEC_SOL = 0,
    CPDLP_VEC_SOL_LAST = 1,
    CPDLP_VEC_SOL_AVG = 2,
    CPDLP_VEC_SOL_AVG_LAST = 3,
    CPDLP_VEC_SOL_RESTART = 4
};

/* ---- plain data ------------------------------------------------------- */

/* KKTErrors (src/components/errors.jl:8-21), in unscaled units. */
typedef struct cpdlp_kkt_errors {
    double primal;
    double primal_scale;
    double dual;
    double dual_scale;
    double gap;
    double gap_scale;
} cpdlp_kkt_errors;

/* Every keyword of Algorithm{A}(T, Ti, M; ...) (src/algorithms/common.jl:53-116)
 * plus the power-method settings of spectral_norm (src/utils/linalg.jl:86-96)
 * and the extensions of this library (marked EXT).  Fill with
 * cpdlp_params_default() and override fields. */
typedef struct cpdlp_params {
    int32_t algorithm;              /* CPDLP_ALGO_* */
    int32_t float_type;             /* CPDLP_VAL_F64 or CPDLP_VAL_F32: iterate precision */
    /* preconditioning (src/components/preconditioning.jl:134-139) */
    double chambolle_pock_alpha;    /* 1.0 */
    int32_t ruiz_iter;              /* 10 (PDLP), 0 (PDHG) */
    /* step sizes (src/components/step_size.jl:8-15) */
    double invnorm_scaling;         /* 0.9 */
    double primal_weight_damping;   /* 0.5 (PDLP), NaN (PDHG) */
    double zero_tol;                /* 1e-8 */
    /* restart (src/components/restart.jl:8-15) */
    double sufficient_decay;        /* 0.2 */
    double necessary_decay;         /* 0.8 */
    double artificial_decay;        /* 0.36 */
    /* generic (src/components/generic.jl:8-15) */
    int32_t show_progress;          /* 0; progress is printed by the caller */
    int32_t check_every;            /* 100 */
    int32_t record_error_history;   /* 1 */
    /* termination (src/components/termination.jl:22-29) */
    double termination_reltol;      /* 1e-4 */
    int64_t max_kkt_passes;         /* 100000 */
    double time_limit;              /* 100.0 seconds */
    /* spectral norm power method: IterativeSolvers.powm! defaults are
     * tol = eps(T) * n^3 (Int64 arithmetic, wraps like Julia's) and
     * maxiter = n.  power_tol_override > 0 or power_maxiter_override > 0
     * replace them (EXT). */
    double power_tol_override;      /* 0 = reference default */
    int64_t power_maxiter_override; /* 0 = reference default */
    uint64_t power_seed;            /* start vector seed (EXT; the reference uses StableRNG(0)) */
    /* EXT: mixed precision for float_type CPDLP_VAL_F32 (0 = off).
     * cpdlp_solve: the FP32 run aims at the smaller of termination_reltol and
     * refine_reltol; when its relative KKT error stalls short of that (not
     * halved over 30 checks while at most 1e-5, or over 300 checks),
     * refinement rounds solve the residual LP of the FP64 point with FP32
     * iterates and add each correction in FP64 (FP64 residuals and KKT
     * errors), and PDLP continues in FP64 if a round makes no progress.
     * Batched solves and jobs continue in FP64 instead (cpdlp_batch_solve). */
    double refine_reltol;
    /* EXT: CSR tile size in nonzeros for the SpMV work partition (0 = autotune). */
    int32_t tile_nnz;
    /* EXT: storage flags (CPDLP_TILE_*); 0 = defaults. */
    int32_t tile_flags;
    /* EXT: infeasibility detection of the single-LP solve (0 = off, as in the
     * reference; 1e-8 is a typical value).  At every check the change of the
     * iterates since the previous check is tested as a certificate: a dual ray
     * y (signs projected onto the row bounds' cone) with reduced costs
     * g = -A'y, r = its part the variable bounds allow, and positive ray
     * objective b(y, r) proves primal infeasibility when |g - r| <=
     * infeasibility_tol * b(y, r); a primal ray x (projected onto the bounds'
     * recession cone) with c'x < 0 proves unboundedness when the distance of
     * A x to the row bounds' recession cone is <= infeasibility_tol * |c'x|.
     * Both tests run in the scaled problem, where they are equivalent. */
    double infeasibility_tol;
    /* matrix_type M of Algorithm{A}(T, Ti, M) (src/components/conversion.jl:
     * 37-55, src/problems/modify.jl:80-105): the product format of the
     * single-LP solve's matrices A and A'.  CPDLP_FMT_CSR: the CSR tile
     * engine (tile shape autotuned for large matrices); CPDLP_FMT_ELL: the
     * reference's ELL layout (column-major, width = the longest row), one
     * thread per row, each row summed in column order; CPDLP_FMT_COO: solved
     * on the CSR engine (the reference's COO product accumulates with atomics
     * in a run-dependent order; CSR sums each row in COO's column order);
     * CPDLP_FMT_AUTO (default, EXT): for matrices of at least 2^21 nonzeros
     * the autotuner times CSR tile shapes and ELL (when its padding is at
     * most 3x the nonzeros) and keeps the fastest per matrix, otherwise CSR.
     * Batched solves and jobs use the CSR engine. */
    int32_t matrix_type;
} cpdlp_params;

/* tile_flags bits.  By default a single-LP solve with FP32 iterates whose
 * matrix values are all exactly +-1 stores the matrix narrow: the signs ride
 * in the column indices (4 bytes per nonzero, no value array) and the kernels
 * apply the diagonal scalings D1, D2 themselves.  CPDLP_TILE_NO_NARROW keeps
 * the scaled values instead.
 * Density order (EXT): CPDLP_TILE_DENSITY_ORDER renumbers the rows and the
 * columns of a single-LP solve's matrices by increasing length, ties in index
 * order -- the order of the reference's sort_rows_columns
 * (src/components/permutation.jl:1-46) -- while every row keeps its entries in
 * their input order, so each row's products and sum are the ones of the
 * unordered problem.  The gathers of the many-times-referenced long rows'
 * entries then share cache lines.  CPDLP_TILE_NO_DENSITY_ORDER never
 * reorders.  With neither, the autotuner (matrix_type CPDLP_FMT_AUTO, at
 * least 2^21 nonzeros, CSR chosen for both matrices) times both fused step
 * kernels in each order and keeps the density order when it is at least 3%
 * faster.  Every vector crossing the ABI (starting points, iterates,
 * solutions, scalings) is in the caller's order either way;
 * cpdlp_problem_order reports the choice. */
enum {
    CPDLP_TILE_NO_NARROW = 1,
    CPDLP_TILE_DENSITY_ORDER = 2,
    CPDLP_TILE_NO_DENSITY_ORDER = 4
};

/* An LP in the reference's "cuPDLPx form" (src/problems/milp.jl:1-20):
 *   min c'x  s.t.  lv <= x <= uv,  lc <= A x <= uc
 * A is m x n in Julia SparseMatrixCSC layout: 1-based colptr (n+1), 1-based
 * rowval (nnz), rows strictly ascending inside each column. */
typedef struct cpdlp_lp {
    int64_t m;
    int64_t n;
    int64_t nnz;
    const int64_t* colptr;
    const int64_t* rowval;
    const double* nzval;
    const double* c;
    const double* lv;
    const double* uv;
    const double* lc;
    const double* uc;
} cpdlp_lp;

/* ConvergenceStats (src/components/termination.jl:44-76) + IterationCounter
 * (src/components/iteration.jl) + StepSizes (src/components/step_size.jl:49-56). */
typedef struct cpdlp_stats {
    cpdlp_kkt_errors err;
    double time_elapsed;
    int64_t kkt_passes;
    int32_t termination_status;     /* CPDLP_OPTIMAL ... */
    int32_t restart_from_avg;
    int64_t outer;
    int64_t inner;
    int64_t total;
    double eta;
    double eta_sum;
    double omega;
    int64_t history_length;         /* entries in the error history */
    int64_t power_iterations;       /* EXT: power-method iterations run */
    int64_t refine_kkt_passes;      /* EXT: passes spent in FP64 refinement */
    double setup_seconds;           /* EXT: preprocess + initialize wall time */
    int64_t kernel_launches;        /* EXT: this library's kernels launched by the state */
} cpdlp_stats;

typedef struct cpdlp_handle cpdlp_handle;
typedef struct cpdlp_matrix cpdlp_matrix;
typedef struct cpdlp_problem cpdlp_problem;
typedef struct cpdlp_state cpdlp_state;
typedef struct cpdlp_job cpdlp_job;

/* ---- library & handle ----------------------------------------------------- */
int cpdlp_abi_version(void);

/* Default keywords of Algorithm{:PDLP} (src/algorithms/common.jl:53-116) or of
 * PDHG() (src/algorithms/pdhg.jl:6-16, which sets ruiz_iter = 0 and NaN
 * restart/weight parameters). */
void cpdlp_params_default(cpdlp_params* params, int32_t algorithm);

/* Backend selection: the KernelAbstractions backend object of the reference
 * (src/components/conversion.jl:14-30); `device` is a CUDA ordinal. */
int cpdlp_create(int32_t device, cpdlp_handle** out);
int cpdlp_destroy(cpdlp_handle* h);
const char* cpdlp_last_error(const cpdlp_handle* h);
int cpdlp_synchronize(cpdlp_handle* h);
/* The handle's CUDA stream (cudaStream_t), for callers that order their own work after ours. */
void* cpdlp_stream(cpdlp_handle* h);

/* ---- pluggable sparse matrices (src/utils/mat_csr.jl, mat_ell.jl, mat_coo.jl) ---- */

/* M(::SparseMatrixCSC): GPUSparseMatrixCSR (mat_csr.jl:58-61),
 * GPUSparseMatrixELL (mat_ell.jl:54-70), GPUSparseMatrixCOO (mat_coo.jl:50-53).
 * The format is built on the device from the 1-based CSC arrays.
 * value_type: CPDLP_VAL_F64 or CPDLP_VAL_F32 (the matrix eltype T), or
 * CPDLP_VAL_PM1 (CSR only, every value exactly +-1, Float32 vectors; the
 * export decodes the signs back into nzval). */
int cpdlp_matrix_from_csc(cpdlp_handle* h, int64_t m, int64_t n, int64_t nnz,
                          const int64_t* colptr, const int64_t* rowval,
                          const double* nzval, int32_t format, int32_t value_type,
                          cpdlp_matrix** out);
int cpdlp_matrix_destroy(cpdlp_matrix* A);

/* size(A), nnz(A) (mat_*.jl: size / SparseArrays.nnz) and the ELL width d. */
int cpdlp_matrix_shape(const cpdlp_matrix* A, int64_t* m, int64_t* n, int64_t* nnz,
                       int64_t* width);

/* Copy the stored arrays to host, 1-based, exactly as the Julia struct fields:
 *  CSR: ptr = rowptr (m+1), idx = colval (nnz), val = nzval (nnz)
 *  ELL: ptr unused, idx = colval (m*d, column-major, 0 = padding), val = nzval (m*d)
 *  COO: ptr = rowval (nnz), idx = colval (nnz), val = nzval (nnz)
 * Values are widened to double. */
int cpdlp_matrix_export(cpdlp_handle* h, const cpdlp_matrix* A, int64_t* ptr,
                        int64_t* idx, double* val);

/* LinearAlgebra.mul!(c, A, b, alpha, beta) (mat_csr.jl:81-92, mat_ell.jl:91-102,
 * mat_coo.jl:68-80): c = alpha*A*b + beta*c with b, c DEVICE vectors of the
 * matrix eltype.  beta == 0 is a strong zero: c is not read. */
int cpdlp_spmv(cpdlp_handle* h, const cpdlp_matrix* A, const void* b, void* c,
               double alpha, double beta);

/* sort_rows_columns(milp) (src/components/permutation.jl:1-46): the LP with
 * its variables ordered by increasing column length and its constraints by
 * increasing row length (stable: ties keep their index order, as Julia's
 * sortperm).  perm_var (n) / perm_cons (m) receive the 1-based permutations
 * (new position k holds old index perm[k]); colptr (n+1), rowval (nnz), nzval
 * (nnz) the permuted CSC A[perm_cons, perm_var], rows ascending per column;
 * c, lv, uv (n) and lc, uc (m) the permuted vectors.  Every output may be NULL.
 * Host computation (the reference runs it on the CPU and solve never calls
 * it); h may be NULL, and then only the status code reports an error. */
int cpdlp_sort_rows_columns(cpdlp_handle* h, const cpdlp_lp* lp, int64_t* perm_var,
                            int64_t* perm_cons, int64_t* colptr, int64_t* rowval,
                            double* nzval, double* c, double* lv, double* uv, double* lc,
                            double* uc);

/* ---- solve path (src/algorithms/common.jl, pdlp.jl, pdhg.jl) ----------- */

/* preprocess(milp, sol, algo) (common.jl:154-169): Ruiz + Pock-Chambolle
 * scaling, conversion to params->float_type and the CSR builds of A and A',
 * all on the device. */
int cpdlp_problem_create(cpdlp_handle* h, const cpdlp_lp* lp, const cpdlp_params* params,
                         cpdlp_problem** out);
int cpdlp_problem_destroy(cpdlp_problem* p);
/* The cumulative preconditioner D1 (m) and D2 (n) of the scaled MILP
 * (preconditioning.jl:61-91). */
int cpdlp_problem_scaling(cpdlp_handle* h, const cpdlp_problem* p, double* d1, double* d2);

/* initialize(milp, sol, algo) (pdlp.jl:45-67, pdhg.jl:40-54): the starting
 * point x0 (n), y0 (m) is in the ORIGINAL units (NULL = zeros) and is
 * preconditioned like precondition(sol, prec) (preconditioning.jl:45-51);
 * runs the power method for the fixed step size. */
int cpdlp_state_create(cpdlp_handle* h, cpdlp_problem* p, const cpdlp_params* params,
                       const double* x0, const double* y0, cpdlp_state** out);
int cpdlp_state_destroy(cpdlp_state* s);

/* solve!(state, milp, algo) (pdlp.jl:69-94, pdhg.jl:56-74). */
int cpdlp_state_solve(cpdlp_handle* h, cpdlp_state* s, cpdlp_stats* stats);

/* solve! with a budget (EXT): at most `max_blocks` rounds of (check_every
 * steps + termination check + restart check) of pdlp.jl:75-91; returns with
 * termination_status CPDLP_STILL_RUNNING when the budget ran out, and a later
 * call continues where this one stopped. */
int cpdlp_state_solve_blocks(cpdlp_handle* h, cpdlp_state* s, int64_t max_blocks,
                             cpdlp_stats* stats);

/* EXT, measurement: mean milliseconds per launch, over `reps` launches timed
 * with CUDA events on the handle's stream, of ms[0] the fused primal step
 * kernel, ms[1] the fused dual step kernel, ms[2] the four-iterate KKT pass.
 * Outputs go to scratch buffers: the state is unchanged. */
int cpdlp_state_profile(cpdlp_handle* h, cpdlp_state* s, int32_t reps, double* ms);

/* EXT, measurement: algorithmic bytes moved by one launch of the same three
 * kernels (each matrix array and vector read or written once). */
int cpdlp_state_kernel_bytes(const cpdlp_state* s, double* bytes);

/* `count` calls of step!(state, milp) (pdlp.jl:96-124, pdhg.jl:76-102)
 * with no termination or restart check in between. */
int cpdlp_state_step(cpdlp_handle* h, cpdlp_state* s, int64_t count);

/* kkt_errors!(scratch, sol, milp) (errors.jl:65-109) of one stored iterate. */
int cpdlp_state_kkt(cpdlp_handle* h, cpdlp_state* s, int32_t which, cpdlp_kkt_errors* err);

/* Stored iterates in the SCALED units of the preconditioned problem, widened to
 * double (x: n, y: m). */
int cpdlp_state_vectors(cpdlp_handle* h, const cpdlp_state* s, int32_t which, double* x,
                        double* y);

/* get_solution(state, milp) (common.jl:233-235): the current iterate,
 * unpreconditioned, in double. */
int cpdlp_state_solution(cpdlp_handle* h, const cpdlp_state* s, double* x, double* y);

/* Current stats without solving. */
int cpdlp_state_stats(cpdlp_handle* h, const cpdlp_state* s, cpdlp_stats* stats);

/* stats.error_history (termination.jl:44-76, pushed at common.jl:226-228):
 * copies up to `capacity` entries, `count` receives the full length. */
int cpdlp_state_history(const cpdlp_state* s, int64_t* kkt_passes, cpdlp_kkt_errors* errs,
                        int64_t capacity, int64_t* count);

/* solve(milp, sol, algo) (common.jl:186-209): preprocess, initialize, the
 * empty-problem early exit, solve!, get_solution.  x0/y0 may be NULL (zeros);
 * x_out (n) and y_out (m) receive the unpreconditioned solution. */
int cpdlp_solve(cpdlp_handle* h, const cpdlp_lp* lp, const cpdlp_params* params,
                const double* x0, const double* y0, double* x_out, double* y_out,
                cpdlp_stats* stats);

/* stats.error_history (termination.jl:44-76, pushed at common.jl:226-228) of
 * the last cpdlp_solve on this handle: copies up to `capacity` entries,
 * `count` receives the full length.  With mixed precision (FP32 iterates and
 * refine_reltol > 0) it holds every phase in order, passes counted from the
 * start of the solve: the FP32 run's checks, the combined point's errors at
 * every check of the refinement rounds plus the final refined point, then the
 * FP64 continuation's checks if one ran (and the returned point's errors if
 * the continuation ended worse than it).  Empty when record_error_history is
 * 0 or the problem took the empty-problem early exit (common.jl:194-198). */
int cpdlp_solve_history(const cpdlp_handle* h, int64_t* kkt_passes, cpdlp_kkt_errors* errs,
                        int64_t capacity, int64_t* count);

/* The product layout the solve of this problem uses, per matrix ([0]: rows
 * of A, the dual step; [1]: rows of A', the primal step): format
 * (CPDLP_FMT_CSR or CPDLP_FMT_ELL), CSR tile size in nonzeros (0 for ELL)
 * and ELL width (0 for CSR).  Any pointer may be NULL.  EXT (measurement). */
int cpdlp_problem_layout(const cpdlp_problem* p, int32_t* format, int32_t* tile_nnz,
                         int64_t* width);

/* Whether the solve of this problem runs in density order
 * (CPDLP_TILE_DENSITY_ORDER); *ordered = 1 or 0.  With order_row (m) and
 * order_col (n) non-NULL and the order applied, they receive the 1-based
 * orders: internal row i is the caller's row order_row[i], as the perm_cons
 * and perm_var of cpdlp_sort_rows_columns.  EXT (measurement). */
int cpdlp_problem_order(cpdlp_handle* h, const cpdlp_problem* p, int32_t* ordered,
                        int64_t* order_row, int64_t* order_col);

/* The reduced costs z = proj_multiplier.(c .- A'y, lv, uv) (n) and the dual
 * objective sum safeprod_left(lc, y+) - sum safeprod_left(uc, y-)
 * + sum safeprod_left(lv, z+) - sum safeprod_left(uv, z-) of a solution y
 * (m, original units), as MOI.optimize! computes them after solve
 * (src/moi.jl:215-227), in FP64 on the device from the LP's original data;
 * (A'y)_j runs over column j of A in row order.  z_out may be NULL. */
int cpdlp_reduced_costs(cpdlp_handle* h, const cpdlp_lp* lp, const double* y, double* z_out,
                        double* dual_objective);

/* spectral_norm(A, A') (linalg.jl:86-96) of the problem's scaled matrix in its
 * float type, with the power-method settings of `params`. */
int cpdlp_problem_spectral_norm(cpdlp_handle* h, cpdlp_problem* p, const cpdlp_params* params,
                                double* norm, int64_t* iterations);

/* c = alpha*A*b + beta*c on caller-owned DEVICE arrays of a 1-based CSR in
 * the layout of a CuArray-backed GPUSparseMatrixCSR{T,Int32}: rowptr (m+1),
 * colval (nnz), nzval (nnz, double or float per value_type), b (n), c (m).
 * beta == 0 does not read c.  No counterpart in the reference: an extra entry
 * point that allocates nothing, for callers that may not call cudaMalloc when
 * they need the product (fixed pre-reserved device budgets, host callbacks or
 * finalizers, CuArray-backed matrices that should not be copied into a
 * cpdlp_matrix).  Its scratch is a fixed 1 MiB device array of this library,
 * shared by all calls and kept until process exit: at most 33,554,432
 * nonzeros (larger inputs return CPDLP_ERR_UNSUPPORTED).  The first call on a
 * device looks up the addresses of that array and of a validation flag (under
 * CUDA's lazy module loading it is also where the array becomes resident, so
 * make it before fixing a memory budget).  Each call blocks until its
 * product is done: it reads the validation flag back on the handle's
 * stream.  Invalid indices return
 * CPDLP_ERR_ARGUMENT after the call (offending entries are skipped).  Calls
 * that overlap on the GPU race on the scratch array and on the validation
 * flag: their results can be wrong, and one call's invalid-input error can be
 * reported by, or lost to, an overlapping call. */
int cpdlp_spmv_csr_noalloc(cpdlp_handle* h, int64_t m, int64_t n, int64_t nnz,
                           const int32_t* rowptr, const int32_t* colval, const void* nzval,
                           int32_t value_type, const void* b, void* c, double alpha,
                           double beta);

/* ---- batched solve (many independent LPs in one persistent launch) -------
 * No counterpart in the reference, which solves one LP per call: this is the
 * batched form of solve(milp, algo) (common.jl:203-209) over `count` LPs.
 * x_out[k] / y_out[k] receive LP k's solution (NULL pointers skip the copy);
 * stats[k] its ConvergenceStats.  All LPs share `params`.  One CTA solves
 * one LP, so an LP's result does not depend on the other LPs of the call.
 * With float_type CPDLP_VAL_F32, an LP that reaches termination_reltol and
 * targets a smaller refine_reltol, or whose FP32 iterates stall (error not
 * halved over 30 checks), continues in FP64 warm-started from its FP32
 * solution (as cpdlp_solve does for one LP).  The power method runs in FP64
 * for both iterate types.  infeasibility_tol is not applied to batched LPs
 * (they run into their limits, as in the reference). */
int cpdlp_batch_solve(cpdlp_handle* h, int64_t count, const cpdlp_lp* lps,
                      const cpdlp_params* params, double* const* x_out,
                      double* const* y_out, cpdlp_stats* stats);

/* ---- asynchronous jobs (continuous batching) -------------------------------
 * No counterpart in the reference.  cpdlp_submit copies the LPs (the caller
 * may free them on return), preprocesses them on the job's own CUDA stream,
 * launches the persistent solve kernel and returns without waiting for it;
 * jobs submitted while others run share the GPU (the CTAs of a finishing job
 * hand their SMs to the others).  reltol: `count` target relative KKT
 * errors, or NULL for params->termination_reltol (refine_reltol for FP32 with
 * refine_reltol > 0).  With FP32 iterates, LPs whose target is below
 * termination_reltol stop there in FP32 and finish in an FP64 phase
 * warm-started from the FP32 solution.  x0 / y0: `count` warm starts in
 * original units (NULL, or NULL entries, for a cold start).  max_ctas > 0
 * caps the CTAs (concurrent LPs) of the job's launches, leaving SMs to jobs
 * submitted later; 0 fills the GPU.
 * Each LP is available as soon as its CTA finishes it: the kernel writes the
 * LP's result into mapped host memory and sets its done flag.
 * cpdlp_poll never blocks: it takes every LP finished so far, launches the
 * FP64 phase (on a new stream) for those that need it, and sets *done = 1
 * once every LP is finished.  cpdlp_job_ready fills ready[count] with 1 for
 * the LPs finished as of the last poll; cpdlp_collect_lp copies one of them.
 * cpdlp_cancel makes the job's kernels stop at their next termination check:
 * unfinished LPs report CPDLP_STILL_RUNNING.  cpdlp_collect (after done)
 * copies x / y / stats per LP like cpdlp_batch_solve.  cpdlp_job_destroy
 * waits for the job's GPU work.  A job must be destroyed before its handle.
 * cpdlp_batch_footprint: upper bound of the device bytes a job over these LPs
 * holds (admission control); -1 on invalid arguments. */
int cpdlp_submit(cpdlp_handle* h, int64_t count, const cpdlp_lp* lps,
                 const cpdlp_params* params, const double* reltol,
                 const double* const* x0, const double* const* y0, int64_t max_ctas,
                 cpdlp_job** out);
int cpdlp_poll(cpdlp_handle* h, cpdlp_job* job, int32_t* done);
int cpdlp_wait(cpdlp_handle* h, cpdlp_job* job);
int cpdlp_cancel(cpdlp_handle* h, cpdlp_job* job);
int cpdlp_collect(cpdlp_handle* h, cpdlp_job* job, double* const* x_out,
                  double* const* y_out, cpdlp_stats* stats);
int cpdlp_job_ready(cpdlp_handle* h, const cpdlp_job* job, int32_t* ready);
int cpdlp_collect_lp(cpdlp_handle* h, cpdlp_job* job, int64_t k, double* x_out,
                     double* y_out, cpdlp_stats* stats);
int64_t cpdlp_job_count(const cpdlp_job* job);
int cpdlp_job_destroy(cpdlp_job* job);
int64_t cpdlp_batch_footprint(int64_t count, const cpdlp_lp* lps, const cpdlp_params* params);

#ifdef __cplusplus
}
#endif

#endif /* COOLPDLP_CUDA_H */
