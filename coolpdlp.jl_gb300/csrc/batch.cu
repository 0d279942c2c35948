// batch.cu -- batched solve.  This first form runs the single-LP device path
// once per LP (the "one LP at a time" GPU baseline).
#include <memory>

#include "batch.cuh"
#include "solver.cuh"

namespace cpdlp {

void batch_solve(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 double* const* x_out, double* const* y_out, cpdlp_stats* stats) {
    for (int64_t k = 0; k < count; k++) {
        double t0 = now_seconds();
        std::unique_ptr<ProblemBase> P(problem_create(h, &lps[k], params));
        std::unique_ptr<StateBase> S(state_create(h, P.get(), params, nullptr, nullptr));
        S->starting_time = t0;
        if (P->m == 0 && P->zero_cost) S->early_exit_zero_problem();
        else S->solve();
        S->solution(x_out ? x_out[k] : nullptr, y_out ? y_out[k] : nullptr);
        if (stats) S->stats(&stats[k]);
    }
}

}  // namespace cpdlp
