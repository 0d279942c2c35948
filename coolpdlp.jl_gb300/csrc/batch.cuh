// batch.cuh -- many independent LPs per call.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

void batch_solve(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 double* const* x_out, double* const* y_out, cpdlp_stats* stats);

}  // namespace cpdlp
