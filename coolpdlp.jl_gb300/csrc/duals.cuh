// duals.cuh -- reduced costs and dual objective of a solution (moi.jl:215-227).
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

// z = proj_multiplier(c - A'y, lv, uv) (n) and the dual objective, FP64 on the
// device from the LP's original data.
void reduced_costs(Handle& h, const cpdlp_lp* lp, const double* y, double* z_out,
                   double* dual_objective);

}  // namespace cpdlp
