// permutation.cuh -- sort_rows_columns (src/components/permutation.jl:1-46), host code.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

// Every output may be null (not computed).  Permutations are 1-based.
void sort_rows_columns(const cpdlp_lp& lp, int64_t* perm_var, int64_t* perm_cons,
                       int64_t* colptr_out, int64_t* rowval_out, double* nzval_out, double* c_out,
                       double* lv_out, double* uv_out, double* lc_out, double* uc_out);

}  // namespace cpdlp
