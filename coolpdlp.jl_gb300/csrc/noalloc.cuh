// noalloc.cuh -- CSR mul! on caller-owned device arrays without allocation.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

// See noalloc.cu: scratch in a fixed file-scope device array, at most
// 33,554,432 nonzeros; blocks until the product is done; calls overlapping on
// the GPU race on that array and on the shared validation flag.
void spmv_csr_noalloc(Handle& h, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr1,
                      const int32_t* colval1, const void* nzval, int32_t value_type,
                      const void* b, void* c, double alpha, double beta);

}  // namespace cpdlp
