// matrix.cuh -- GPUSparseMatrixCSR / ELL / COO on the device.
#pragma once

#include "cpdlp_common.cuh"
#include "sparse_build.cuh"
#include "tiles.cuh"

namespace cpdlp {

// Storage per format (device, int32 indices):
//  CSR: ptr = rowptr (m+1, 0-based), idx = colval (0-based), values; tile plan
//  ELL: idx = colval (m*width, column-major, 1-based, 0 = padding), values
//  COO: ptr = rowval (0-based), idx = colval (0-based), values, findnz order
struct Matrix {
    Handle* h = nullptr;
    int32_t format = CPDLP_FMT_CSR;
    int32_t vt = CPDLP_VAL_F64;
    int64_t m = 0, n = 0, nnz = 0, width = 0;
    DBuf<int32_t> ptr, idx;
    DBuf<double> vd;
    DBuf<float> vf;
    TilePlan plan;
    DBuf<unsigned char> part;  // long-row partials (bytes)
};

Matrix* matrix_from_csc(Handle& h, int64_t m, int64_t n, int64_t nnz, const int64_t* colptr,
                        const int64_t* rowval, const double* nzval, int32_t format, int32_t vt);
void matrix_spmv(Handle& h, const Matrix& M, const void* b, void* c, double alpha, double beta);
void matrix_export(Handle& h, const Matrix& M, int64_t* ptr, int64_t* idx, double* val);

}  // namespace cpdlp
