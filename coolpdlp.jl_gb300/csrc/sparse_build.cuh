// sparse_build.cuh -- device construction of the sparse formats.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

// Exclusive prefix sum of `n` int32 counts into `out` (n+1 entries, out[n] =
// total), on `stream`.  Deterministic.
void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t stream);

// Stable LSD radix sort (8-bit digits) of `n` (key, payload) pairs by key,
// keys < 2^key_bits.  Inputs are consumed (used as ping-pong space); the
// sorted pairs end in *keys/*vals (pointers may be swapped).
void radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& keys_tmp, uint32_t*& vals_tmp,
                      int64_t n, int key_bits, cudaStream_t stream);

// A CSC matrix uploaded to the device, validated, with its transpose.
//   S1 = CSC(A) = CSR(A'): ptr1 (n+1), idx1 (row of A), col1 (column of each entry)
//   S2 = CSR(A) = CSC(A'): ptr2 (m+1), idx2 (column of A), row2 (row of each entry)
//   p21[k2] = S1 position of S2 entry k2 (the permutation of sparse(transpose(A)))
//   val1: input values in S1 order (double)
struct CscPair {
    int64_t m = 0, n = 0, nnz = 0;
    DBuf<int32_t> ptr1, idx1, col1, ptr2, idx2, row2, p21;
    DBuf<double> val1;
};

// Uploads 1-based CSC host arrays, validates them on the device (monotone
// colptr, rows in range and strictly ascending inside each column) and builds
// the transpose.  Throws Error(CPDLP_ERR_ARGUMENT/DIMENSION/UNSUPPORTED).
void build_csc_pair(Handle& h, int64_t m, int64_t n, int64_t nnz, const int64_t* colptr1,
                    const int64_t* rowval1, const double* nzval, CscPair& out);

// Expands a row-pointer array into the row index of every entry.
void expand_rows(const int32_t* ptr, int64_t rows, int32_t* row_of, int64_t nnz, cudaStream_t s);

// Gathers `out[k] = in[perm[k]]`, converting the value type.
template <class TO, class TI>
void gather_values(const TI* in, const int32_t* perm, TO* out, int64_t nnz, cudaStream_t s);

// The rows of a CSR by increasing length, ties in index order (a stable sort,
// like Julia's sortperm): order[i] = the i-th row, inv[order[i]] = i.
// max_len bounds the row lengths.
void order_by_length(const int32_t* ptr, int64_t rows, int64_t max_len, int32_t* order, int32_t* inv,
                     cudaStream_t s);

// A CSR with its rows reordered -- row i of the output is row order[i] of the
// input -- and its column indices renamed by col_inv (input column -> output
// column).  Every row keeps its entries in their input order, so a row's sum
// runs in the same order as before.  val may be null (narrow +-1 storage,
// whose -1 entries keep the ~col encoding).  ptr_out: rows + 1 entries.
template <class T>
void reorder_csr(const int32_t* ptr, const int32_t* idx, const T* val, int64_t rows, int64_t nnz,
                 const int32_t* order, const int32_t* col_inv, int32_t* ptr_out, int32_t* idx_out,
                 T* val_out, cudaStream_t s);

}  // namespace cpdlp
