// sparse_build.cu -- device builds of CSR / transpose from Julia CSC input.
//
// The CSR of A that GPUSparseMatrixCSR stores is sparse(transpose(A))
// (src/utils/mat_csr.jl:58-61): rows in order, columns ascending inside each
// row.  SparseArrays produces it with a sequential counting sort; here it is a
// stable LSD radix sort of the CSC entries by row, which yields the same
// (unique) order, so the index arrays match the reference bit for bit.
#include <cstdlib>

#include "sparse_build.cuh"

namespace cpdlp {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SC_T = 256;
constexpr int SC_I = 8;
constexpr int SC_C = SC_T * SC_I;

__device__ __forceinline__ int32_t warp_incl_scan(int32_t x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// exclusive scan of one value per thread across a 256-thread block
__device__ int32_t block_excl_scan(int32_t v, int32_t* sm, int32_t& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = warp_incl_scan(v);
    if (lane == 31) sm[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t s = (lane < SC_T / 32) ? sm[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < SC_T / 32) sm[lane] = s;
    }
    __syncthreads();
    int32_t off = (w > 0) ? sm[w - 1] : 0;
    total = sm[SC_T / 32 - 1];
    __syncthreads();
    return off + x - v;
}

__global__ void k_scan_reduce(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int32_t sm[SC_T / 32];
    int64_t base = (int64_t)blockIdx.x * SC_C;
    int32_t s = 0;
    for (int i = threadIdx.x; i < SC_C; i += SC_T) {
        int64_t g = base + i;
        if (g < n) s += in[g];
    }
    int32_t tot;
    block_excl_scan(s, sm, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_apply(const int32_t* __restrict__ in, int64_t n,
                             const int32_t* __restrict__ offs, int32_t* __restrict__ out) {
    __shared__ int32_t sm[SC_T / 32];
    int64_t base = (int64_t)blockIdx.x * SC_C + (int64_t)threadIdx.x * SC_I;
    int32_t v[SC_I];
    int32_t local = 0;
#pragma unroll
    for (int i = 0; i < SC_I; i++) {
        int64_t g = base + i;
        v[i] = (g < n) ? in[g] : 0;
        local += v[i];
    }
    int32_t tot;
    int32_t pre = block_excl_scan(local, sm, tot);
    int32_t off = offs ? offs[blockIdx.x] : 0;
    int32_t run = off + pre;
#pragma unroll
    for (int i = 0; i < SC_I; i++) {
        int64_t g = base + i;
        if (g < n) out[g] = run;
        run += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = off + tot;
}

// ---- radix sort --------------------------------------------------------------
constexpr int RS_T = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_C = RS_T * RS_ROUNDS;

__global__ void k_rs_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                          int32_t* __restrict__ hist, int nblocks) {
    __shared__ int32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RS_C;
    for (int i = threadIdx.x; i < RS_C; i += RS_T) {
        int64_t g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items of the block are visited in index order, 256 per round;
// inside a round, warp w holds items [32w, 32w+32) of the round.
__global__ void k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                             uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
                             int shift, const int32_t* __restrict__ offs, int nblocks) {
    __shared__ int32_t run[256];
    __shared__ int32_t wc[RS_T / 32][257];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    run[t] = offs[(int64_t)t * nblocks + blockIdx.x];
    const unsigned lt_mask = (1u << lane) - 1u;
    int64_t base = (int64_t)blockIdx.x * RS_C;
    for (int r = 0; r < RS_ROUNDS; r++) {
#pragma unroll
        for (int q = 0; q < RS_T / 32; q++) wc[q][t] = 0;
        if (t == 0)
            for (int q = 0; q < RS_T / 32; q++) wc[q][256] = 0;
        __syncthreads();
        int64_t g = base + (int64_t)r * RS_T + t;
        bool valid = g < n;
        uint32_t key = valid ? kin[g] : 0u;
        uint32_t val = valid ? vin[g] : 0u;
        int digit = valid ? (int)((key >> shift) & 255u) : 256;
        unsigned peers = __match_any_sync(FULL, digit);
        int rank = __popc(peers & lt_mask);
        if (rank == 0) wc[w][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            int32_t before = 0;
            for (int q = 0; q < w; q++) before += wc[q][digit];
            int32_t pos = run[digit] + before + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        int32_t add = 0;
#pragma unroll
        for (int q = 0; q < RS_T / 32; q++) add += wc[q][t];
        run[t] += add;
        __syncthreads();
    }
}

__global__ void k_iota(uint32_t* v, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

// ---- CSC validation and conversion ------------------------------------------------
enum : int {
    BAD_START = 1, BAD_MONO = 2, BAD_END = 4, BAD_ROW = 8, BAD_ORDER = 16
};

__global__ void k_check_colptr(const int64_t* __restrict__ cp, int64_t n, int64_t nnz,
                               int32_t* __restrict__ ptr1, int* flags) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > n) return;
    int64_t v = cp[j];
    if (j == 0 && v != 1) atomicOr(flags, BAD_START);
    if (j == n && v != nnz + 1) atomicOr(flags, BAD_END);
    if (j < n && cp[j + 1] < v) atomicOr(flags, BAD_MONO);
    ptr1[j] = (int32_t)(v - 1);
}

__global__ void k_check_rows(const int64_t* __restrict__ rv, const int32_t* __restrict__ ptr1,
                             int64_t m, int64_t n, int64_t nnz, int32_t* __restrict__ idx1,
                             int32_t* __restrict__ col1, int* flags) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    int64_t r = rv[k] - 1;
    if (r < 0 || r >= m) {
        atomicOr(flags, BAD_ROW);
        r = 0;
    }
    idx1[k] = (int32_t)r;
    // column: largest j with ptr1[j] <= k
    int64_t lo = 0, hi = n;  // ptr1[lo] <= k < ptr1[hi]
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (ptr1[mid] <= k) lo = mid; else hi = mid;
    }
    col1[k] = (int32_t)lo;
    if (k + 1 < ptr1[lo + 1] && !(rv[k] < rv[k + 1])) atomicOr(flags, BAD_ORDER);
}

__global__ void k_row_hist(const int32_t* __restrict__ rows, int64_t nnz, int32_t* __restrict__ cnt) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) atomicAdd(&cnt[rows[k]], 1);
}

__global__ void k_finish_transpose(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals,
                                   const int32_t* __restrict__ col1, int64_t nnz,
                                   int32_t* __restrict__ idx2, int32_t* __restrict__ row2,
                                   int32_t* __restrict__ p21) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    uint32_t k = svals[p];
    idx2[p] = col1[k];
    row2[p] = (int32_t)skeys[p];
    p21[p] = (int32_t)k;
}

__global__ void k_expand_rows(const int32_t* __restrict__ ptr, int64_t rows,
                              int32_t* __restrict__ row_of, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    int64_t lo = 0, hi = rows;
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (ptr[mid] <= k) lo = mid; else hi = mid;
    }
    row_of[k] = (int32_t)lo;
}

template <class TO, class TI>
__global__ void k_gather_values(const TI* __restrict__ in, const int32_t* __restrict__ perm,
                                TO* __restrict__ out, int64_t nnz) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) out[k] = (TO)in[perm[k]];
}

// lengths of the reordered rows: len[i] = length of row order[i]
__global__ void k_ordered_lengths(const int32_t* __restrict__ ptr, const int32_t* __restrict__ order,
                                  int64_t rows, int32_t* __restrict__ len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) len[i] = ptr[order[i] + 1] - ptr[order[i]];
}

__global__ void k_lengths_u32(const int32_t* __restrict__ ptr, int64_t rows, uint32_t* __restrict__ len) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) len[i] = (uint32_t)(ptr[i + 1] - ptr[i]);
}
__global__ void k_order_out(const uint32_t* __restrict__ sorted, int64_t n, int32_t* __restrict__ order,
                            int32_t* __restrict__ inv) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        order[k] = (int32_t)sorted[k];
        inv[sorted[k]] = (int32_t)k;
    }
}

// entry k of the reordered CSR: the same place in row order[i] of the input,
// its column renamed (a narrow +-1 index ~c of a -1 entry stays encoded)
template <class T>
__global__ void k_reorder_entries(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                  const T* __restrict__ val, const int32_t* __restrict__ ptr_out,
                                  const int32_t* __restrict__ row_of,
                                  const int32_t* __restrict__ order,
                                  const int32_t* __restrict__ col_inv, int64_t nnz,
                                  int32_t* __restrict__ idx_out, T* __restrict__ val_out) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    const int32_t i = row_of[k];
    const int64_t src = (int64_t)ptr[order[i]] + (k - ptr_out[i]);
    const int32_t c = idx[src];
    idx_out[k] = c >= 0 ? col_inv[c] : ~col_inv[~c];
    if (val) val_out[k] = val[src];
}

}  // namespace

void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
    int64_t nb = (n + SC_C - 1) / SC_C;
    if (nb <= 1) {
        k_scan_apply<<<1, SC_T, 0, s>>>(in, n, nullptr, out);
        CK_LAUNCH();
        return;
    }
    DBuf<int32_t> sums((size_t)nb), sums_scan((size_t)nb + 1);
    k_scan_reduce<<<(unsigned)nb, SC_T, 0, s>>>(in, n, sums.p);
    CK_LAUNCH();
    exclusive_scan_i32(sums.p, sums_scan.p, nb, s);
    k_scan_apply<<<(unsigned)nb, SC_T, 0, s>>>(in, n, sums_scan.p, out);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s));
}

void radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& keys_tmp, uint32_t*& vals_tmp,
                      int64_t n, int key_bits, cudaStream_t s) {
    if (n <= 0) return;
    int nblocks = (int)((n + RS_C - 1) / RS_C);
    DBuf<int32_t> hist((size_t)256 * nblocks), offs((size_t)256 * nblocks + 1);
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_rs_hist<<<nblocks, RS_T, 0, s>>>(keys, n, shift, hist.p, nblocks);
        CK_LAUNCH();
        exclusive_scan_i32(hist.p, offs.p, (int64_t)256 * nblocks, s);
        k_rs_scatter<<<nblocks, RS_T, 0, s>>>(keys, vals, keys_tmp, vals_tmp, n, shift, offs.p,
                                              nblocks);
        CK_LAUNCH();
        std::swap(keys, keys_tmp);
        std::swap(vals, vals_tmp);
    }
    CK(cudaStreamSynchronize(s));
}

void expand_rows(const int32_t* ptr, int64_t rows, int32_t* row_of, int64_t nnz, cudaStream_t s) {
    if (nnz <= 0) return;
    k_expand_rows<<<grid_for(nnz, 256), 256, 0, s>>>(ptr, rows, row_of, nnz);
    CK_LAUNCH();
}

template <class TO, class TI>
void gather_values(const TI* in, const int32_t* perm, TO* out, int64_t nnz, cudaStream_t s) {
    if (nnz <= 0) return;
    k_gather_values<TO, TI><<<grid_for(nnz, 256), 256, 0, s>>>(in, perm, out, nnz);
    CK_LAUNCH();
}
template void gather_values<double, double>(const double*, const int32_t*, double*, int64_t, cudaStream_t);
template void gather_values<float, double>(const double*, const int32_t*, float*, int64_t, cudaStream_t);
template void gather_values<float, float>(const float*, const int32_t*, float*, int64_t, cudaStream_t);

static int bit_width(uint64_t v) {
    int b = 0;
    while (v) { b++; v >>= 1; }
    return b;
}

void order_by_length(const int32_t* ptr, int64_t rows, int64_t max_len, int32_t* order, int32_t* inv,
                     cudaStream_t s) {
    if (rows <= 0) return;
    DBuf<uint32_t> k0((size_t)rows), v0((size_t)rows), k1((size_t)rows), v1((size_t)rows);
    k_lengths_u32<<<grid_for(rows, 256), 256, 0, s>>>(ptr, rows, k0.p);
    k_iota<<<grid_for(rows, 256), 256, 0, s>>>(v0.p, rows);
    CK_LAUNCH();
    uint32_t *kp = k0.p, *vp = v0.p, *kt = k1.p, *vt = v1.p;
    radix_sort_pairs(kp, vp, kt, vt, rows, bit_width((uint64_t)(max_len > 0 ? max_len : 0)), s);
    k_order_out<<<grid_for(rows, 256), 256, 0, s>>>(vp, rows, order, inv);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s));
}

template <class T>
void reorder_csr(const int32_t* ptr, const int32_t* idx, const T* val, int64_t rows, int64_t nnz,
                 const int32_t* order, const int32_t* col_inv, int32_t* ptr_out, int32_t* idx_out,
                 T* val_out, cudaStream_t s) {
    DBuf<int32_t> len((size_t)(rows > 0 ? rows : 1));
    if (rows > 0) {
        k_ordered_lengths<<<grid_for(rows, 256), 256, 0, s>>>(ptr, order, rows, len.p);
        CK_LAUNCH();
    }
    exclusive_scan_i32(len.p, ptr_out, rows, s);
    if (nnz > 0) {
        DBuf<int32_t> row_of((size_t)nnz);
        expand_rows(ptr_out, rows, row_of.p, nnz, s);
        k_reorder_entries<T><<<grid_for(nnz, 256), 256, 0, s>>>(ptr, idx, val, ptr_out, row_of.p,
                                                               order, col_inv, nnz, idx_out,
                                                               val_out);
        CK_LAUNCH();
    }
    CK(cudaStreamSynchronize(s));
}
template void reorder_csr<float>(const int32_t*, const int32_t*, const float*, int64_t, int64_t,
                                 const int32_t*, const int32_t*, int32_t*, int32_t*, float*,
                                 cudaStream_t);
template void reorder_csr<double>(const int32_t*, const int32_t*, const double*, int64_t, int64_t,
                                  const int32_t*, const int32_t*, int32_t*, int32_t*, double*,
                                  cudaStream_t);


void build_csc_pair(Handle& h, int64_t m, int64_t n, int64_t nnz, const int64_t* colptr1,
                    const int64_t* rowval1, const double* nzval, CscPair& out) {
    // CPDLP_TRACE=1: the time of each phase
    static const bool trace = [] {
        const char* v = std::getenv("CPDLP_TRACE");
        return v && std::atoi(v) > 0;
    }();
    double t_mark = now_seconds();
    auto mark = [&](const char* what) {
        if (!trace) return;
        CK(cudaStreamSynchronize(h.stream));
        const double t = now_seconds();
        fprintf(stderr, "[cpdlp setup]   %-26s %8.2f ms\n", what, 1e3 * (t - t_mark));
        t_mark = t;
    };
    if (m < 0 || n < 0 || nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative matrix size");
    if (!colptr1 || (nnz > 0 && (!rowval1 || !nzval)))
        fail(CPDLP_ERR_ARGUMENT, "null CSC array pointer");
    if (m >= INT32_MAX || n >= INT32_MAX || nnz >= INT32_MAX)
        fail(CPDLP_ERR_UNSUPPORTED, "matrix dimensions and nnz must be below 2^31 - 1");
    cudaStream_t s = h.stream;
    out.m = m; out.n = n; out.nnz = nnz;
    DBuf<int64_t> cp((size_t)n + 1), rv((size_t)(nnz > 0 ? nnz : 1));
    out.val1.alloc((size_t)(nnz > 0 ? nnz : 1));
    mark("allocate");
    CK(cudaMemcpyAsync(cp.p, colptr1, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice, s));
    if (nnz > 0) {
        CK(cudaMemcpyAsync(rv.p, rowval1, sizeof(int64_t) * (size_t)nnz, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(out.val1.p, nzval, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s));
    }
    DBuf<int> flags(1);
    CK(cudaMemsetAsync(flags.p, 0, sizeof(int), s));
    out.ptr1.alloc((size_t)n + 1);
    mark("upload");
    k_check_colptr<<<grid_for(n + 1, 256), 256, 0, s>>>(cp.p, n, nnz, out.ptr1.p, flags.p);
    CK_LAUNCH();
    int hflags = 0;
    CK(cudaMemcpyAsync(&hflags, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hflags & BAD_START) fail(CPDLP_ERR_ARGUMENT, "invalid CSC: colptr[1] != 1");
    if (hflags & BAD_MONO) fail(CPDLP_ERR_ARGUMENT, "invalid CSC: colptr is not monotone");
    if (hflags & BAD_END) fail(CPDLP_ERR_DIMENSION, "invalid CSC: colptr[n+1] != nnz + 1");
    size_t zn = (size_t)(nnz > 0 ? nnz : 1);
    // index arrays carry 16 padding elements for the tile engine's aligned loads
    out.idx1.alloc(zn + 16);
    CK(cudaMemsetAsync(out.idx1.p, 0, sizeof(int32_t) * (zn + 16), s));
    out.col1.alloc(zn);
    if (nnz > 0) {
        k_check_rows<<<grid_for(nnz, 256), 256, 0, s>>>(rv.p, out.ptr1.p, m, n, nnz, out.idx1.p,
                                                        out.col1.p, flags.p);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(&hflags, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (hflags & BAD_ROW) fail(CPDLP_ERR_ARGUMENT, "invalid CSC: row index out of range");
        if (hflags & BAD_ORDER)
            fail(CPDLP_ERR_ARGUMENT, "invalid CSC: rows not strictly ascending inside a column");
    }
    mark("checks");
    // transpose: stable sort of the entries by row
    out.ptr2.alloc((size_t)m + 1);
    out.idx2.alloc(zn + 16);
    CK(cudaMemsetAsync(out.idx2.p, 0, sizeof(int32_t) * (zn + 16), s));
    out.row2.alloc(zn);
    out.p21.alloc(zn);
    DBuf<int32_t> cnt((size_t)(m > 0 ? m : 1));
    CK(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (size_t)(m > 0 ? m : 1), s));
    if (nnz > 0) {
        k_row_hist<<<grid_for(nnz, 256), 256, 0, s>>>(out.idx1.p, nnz, cnt.p);
        CK_LAUNCH();
    }
    exclusive_scan_i32(cnt.p, out.ptr2.p, m, s);
    if (nnz > 0) {
        DBuf<uint32_t> k0(zn), v0(zn), k1(zn), v1(zn);
        CK(cudaMemcpyAsync(k0.p, out.idx1.p, sizeof(uint32_t) * zn, cudaMemcpyDeviceToDevice, s));
        k_iota<<<grid_for(nnz, 256), 256, 0, s>>>(v0.p, nnz);
        CK_LAUNCH();
        uint32_t *kp = k0.p, *vp = v0.p, *kt = k1.p, *vt = v1.p;
        int bits = bit_width((uint64_t)(m > 1 ? m - 1 : 1));
        radix_sort_pairs(kp, vp, kt, vt, nnz, bits, s);
        k_finish_transpose<<<grid_for(nnz, 256), 256, 0, s>>>(kp, vp, out.col1.p, nnz, out.idx2.p,
                                                              out.row2.p, out.p21.p);
        CK_LAUNCH();
    }
    CK(cudaStreamSynchronize(s));
    mark("transpose");
}

}  // namespace cpdlp
