// noalloc.cu -- cpdlp_spmv_csr_noalloc: CSR mul! on caller-owned device arrays
// that allocates nothing.
//
// Who needs it: callers that may not call cudaMalloc at the moment they need a
// product -- code that runs on a pre-reserved, fixed device-memory budget, a
// host callback or finalizer that must not enter the allocator, or a Julia
// `mul!` on a CuArray-backed GPUSparseMatrixCSR whose arrays already live on
// the device and which should not be copied into a library matrix object.
// cpdlp_spmv needs a cpdlp_matrix (device copies of the arrays and a work
// partition built at construction); this entry point reads the caller's own
// 1-based int32 row pointer / column indices / values directly.
//
// Work split: warp w owns nonzeros [512*w, 512*(w+1)).  Rows entirely inside
// one warp's range are finished by that warp (lane-strided products, fixed
// shuffle tree).  A row that crosses warp ranges leaves one partial sum per
// warp in the scratch array below; a second, thread-per-row pass adds those
// partials in warp order (deterministic) and also writes the rows without
// nonzeros.  A warp skips a run of empty rows with one binary search, so its
// work does not grow with the number of empty rows.
//
// Scratch: a file-scope device array of NA_MAX_WARPS * 2 doubles (1 MiB),
// resident on every GPU that loads this library until the process exits.  It
// bounds nnz at NA_MAX_WARPS * 512 = 33,554,432 nonzeros; larger matrices are
// rejected with CPDLP_ERR_UNSUPPORTED.  Host code cannot use the array's name
// as a device address, so the address is looked up with cudaGetSymbolAddress
// once per device (thread-safe), on that device's first call, with the device
// current.  With CUDA's lazy module loading that first call is also the one
// that makes the array resident, so make it before the device-memory budget
// is fixed.  Every call
// shares the array and it keeps the last call's contents; no part needs
// clearing, because every slot a call reads is written earlier in the same
// call.
//
// Validation flag: a second file-scope device word records invalid CSR input.
// Each call clears it on its stream before its kernels and reads it back after
// them, so every call blocks until its product is done.
//
// Calls that overlap on the GPU (different streams or handles at the same
// time) race on both the scratch array and the validation flag: their
// results can be wrong, and an invalid-input error of one call can be
// reported by, or lost to, a call that overlaps it.  Serialise them.
#include "noalloc.cuh"

#include <mutex>

namespace cpdlp {
namespace {

constexpr int NA_CHUNK = 512;
constexpr int NA_MAX_WARPS = 1 << 16;
constexpr int NA_WARPS_PER_BLOCK = 8;

static __device__ __align__(256) double g_spmv_noalloc_scratch[2 * NA_MAX_WARPS];
// set when the caller's arrays are not a valid 1-based CSR (column outside
// 1..n, row pointer outside 1..nnz+1 or decreasing); offending entries are
// skipped, never dereferenced
static __device__ int g_spmv_noalloc_bad = 0;

// slot 2w  : partial of the row that started before warp w's range
// slot 2w+1: partial of the row that starts in warp w's range and ends after it
template <class T>
__global__ void __launch_bounds__(NA_WARPS_PER_BLOCK * 32)
    k_na_chunks(int64_t m, int64_t n, int64_t nnz, const int32_t* __restrict__ rowptr1,
                const int32_t* __restrict__ colval1, const T* __restrict__ val,
                const T* __restrict__ b, T* __restrict__ c, T alpha, T beta, int use_beta,
                double* __restrict__ scratch) {
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t lo = w * NA_CHUNK;
    if (lo >= nnz) return;
    const int64_t hi = min(lo + (int64_t)NA_CHUNK, nnz);
    // row containing nonzero lo: largest r with rowptr[r] - 1 <= lo
    int64_t rlo = 0, rhi = m;  // rowptr0[rlo] <= lo < rowptr0[rhi]
    while (rhi - rlo > 1) {
        const int64_t mid = (rlo + rhi) >> 1;
        if ((int64_t)rowptr1[mid] - 1 <= lo) rlo = mid; else rhi = mid;
    }
    for (int64_t r = rlo; r < m;) {
        const int64_t ra = (int64_t)rowptr1[r] - 1, rb = (int64_t)rowptr1[r + 1] - 1;
        if (ra >= hi) break;
        // the next row to visit: the last q in (r, m] with rowptr0[q] <= rb,
        // so a run of empty rows (written by the second pass) costs one
        // binary search; q always advances, whatever the input
        int64_t nlo = r + 1, nhi = m;
        if ((int64_t)rowptr1[nlo] - 1 <= rb) {
            while (nhi > nlo) {
                const int64_t mid = (nlo + nhi + 1) >> 1;
                if ((int64_t)rowptr1[mid] - 1 <= rb) nlo = mid; else nhi = mid - 1;
            }
        }
        const int64_t next = nlo;
        if (rb <= ra) { r = next; continue; }
        const int64_t a = max(ra, lo), e = min(rb, hi);
        T s = T(0);
        for (int64_t k = a + lane; k < e; k += 32) {
            const int64_t j = (int64_t)colval1[k] - 1;
            if (j < 0 || j >= n) {
                g_spmv_noalloc_bad = 1;
                continue;
            }
            s = add_rn(s, mul_rn(val[k], b[j]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = add_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
        if (lane == 0) {
            if (ra >= lo && rb <= hi) {
                T v = mul_rn(alpha, s);
                if (use_beta) v = add_rn(v, mul_rn(beta, c[r]));
                c[r] = v;
            } else if (ra < lo) {
                scratch[2 * w] = (double)s;
            } else {
                scratch[2 * w + 1] = (double)s;
            }
        }
        r = next;
    }
}

// rows without nonzeros, and rows spanning several warp ranges
template <class T>
__global__ void k_na_fixup(int64_t m, int64_t nnz, const int32_t* __restrict__ rowptr1,
                           T* __restrict__ c, T alpha, T beta, int use_beta,
                           const double* __restrict__ scratch) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int64_t ra = (int64_t)rowptr1[r] - 1, rb = (int64_t)rowptr1[r + 1] - 1;
    if (ra < 0 || rb > nnz || rb < ra) {
        g_spmv_noalloc_bad = 1;
        return;
    }
    T s;
    if (rb <= ra) {
        s = T(0);
    } else {
        const int64_t w1 = ra / NA_CHUNK, w2 = (rb - 1) / NA_CHUNK;
        if (w1 == w2) return;  // finished by its warp
        T acc = (T)scratch[2 * w1 + 1];
        for (int64_t w = w1 + 1; w <= w2; w++) acc = add_rn(acc, (T)scratch[2 * w]);
        s = acc;
    }
    T v = mul_rn(alpha, s);
    if (use_beta) v = add_rn(v, mul_rn(beta, c[r]));
    c[r] = v;
}

// device addresses of the scratch array and of the validation flag, looked up
// once per device (the device is current: every entry point sets the handle's
// device first)
struct NaSymbols {
    double* scratch = nullptr;
    int* bad = nullptr;
};
NaSymbols symbols(int device) {
    static std::once_flag once[64];
    static NaSymbols addr[64];
    if (device < 0 || device >= 64) fail(CPDLP_ERR_UNSUPPORTED, "device ordinal above 63");
    std::call_once(once[device], [device] {
        void* p = nullptr;
        void* q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_spmv_noalloc_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_spmv_noalloc_bad);
        if (e != cudaSuccess)
            fail(CPDLP_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") +
                                     cudaGetErrorString(e));
        addr[device].scratch = static_cast<double*>(p);
        addr[device].bad = static_cast<int*>(q);
    });
    return addr[device];
}

template <class T>
void run(Handle& h, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr1,
         const int32_t* colval1, const void* nzval, const void* b, void* c, double alpha,
         double beta) {
    const NaSymbols sym = symbols(h.device);
    double* scratch = sym.scratch;
    CK(cudaMemsetAsync(sym.bad, 0, sizeof(int), h.stream));
    const int use_beta = beta != 0.0;
    const int64_t warps = (nnz + NA_CHUNK - 1) / NA_CHUNK;
    if (warps > 0) {
        const unsigned grid = (unsigned)((warps + NA_WARPS_PER_BLOCK - 1) / NA_WARPS_PER_BLOCK);
        k_na_chunks<T><<<grid, NA_WARPS_PER_BLOCK * 32, 0, h.stream>>>(
            m, n, nnz, rowptr1, colval1, static_cast<const T*>(nzval), static_cast<const T*>(b),
            static_cast<T*>(c), (T)alpha, (T)beta, use_beta, scratch);
        CK_LAUNCH();
    }
    if (m > 0) {
        k_na_fixup<T><<<grid_for(m, 256), 256, 0, h.stream>>>(
            m, nnz, rowptr1, static_cast<T*>(c), (T)alpha, (T)beta, use_beta, scratch);
        CK_LAUNCH();
    }
}

}  // namespace

void spmv_csr_noalloc(Handle& h, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr1,
                      const int32_t* colval1, const void* nzval, int32_t value_type,
                      const void* b, void* c, double alpha, double beta) {
    if (m < 0 || n < 0 || nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative matrix size");
    if (m >= INT32_MAX || n >= INT32_MAX)
        fail(CPDLP_ERR_UNSUPPORTED, "matrix dimensions must be below 2^31 - 1");
    if (nnz > (int64_t)NA_MAX_WARPS * NA_CHUNK)
        fail(CPDLP_ERR_UNSUPPORTED,
             "cpdlp_spmv_csr_noalloc handles at most 33554432 nonzeros (fixed 1 MiB scratch); "
             "use cpdlp_matrix_from_csc + cpdlp_spmv for larger matrices");
    if (m > 0 && (!rowptr1 || !c)) fail(CPDLP_ERR_ARGUMENT, "null row pointer or output vector");
    if (nnz > 0 && (!colval1 || !nzval || !b)) fail(CPDLP_ERR_ARGUMENT, "null CSR array or input vector");
    if (value_type == CPDLP_VAL_F64)
        run<double>(h, m, n, nnz, rowptr1, colval1, nzval, b, c, alpha, beta);
    else if (value_type == CPDLP_VAL_F32)
        run<float>(h, m, n, nnz, rowptr1, colval1, nzval, b, c, alpha, beta);
    else
        fail(CPDLP_ERR_ARGUMENT, "value_type must be CPDLP_VAL_F64 or CPDLP_VAL_F32");
    // stream-ordered read of the flag on the handle's stream (the legacy
    // default stream is not touched); a copy into pageable memory returns
    // once it is done
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, symbols(h.device).bad, sizeof(int), cudaMemcpyDeviceToHost,
                       h.stream));
    CK(cudaStreamSynchronize(h.stream));
    if (bad) {
        fail(CPDLP_ERR_ARGUMENT,
             "cpdlp_spmv_csr_noalloc: arrays are not a valid 1-based CSR (column outside 1..n "
             "or row pointer outside 1..nnz+1); offending entries were skipped");
    }
}

}  // namespace cpdlp
