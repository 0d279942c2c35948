// tiles.cuh -- the warp-tile CSR SpMV engine with fused per-row epilogues.
//
// Work partition (built once per matrix on the host from its row pointer):
//  * short tile {r0, r1, nz0, nz1}: consecutive rows [r0, r1), each at most
//    TILE = 32*ITEMS nonzeros, together at most TILE nonzeros and at most
//    MAX_TILE_ROWS rows.  One warp
//      1. prefetches the row pointers and the epilogue inputs of its rows,
//      2. loads the tile's values and column indices with 128-bit loads
//         (window aligned down to 4 elements), all issued before any use,
//      3. gathers x[col] for the whole tile in one batch,
//      4. writes value*x products to shared memory, and
//      5. lets every lane reduce its rows of at most LONG_ROW nonzeros in
//         ascending column order (the reference's order), while longer rows
//         are reduced by the whole warp; the fused epilogue follows.
//  * long-row piece {row, -(piece+1), long_id, slot_base}: a row longer than
//    TILE is cut into TILE-sized pieces, one warp each, reduced with warp
//    shuffles.  A row of several pieces writes each partial to a scratch slot;
//    the warp that completes the row (atomic counter, no waiting) adds the
//    partials in piece order and applies the epilogue, so results do not
//    depend on scheduling.
// Row sums use explicit round-to-nearest multiply/add (no FMA contraction), so
// rows of at most LONG_ROW nonzeros reproduce a sequential CPU sum exactly.
// Index and value arrays must be allocated with PAD_ELEMS extra elements:
// the aligned 128-bit window may read up to 3 elements past the last row.
#pragma once

#include <atomic>
#include <cmath>
#include <type_traits>

#include "cpdlp_common.cuh"

namespace cpdlp {

constexpr int MAX_TILE_ROWS = 128;
constexpr int ROWS_PER_LANE = MAX_TILE_ROWS / 32;
constexpr int LONG_ROW = 64;
constexpr int PAD_ELEMS = 16;
constexpr unsigned FULL_MASK = 0xffffffffu;

struct TilePlan {
    int32_t rows = 0;
    int32_t items = 16;     // nonzeros per lane of a short tile
    int32_t ntasks = 0;
    int32_t nshort = 0;
    int32_t nlong = 0;      // rows that take the warp path
    int32_t npieces = 0;    // pieces of all long rows
    int32_t nltasks = 0;    // long-row pieces (tasks of the long-row kernel)
    int32_t rpl = ROWS_PER_LANE;  // rows per lane of a short tile (row cap / 32)
    bool medium = false;    // some short tile holds a row longer than LONG_ROW
    DBuf<int4> tasks;       // short tiles
    DBuf<int4> ltasks;      // long-row pieces
    DBuf<int32_t> counters; // per long row, zero between launches
    std::vector<int32_t> long_rows;
    int tile_nnz() const { return 32 * items; }
};

// Host-side partition of the rows of a CSR (ptr on the host, 0-based, rows+1).
// With seg_rows (segment start rows, last = rows) no tile crosses a segment
// start, and seg_tasks / seg_ltasks / seg_lids receive, per segment, the first
// short task, long task and long-row id (one extra final entry = totals).
// max_rows caps the rows of a short tile (a multiple of 32, at most
// MAX_TILE_ROWS): kernels built for max_rows / 32 rows per lane.  With the
// default cap, a matrix with rows of LONG_ROW+1 .. TILE nonzeros (which short
// tiles sum with the whole warp) gets tiles of at most 64 rows: the kernels
// that handle such rows keep two rows per lane in registers instead of four.
void build_tile_plan(const std::vector<int32_t>& ptr, int32_t rows, int items, TilePlan& plan,
                     cudaStream_t s, const std::vector<int64_t>* seg_rows = nullptr,
                     std::vector<int32_t>* seg_tasks = nullptr,
                     std::vector<int32_t>* seg_ltasks = nullptr,
                     std::vector<int32_t>* seg_lids = nullptr, int max_rows = MAX_TILE_ROWS);

// Picks nonzeros-per-lane from the size and mean row length (autotuner default).
int choose_items(int64_t nnz, int64_t rows, int requested_tile_nnz);

template <class V, class T>
struct CsrView {
    const int32_t* __restrict__ ptr;
    const int32_t* __restrict__ idx;
    const V* __restrict__ val;
    const int4* __restrict__ tasks;       // short tiles
    int32_t ntasks;
    const int4* __restrict__ ltasks;      // long-row pieces
    int32_t nltasks;
    int32_t* counters;
    T* partials;   // npieces * NVEC
};

// Matrices whose values are all exactly +-1 store no value array: the sign is
// carried by the column index (col for +1, ~col for -1), so a nonzero costs 4
// bytes instead of 8 or 12.  Products with +-1 are exact.
struct Pm1 {};
template <class V>
struct is_pm1 : std::false_type {};
template <>
struct is_pm1<Pm1> : std::true_type {};
__host__ __device__ __forceinline__ int pm1_col(int c) { return c ^ (c >> 31); }
template <class T>
__device__ __forceinline__ T pm1_apply(int c, T x) { return c < 0 ? -x : x; }

// The input vectors of one product.  COH = false gathers them through the
// non-coherent read-only path, valid when nothing in the same launch writes
// them (one product per launch).  COH = true uses coherent loads, for kernels
// that rewrite the vectors between products (the batched solver's step loop).
template <class T, int NVEC, bool COH = false>
struct VecSet {
    const T* v[NVEC];
};

// v[p] for a runtime p without indexing a parameter array dynamically (which
// would copy it to local memory)
template <class T, int N>
__device__ __forceinline__ const T* pick(const T* const (&v)[N], int p) {
    const T* r = v[0];
#pragma unroll
    for (int q = 1; q < N; q++)
        if (p == q) r = v[q];
    return r;
}

// ---- 4-element chunk loads (the chunk start is a multiple of 4 elements) ----
// Streaming (evict-first) loads written as volatile PTX: they keep their
// program order, so a batch of them is issued back to back before the first
// result is consumed.  The matrix is read once per pass; evict-first keeps
// the gathered vectors resident in L2.
__device__ __forceinline__ void load4(const int32_t* p, int (&o)[4]) {
    asm volatile("ld.global.cs.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3])
                 : "l"(p));
}
template <class T>
__device__ __forceinline__ void load4v(const float* p, T (&o)[4]) {
    float a, b, c, d;
    asm volatile("ld.global.cs.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(a), "=f"(b), "=f"(c), "=f"(d)
                 : "l"(p));
    o[0] = (T)a; o[1] = (T)b; o[2] = (T)c; o[3] = (T)d;
}
template <class T>
__device__ __forceinline__ void load4v(const double* p, T (&o)[4]) {
    double a, b, c, d;
    asm volatile("ld.global.cs.v2.f64 {%0, %1}, [%2];" : "=d"(a), "=d"(b) : "l"(p));
    asm volatile("ld.global.cs.v2.f64 {%0, %1}, [%2];" : "=d"(c), "=d"(d) : "l"(p + 2));
    o[0] = (T)a; o[1] = (T)b; o[2] = (T)c; o[3] = (T)d;
}
// gathers of x[col]: through the read-only path (COH = false) or with a
// coherent load (COH = true); same ordering property as the loads above
template <bool COH>
__device__ __forceinline__ float gather(const float* p) {
    float v;
    if (COH) asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(p));
    else asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
template <bool COH>
__device__ __forceinline__ double gather(const double* p) {
    double v;
    if (COH) asm volatile("ld.global.f64 %0, [%1];" : "=d"(v) : "l"(p));
    else asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
// four interleaved values p[0..3] (16-byte aligned) in one request (two for
// FP64): the packed iterates of the KKT pass
__device__ __forceinline__ void gather4(const float* p, float (&o)[4]) {
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
                 : "l"(p));
}
__device__ __forceinline__ void gather4(const double* p, double (&o)[4]) {
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(o[0]), "=d"(o[1]) : "l"(p));
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(o[2]), "=d"(o[3]) : "l"(p + 2));
}
// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned):
// a gather that holds no registers while in flight
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}
// four values to 16-byte-aligned shared memory (one vector store for FP32,
// two for FP64)
__device__ __forceinline__ void store4_shared(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store4_shared(double* p, const double (&v)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
template <class V, class T>
__device__ __forceinline__ T load1v(const V* p) {
    return (T)__ldcs(p);
}

template <class T>
__device__ __forceinline__ T warp_sum_tree(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = add_rn(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

// GPU wall clock in nanoseconds
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int TILE_WARPS = 8;
// elements of a warp's short-tile product buffer (16-byte aligned): the tile's
// nonzeros from the 4-element-aligned window start, plus the window's slack
template <int ITEMS>
constexpr int tile_buf() { return 32 * ITEMS + 4; }
// Warps per block of the KKT pass: the four iterates' gathered values of a
// whole tile live in shared memory, within the static 48 KB (4 warps for FP32
// iterates, 2 for FP64).
template <class T>
constexpr int kkt_warps() { return sizeof(T) == 4 ? 4 : 2; }
// Resident blocks per SM of the four-iterate KKT pass, which caps its grid at
// SMs x this (the kernel loops over its tasks): 4 x 4 warps for FP32 (up to
// 109 registers a thread), 6 x 2 warps for FP64 (33 KB of shared memory a
// block).
template <class T>
constexpr int kkt_blocks_per_sm() { return sizeof(T) == 4 ? 4 : 6; }

// One warp, one short tile.  All loads of a phase are volatile PTX issued back
// to back, so they are in flight together: (1) the tile's indices and values
// with 128-bit loads over the 4-element-aligned window plus the row pointers
// and epilogue inputs of this lane's rows, (2) one batch of gathers.  Then
// products go to shared memory and every lane reduces whole rows in column
// order before the fused epilogue.  RPL: rows per lane, the plan's row cap / 32.
template <int ITEMS, int NVEC, class V, class T, class Epi, bool COH, int RPL = ROWS_PER_LANE,
          bool MED = false>
__device__ __forceinline__ void short_tile(const CsrView<V, T>& A, const VecSet<T, NVEC, COH>& xs,
                                           Epi& epi, typename Epi::Acc& acc, int r0, int r1,
                                           int nz0, int nz1, int lane, T* prod) {
    constexpr int NV4 = ITEMS / 4 + 1;  // 4-element chunks per lane (+1: alignment slack)
    const int base = nz0 & ~3;
    int ra[RPL], rb[RPL];
    typename Epi::Pre pre[RPL];
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        const int r = r0 + lane + 32 * k;
        if (r < r1) {
            ra[k] = ld_keep(A.ptr + r);
            rb[k] = ld_keep(A.ptr + r + 1);
            pre[k] = epi.pre_global(r);
        } else {
            ra[k] = rb[k] = 0;
        }
    }
    int cc[NV4][4];
    T vv[NV4][4];
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
        if (e < nz1) {
            load4(A.idx + e, cc[j]);
            if constexpr (!is_pm1<V>::value) load4v<T>(A.val + e, vv[j]);
            else vv[j][0] = vv[j][1] = vv[j][2] = vv[j][3] = T(0);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) { cc[j][q] = 0; vv[j][q] = T(0); }
        }
    }
    // one input vector at a time (not unrolled): with several vectors this
    // keeps one batch of gathers in registers instead of all of them
#pragma unroll 1
    for (int p = 0; p < NVEC; p++) {
        const T* xv = pick(xs.v, p);
        T xg[NV4][4];
#pragma unroll
        for (int j = 0; j < NV4; j++) {
            const int e = base + 4 * (lane + 32 * j);
#pragma unroll
            for (int q = 0; q < 4; q++)
                xg[j][q] = (e + q >= nz0 && e + q < nz1)
                               ? gather<COH>(xv + (is_pm1<V>::value ? pm1_col(cc[j][q]) : cc[j][q]))
                               : T(0);
        }
        // products to shared memory, indexed from the aligned window start.
        // FP32 tiles with medium rows store a chunk's four products with one
        // 16-byte store (fewer shared-store wavefronts; the entries outside
        // the tile are never read); the other kernels store the tile's
        // entries one by one, which keeps them at fewer registers (measured
        // on C1: the vector store took the primal step from 64 to 72
        // registers and 0.124 to 0.130 ms, and the dual step from 0.120 to
        // 0.111 ms)
        constexpr bool VEC_STORE = MED && sizeof(T) == 4;
#pragma unroll
        for (int j = 0; j < NV4; j++) {
            const int e = base + 4 * (lane + 32 * j);
            if constexpr (VEC_STORE) {
                if (e < nz1) {
                    T pr[4];
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        pr[q] = is_pm1<V>::value ? pm1_apply(cc[j][q], xg[j][q])
                                                 : mul_rn(vv[j][q], xg[j][q]);
                    store4_shared(prod + (e - base), pr);
                }
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (e + q >= nz0 && e + q < nz1)
                        prod[e + q - base] = is_pm1<V>::value ? pm1_apply(cc[j][q], xg[j][q])
                                                              : mul_rn(vv[j][q], xg[j][q]);
            }
        }
        __syncwarp();
        const T* prow = prod + (nz0 - base);  // prow[i - nz0]: nonzero i of the tile
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            const int r = r0 + lane + 32 * k;
            const int len = rb[k] - ra[k];
            T sum = T(0);
            if constexpr (MED) {
                // rows longer than LONG_ROW: the whole warp, lane-strided
                // partial sums and a fixed shuffle tree (a long-row piece's order)
                unsigned med = __ballot_sync(FULL_MASK, r < r1 && len > LONG_ROW);
                while (med) {
                    const int l = __ffs(med) - 1;
                    med &= med - 1;
                    const int a = __shfl_sync(FULL_MASK, ra[k], l) - nz0;
                    const int b = __shfl_sync(FULL_MASK, rb[k], l) - nz0;
                    T part = T(0);
                    for (int i = a + lane; i < b; i += 32) part = add_rn(part, prow[i]);
                    part = warp_sum_tree(part);
                    if (lane == l) sum = part;
                }
            }
            if (r < r1) {
                if (len <= LONG_ROW)
                    for (int i = ra[k] - nz0; i < rb[k] - nz0; i++) sum = add_rn(sum, prow[i]);
                epi.row(p, r, sum, pre[k], acc);
            }
        }
        __syncwarp();
    }
}

// One warp, one TILE-sized piece of a row longer than TILE: lane-strided
// coalesced loads, lane partial sums, a fixed shuffle tree.  Multi-piece rows
// combine through scratch slots: the warp that completes the row (atomic
// counter, no waiting) adds the partials in piece order and applies the
// epilogue.
template <int ITEMS, int NVEC, class V, class T, class Epi, bool COH>
__device__ __forceinline__ void long_piece(const CsrView<V, T>& A, const VecSet<T, NVEC, COH>& xs,
                                           Epi& epi, typename Epi::Acc& acc, int4 t, int lane) {
    constexpr int TILE = 32 * ITEMS;
    const int row = t.x, piece = -t.y - 1, lid = t.z, base_slot = t.w;
    const int rb = ld_keep(A.ptr + row), re = ld_keep(A.ptr + row + 1);
    const int npieces = (re - rb + TILE - 1) / TILE;
    const int a = rb + piece * TILE;
    const int b = min(a + TILE, re);
    T s[NVEC];
#pragma unroll
    for (int p = 0; p < NVEC; p++) s[p] = T(0);
    for (int e = a + lane; e < b; e += 32) {
        const int cc = __ldcs(A.idx + e);
        if constexpr (is_pm1<V>::value) {
#pragma unroll
            for (int p = 0; p < NVEC; p++)
                s[p] = add_rn(s[p], pm1_apply(cc, gather<COH>(xs.v[p] + pm1_col(cc))));
        } else {
            const T vv = load1v<V, T>(A.val + e);
#pragma unroll
            for (int p = 0; p < NVEC; p++) s[p] = add_rn(s[p], mul_rn(vv, gather<COH>(xs.v[p] + cc)));
        }
    }
#pragma unroll
    for (int p = 0; p < NVEC; p++) s[p] = warp_sum_tree(s[p]);
    if (npieces == 1) {
        if (lane == 0) {
#pragma unroll
            for (int p = 0; p < NVEC; p++) epi.row_long(p, row, s[p], lid, acc);
        }
        return;
    }
    int done = 0;
    if (lane == 0) {
#pragma unroll
        for (int p = 0; p < NVEC; p++) A.partials[(size_t)(base_slot + piece) * NVEC + p] = s[p];
        __threadfence();
        done = atomicAdd(&A.counters[lid], 1);
    }
    done = __shfl_sync(FULL_MASK, done, 0);
    if (done == npieces - 1) {
        __threadfence();
        if (lane == 0) {
#pragma unroll
            for (int p = 0; p < NVEC; p++) {
                T tot = T(0);
                for (int q = 0; q < npieces; q++)
                    tot = add_rn(tot, __ldcg(A.partials + (size_t)(base_slot + q) * NVEC + p));
                epi.row_long(p, row, tot, lid, acc);
            }
            A.counters[lid] = 0;
        }
    }
}

// One launch covers both kinds of work: the first warps take the long-row
// pieces (so they start early), the rest the short tiles.
// FP64 iterates: at least CPDLP_F64_MIN_BLOCKS resident blocks per SM (a
// register cap; unbounded, the FP64 step kernels took up to 159 registers and
// one 8-warp block per SM).  FP32 kernels are left to the compiler (56-64
// registers; a cap of 64 made it spill).
#ifndef CPDLP_F64_MIN_BLOCKS
#define CPDLP_F64_MIN_BLOCKS 2
#endif
template <int ITEMS, int WARPS, int NVEC, class V, class T, class Epi, int RPL, bool MED>
__global__ void __launch_bounds__(WARPS * 32, sizeof(T) == 8 ? CPDLP_F64_MIN_BLOCKS : 1)
    k_tiles(CsrView<V, T> A, VecSet<T, NVEC> xs, Epi epi) {
    __shared__ __align__(16) T prod[WARPS][tile_buf<ITEMS>()];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int task = blockIdx.x * WARPS + w;
    typename Epi::Acc acc;
    epi.init(acc);
    if (task < A.nltasks) {
        long_piece<ITEMS, NVEC>(A, xs, epi, acc, A.ltasks[task], lane);
    } else if (task - A.nltasks < A.ntasks) {
        const int4 t = A.tasks[task - A.nltasks];
        short_tile<ITEMS, NVEC, V, T, Epi, false, RPL, MED>(A, xs, epi, acc, t.x, t.y, t.z, t.w,
                                                            lane, prod[w]);
    }
    epi.finish(acc);
}

// Launches the tile kernel on `s` with WARPS warps per block.  Reducing
// epilogues write one row of block partials per block.
// The unified L1 / shared memory of an SM is split by a carveout; the driver
// picks one that fits many blocks of a kernel, which leaves the gathers'
// L1 data cache smaller than these kernels need.  Once per kernel, outside a
// stream capture, this asks for just the shared memory of the kernel's
// resident blocks (by registers) and leaves the rest to L1 (C1's primal step:
// 0.1185 -> 0.1156 ms, dual step 0.1096 -> 0.1084 ms).
// Set while a caller walks its launch sequence only to apply prefer_l1 (the
// step kernels, before their CUDA-graph capture): the tile launchers then
// skip the launches themselves.
inline bool& tiles_dry_run() {
    static thread_local bool dry = false;
    return dry;
}

template <auto Kernel>
void prefer_l1(int threads, cudaStream_t s) {
    static std::atomic<int> state{0};  // 0: not yet, 1: in progress, 2: done
    if (state.load(std::memory_order_acquire) == 2) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    int expected = 0;
    if (!state.compare_exchange_strong(expected, 1)) return;
    cudaFuncAttributes fa{};
    int blocks = 0, dev = 0, smem_sm = 0;
    if (cudaFuncGetAttributes(&fa, Kernel) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, Kernel, threads, 0) == cudaSuccess &&
        cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        blocks > 0 && smem_sm > 0) {
        const double need = (double)blocks * (double)(fa.sharedSizeBytes + 1024);
        const int pct = std::min(100, (int)std::ceil(100.0 * need / smem_sm) + 1);
        cudaFuncSetAttribute(Kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    }
    cudaGetLastError();  // a refused hint leaves the driver's choice
    state.store(2, std::memory_order_release);
}

template <int WARPS, int NVEC, class V, class T, class Epi>
void launch_tiles_w(const TilePlan& plan, const CsrView<V, T>& view, const VecSet<T, NVEC>& xs,
                    const Epi& epi, cudaStream_t s) {
    const int64_t tasks = (int64_t)plan.ntasks + plan.nltasks;
    if (tasks == 0) return;
    const unsigned grid = (unsigned)((tasks + WARPS - 1) / WARPS);
#define CPDLP_TILES(IT, R, M)                                                 \
    prefer_l1<k_tiles<IT, WARPS, NVEC, V, T, Epi, R, M>>(WARPS * 32, s);      \
    if (!tiles_dry_run())                                                     \
        k_tiles<IT, WARPS, NVEC, V, T, Epi, R, M><<<grid, WARPS * 32, 0, s>>>(view, xs, epi)
    if (plan.medium) {
        if (plan.rpl != 2) fail(CPDLP_ERR_ARGUMENT, "tile plan with long rows needs 64-row tiles");
        switch (plan.items) {
            case 4: CPDLP_TILES(4, 2, true); break;
            case 8: CPDLP_TILES(8, 2, true); break;
            default: CPDLP_TILES(16, 2, true); break;
        }
    } else {
        if (plan.rpl != ROWS_PER_LANE && plan.rpl != 2 && plan.rpl != 1)
            fail(CPDLP_ERR_ARGUMENT, "tile plan row cap");
        switch (plan.items) {
            case 4: CPDLP_TILES(4, ROWS_PER_LANE, false); break;
            case 8: CPDLP_TILES(8, ROWS_PER_LANE, false); break;
            default: CPDLP_TILES(16, ROWS_PER_LANE, false); break;
        }
    }
#undef CPDLP_TILES
    CK_LAUNCH();
}
template <int NVEC, class V, class T, class Epi>
void launch_tiles(const TilePlan& plan, const CsrView<V, T>& view, const VecSet<T, NVEC>& xs,
                  const Epi& epi, cudaStream_t s) {
    launch_tiles_w<TILE_WARPS>(plan, view, xs, epi, s);
}

// ---- four iterates per pass (the KKT evaluation) ------------------------------
// x4 holds the four gathered vectors interleaved (x4[4*col + p]), so one
// request per nonzero fetches all four.  The gathers are asynchronous copies
// (cp.async) straight into the warp's shared buffer g[k][0..3] (k = the
// nonzero's place in the tile): they hold no registers, so all of a lane's
// gathers are in flight at once.  Each lane then multiplies its own nonzeros'
// four values in place, and every lane reduces its rows for the four iterates
// side by side, each in ascending column order: iterate p's row sums are the
// ones a one-iterate pass over x_p computes.
template <int ITEMS, class V, class T, class Epi, int RPL = ROWS_PER_LANE, bool MED = false>
__device__ __forceinline__ void short_tile4(const CsrView<V, T>& A, const T* __restrict__ x4,
                                            Epi& epi, typename Epi::Acc& acc, int r0, int r1,
                                            int nz0, int nz1, int lane, T* g) {
    constexpr int NV4 = ITEMS / 4 + 1;
    const int base = nz0 & ~3;
    int ra[RPL], rb[RPL];
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        const int r = r0 + lane + 32 * k;
        if (r < r1) {
            ra[k] = ld_keep(A.ptr + r);
            rb[k] = ld_keep(A.ptr + r + 1);
        } else {
            ra[k] = rb[k] = 0;
        }
    }
    int cc[NV4][4];
    T vv[NV4][4];
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
        if (e < nz1) {
            load4(A.idx + e, cc[j]);
            if constexpr (!is_pm1<V>::value) load4v<T>(A.val + e, vv[j]);
            else vv[j][0] = vv[j][1] = vv[j][2] = vv[j][3] = T(0);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) { cc[j][q] = 0; vv[j][q] = T(0); }
        }
    }
    // the gathers: 4 values of T per nonzero, 16 bytes per copy
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (e + q >= nz0 && e + q < nz1) {
                const int col = is_pm1<V>::value ? pm1_col(cc[j][q]) : cc[j][q];
                const T* src = x4 + 4 * (size_t)col;
                T* dst = g + 4 * (e + q - nz0);
#pragma unroll
                for (int h = 0; h < (int)(4 * sizeof(T)) / 16; h++)
                    cp_async16(dst + h * (16 / sizeof(T)), src + h * (16 / sizeof(T)));
            }
    }
    cp_async_wait_all();
    // products in place (each lane its own nonzeros)
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (e + q >= nz0 && e + q < nz1) {
                T* gk = g + 4 * (e + q - nz0);
#pragma unroll
                for (int p = 0; p < 4; p++)
                    gk[p] = is_pm1<V>::value ? pm1_apply(cc[j][q], gk[p]) : mul_rn(vv[j][q], gk[p]);
            }
    }
    __syncwarp();
    // rows longer than LONG_ROW: the whole warp, lane-strided sums and a tree
#pragma unroll
    for (int k = 0; k < (MED ? RPL : 0); k++) {
        const int r = r0 + lane + 32 * k;
        unsigned med = __ballot_sync(FULL_MASK, r < r1 && rb[k] - ra[k] > LONG_ROW);
        while (med) {
            const int l = __ffs(med) - 1;
            med &= med - 1;
            const int a = __shfl_sync(FULL_MASK, ra[k], l) - nz0;
            const int b = __shfl_sync(FULL_MASK, rb[k], l) - nz0;
            T m0 = T(0), m1 = T(0), m2 = T(0), m3 = T(0);
            for (int i = a + lane; i < b; i += 32) {
                const T* gi = g + 4 * i;
                m0 = add_rn(m0, gi[0]);
                m1 = add_rn(m1, gi[1]);
                m2 = add_rn(m2, gi[2]);
                m3 = add_rn(m3, gi[3]);
            }
            m0 = warp_sum_tree(m0);
            m1 = warp_sum_tree(m1);
            m2 = warp_sum_tree(m2);
            m3 = warp_sum_tree(m3);
            if (lane == l) {
                const typename Epi::Pre pre{};
                epi.row(0, r, m0, pre, acc);
                epi.row(1, r, m1, pre, acc);
                epi.row(2, r, m2, pre, acc);
                epi.row(3, r, m3, pre, acc);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        const int r = r0 + lane + 32 * k;
        if (r < r1 && rb[k] - ra[k] <= LONG_ROW) {
            T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
            for (int i = ra[k] - nz0; i < rb[k] - nz0; i++) {
                const T* gi = g + 4 * i;
                s0 = add_rn(s0, gi[0]);
                s1 = add_rn(s1, gi[1]);
                s2 = add_rn(s2, gi[2]);
                s3 = add_rn(s3, gi[3]);
            }
            const typename Epi::Pre pre{};
            epi.row(0, r, s0, pre, acc);
            epi.row(1, r, s1, pre, acc);
            epi.row(2, r, s2, pre, acc);
            epi.row(3, r, s3, pre, acc);
        }
    }
    __syncwarp();
}

// one TILE-sized piece of a long row, four packed iterates (see long_piece):
// the gathers are asynchronous copies into the warp's buffer g, and each lane
// sums its own elements' products for the four iterates
template <int ITEMS, class V, class T, class Epi>
__device__ __forceinline__ void long_piece4(const CsrView<V, T>& A, const T* __restrict__ x4,
                                            Epi& epi, typename Epi::Acc& acc, int4 t, int lane,
                                            T* g) {
    constexpr int TILE = 32 * ITEMS;
    constexpr int NV4 = ITEMS / 4 + 1;
    const int row = t.x, piece = -t.y - 1, lid = t.z, base_slot = t.w;
    const int rb = ld_keep(A.ptr + row), re = ld_keep(A.ptr + row + 1);
    const int npieces = (re - rb + TILE - 1) / TILE;
    const int a = rb + piece * TILE;
    const int b = min(a + TILE, re);
    const int base = a & ~3;
    int cc[NV4][4];
    T vv[NV4][4];
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
        if (e < b) {
            load4(A.idx + e, cc[j]);
            if constexpr (!is_pm1<V>::value) load4v<T>(A.val + e, vv[j]);
            else vv[j][0] = vv[j][1] = vv[j][2] = vv[j][3] = T(0);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) { cc[j][q] = 0; vv[j][q] = T(0); }
        }
    }
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (e + q >= a && e + q < b) {
                const int col = is_pm1<V>::value ? pm1_col(cc[j][q]) : cc[j][q];
                const T* src = x4 + 4 * (size_t)col;
                T* dst = g + 4 * (e + q - a);
#pragma unroll
                for (int h = 0; h < (int)(4 * sizeof(T)) / 16; h++)
                    cp_async16(dst + h * (16 / sizeof(T)), src + h * (16 / sizeof(T)));
            }
    }
    cp_async_wait_all();
    T s[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int j = 0; j < NV4; j++) {
        const int e = base + 4 * (lane + 32 * j);
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (e + q >= a && e + q < b) {
                const T* gk = g + 4 * (e + q - a);
#pragma unroll
                for (int p = 0; p < 4; p++)
                    s[p] = add_rn(s[p], is_pm1<V>::value ? pm1_apply(cc[j][q], gk[p])
                                                         : mul_rn(vv[j][q], gk[p]));
            }
    }
    __syncwarp();
#pragma unroll
    for (int p = 0; p < 4; p++) s[p] = warp_sum_tree(s[p]);
    if (npieces == 1) {
        if (lane == 0) {
#pragma unroll
            for (int p = 0; p < 4; p++) epi.row_long(p, row, s[p], lid, acc);
        }
        return;
    }
    int done = 0;
    if (lane == 0) {
#pragma unroll
        for (int p = 0; p < 4; p++) A.partials[(size_t)(base_slot + piece) * 4 + p] = s[p];
        __threadfence();
        done = atomicAdd(&A.counters[lid], 1);
    }
    done = __shfl_sync(FULL_MASK, done, 0);
    if (done == npieces - 1) {
        __threadfence();
        if (lane == 0) {
#pragma unroll
            for (int p = 0; p < 4; p++) {
                T tot = T(0);
                for (int q = 0; q < npieces; q++)
                    tot = add_rn(tot, __ldcg(A.partials + (size_t)(base_slot + q) * 4 + p));
                epi.row_long(p, row, tot, lid, acc);
            }
            A.counters[lid] = 0;
        }
    }
}

template <int ITEMS, int WARPS, class V, class T, class Epi, int RPL, bool MED>
__global__ void __launch_bounds__(WARPS * 32)
    k_tiles4(CsrView<V, T> A, const T* __restrict__ x4, Epi epi) {
    __shared__ __align__(16) T prod[WARPS][4 * 32 * ITEMS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    typename Epi::Acc acc;
    epi.init(acc);
    // the grid may be capped (tiles4_grid): each warp then takes every
    // (gridDim.x * WARPS)-th task, in a fixed order, and a block's FP64 sums
    // are reduced once for all its tasks (the block reduction's FP64 shuffles
    // cost as much as the per-row terms when every block has one task each)
    const int total = A.nltasks + A.ntasks;
    for (int task = blockIdx.x * WARPS + w; task < total; task += gridDim.x * WARPS) {
        if (task < A.nltasks) {
            long_piece4<ITEMS>(A, x4, epi, acc, A.ltasks[task], lane, prod[w]);
        } else {
            const int4 t = A.tasks[task - A.nltasks];
            short_tile4<ITEMS, V, T, Epi, RPL, MED>(A, x4, epi, acc, t.x, t.y, t.z, t.w, lane,
                                                    prod[w]);
        }
        __syncwarp();
    }
    epi.finish(acc);
}

// blocks of a four-iterate pass: one task per warp, at most max_blocks (0: no
// cap); the block-partial rows of its reducing epilogue
inline unsigned tiles4_grid(const TilePlan& plan, int warps, int64_t max_blocks) {
    int64_t g = ((int64_t)plan.ntasks + plan.nltasks + warps - 1) / warps;
    if (max_blocks > 0 && g > max_blocks) g = max_blocks;
    return (unsigned)g;
}

template <int WARPS, class V, class T, class Epi>
void launch_tiles4(const TilePlan& plan, const CsrView<V, T>& view, const T* x4, const Epi& epi,
                   int64_t max_blocks, cudaStream_t s) {
    const int64_t tasks = (int64_t)plan.ntasks + plan.nltasks;
    if (tasks == 0) return;
    const unsigned grid = tiles4_grid(plan, WARPS, max_blocks);
#define CPDLP_TILES4(IT, R, M)                                                \
    prefer_l1<k_tiles4<IT, WARPS, V, T, Epi, R, M>>(WARPS * 32, s);           \
    if (!tiles_dry_run())                                                     \
        k_tiles4<IT, WARPS, V, T, Epi, R, M><<<grid, WARPS * 32, 0, s>>>(view, x4, epi)
    if (plan.medium) {
        if (plan.rpl != 2) fail(CPDLP_ERR_ARGUMENT, "tile plan with long rows needs 64-row tiles");
        switch (plan.items) {
            case 4: CPDLP_TILES4(4, 2, true); break;
            case 8: CPDLP_TILES4(8, 2, true); break;
            default: CPDLP_TILES4(16, 2, true); break;
        }
    } else {
        switch (plan.items) {
            case 4: CPDLP_TILES4(4, ROWS_PER_LANE, false); break;
            case 8: CPDLP_TILES4(8, ROWS_PER_LANE, false); break;
            default: CPDLP_TILES4(16, ROWS_PER_LANE, false); break;
        }
    }
#undef CPDLP_TILES4
    CK_LAUNCH();
}

// number of kernels launch_tiles issues for this plan
inline int tiles_launches(const TilePlan& plan) { return (plan.ntasks + plan.nltasks) ? 1 : 0; }

// block-partial rows written by a reducing epilogue (WARPS warps per block)
inline unsigned tiles_grid(const TilePlan& plan, int warps = TILE_WARPS) {
    return (unsigned)(((int64_t)plan.ntasks + plan.nltasks + warps - 1) / warps);
}

// ---- block reduction of per-thread FP64 accumulators -------------------------
// Every thread of a TILE_WARPS*32 block calls it; thread 0..Q-1 of the block
// write the block's sums to out[blockIdx.x * Q + q].
template <int Q, int W = TILE_WARPS>
__device__ __forceinline__ void block_reduce_store(const double (&v)[Q], double* out) {
    __shared__ double red[W][Q];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL_MASK, x, o);
        if (lane == 0) red[w][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < Q) {
        double s = 0.0;
#pragma unroll
        for (int ww = 0; ww < W; ww++) s += red[ww][threadIdx.x];
        out[(size_t)blockIdx.x * Q + threadIdx.x] = s;
    }
}

// Sums `nrows` rows of q partials into out[q] in a fixed order (one block);
// with nseg > 1, segment k (rows [k*nrows, (k+1)*nrows)) goes to out[k*q..].
void reduce_partials(const double* partials, int64_t nrows, int q, double* out, cudaStream_t s,
                     int nseg = 1);

}  // namespace cpdlp
