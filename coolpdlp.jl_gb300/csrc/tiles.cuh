// tiles.cuh -- the warp-tile CSR SpMV engine with fused per-row epilogues.
//
// Work partition (built once per matrix on the host from its row pointer):
//  * short tile  {r0, r1, -1, 0}: consecutive rows [r0, r1) holding at most
//    TILE = 32*ITEMS nonzeros and at most MAX_TILE_ROWS rows.  One warp loads
//    the tile's values and column indices coalesced into registers, writes
//    value*x[col] products to shared memory and then every lane reduces whole
//    rows in ascending column order (the reference's order) and applies the
//    epilogue of that row.
//  * long-row piece {row, piece, long_id, slot_base}: a row longer than TILE is
//    cut into TILE-sized pieces, one warp each.  Each warp writes its partial
//    sum to a scratch slot; the warp that completes the row (atomic counter,
//    no waiting) adds the partials in piece order and applies the epilogue, so
//    results do not depend on scheduling.
// All arithmetic of the row sums uses explicit round-to-nearest multiply/add
// (no FMA contraction); short rows therefore reproduce a sequential CPU sum
// exactly.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

constexpr int MAX_TILE_ROWS = 256;
constexpr unsigned FULL_MASK = 0xffffffffu;

struct TilePlan {
    int32_t rows = 0;
    int32_t items = 16;     // nonzeros per lane of a short tile
    int32_t ntasks = 0;
    int32_t nshort = 0;
    int32_t nlong = 0;      // rows longer than a tile
    int32_t npieces = 0;    // pieces of all long rows
    DBuf<int4> tasks;
    DBuf<int32_t> counters; // per long row, zero between launches
    std::vector<int32_t> long_rows;
    int tile_nnz() const { return 32 * items; }
};

// Host-side partition of the rows of a CSR (ptr on the host, 0-based, rows+1).
void build_tile_plan(const std::vector<int32_t>& ptr, int32_t rows, int items, TilePlan& plan,
                     cudaStream_t s);

// Picks nonzeros-per-lane from the mean row length (autotuner default).
int choose_items(int64_t nnz, int64_t rows, int requested_tile_nnz);

template <class V, class T>
struct CsrView {
    const int32_t* __restrict__ ptr;
    const int32_t* __restrict__ idx;
    const V* __restrict__ val;
    const int4* __restrict__ tasks;
    int32_t ntasks;
    int32_t* counters;
    T* partials;   // npieces * NVEC
};

template <class T, int NVEC>
struct VecSet {
    const T* v[NVEC];
};

template <class V, class T>
__device__ __forceinline__ T load_val(const V* p) {
    return (T)__ldcs(p);
}
template <>
__device__ __forceinline__ float load_val<int8_t, float>(const int8_t* p) {
    return (float)__ldcs(reinterpret_cast<const signed char*>(p));
}
template <>
__device__ __forceinline__ double load_val<int8_t, double>(const int8_t* p) {
    return (double)__ldcs(reinterpret_cast<const signed char*>(p));
}

template <class T>
__device__ __forceinline__ T warp_sum_tree(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = add_rn(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

// One warp processes one task.  `prod` is this warp's shared-memory slice of
// 32*ITEMS products, reused for each of the NVEC input vectors.
template <int ITEMS, int NVEC, class V, class T, class Epi>
__device__ __forceinline__ void tile_task(const CsrView<V, T>& A, const VecSet<T, NVEC>& xs,
                                          Epi& epi, typename Epi::Acc& acc, int task, int lane,
                                          T* prod) {
    constexpr int TILE = 32 * ITEMS;
    const int4 t = A.tasks[task];
    if (t.z < 0) {
        const int r0 = t.x, r1 = t.y;
        const int nz0 = __ldg(&A.ptr[r0]);
        const int len = __ldg(&A.ptr[r1]) - nz0;
        T v[ITEMS];
        int c[ITEMS];
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const int e = lane + 32 * i;
            if (e < len) {
                v[i] = load_val<V, T>(A.val + nz0 + e);
                c[i] = __ldcs(A.idx + nz0 + e);
            } else {
                v[i] = T(0);
                c[i] = 0;
            }
        }
#pragma unroll
        for (int p = 0; p < NVEC; p++) {
#pragma unroll
            for (int i = 0; i < ITEMS; i++) {
                const int e = lane + 32 * i;
                if (e < len) prod[e] = mul_rn(v[i], __ldg(xs.v[p] + c[i]));
            }
            __syncwarp();
            for (int r = r0 + lane; r < r1; r += 32) {
                const int a = __ldg(&A.ptr[r]) - nz0, b = __ldg(&A.ptr[r + 1]) - nz0;
                T s = T(0);
                for (int k = a; k < b; k++) s = add_rn(s, prod[k]);
                epi.row(p, r, s, acc);
            }
            __syncwarp();
        }
        (void)TILE;
    } else {
        const int row = t.x, piece = t.y, lid = t.z, base = t.w;
        const int rb = __ldg(&A.ptr[row]), re = __ldg(&A.ptr[row + 1]);
        const int npieces = (re - rb + TILE - 1) / TILE;
        const int a = rb + piece * TILE;
        const int b = min(a + TILE, re);
        T s[NVEC];
#pragma unroll
        for (int p = 0; p < NVEC; p++) s[p] = T(0);
        for (int e = a + lane; e < b; e += 32) {
            const T vv = load_val<V, T>(A.val + e);
            const int cc = __ldcs(A.idx + e);
#pragma unroll
            for (int p = 0; p < NVEC; p++) s[p] = add_rn(s[p], mul_rn(vv, __ldg(xs.v[p] + cc)));
        }
#pragma unroll
        for (int p = 0; p < NVEC; p++) s[p] = warp_sum_tree(s[p]);
        int done = 0;
        if (lane == 0) {
#pragma unroll
            for (int p = 0; p < NVEC; p++) A.partials[(size_t)(base + piece) * NVEC + p] = s[p];
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
                        tot = add_rn(tot, __ldcg(A.partials + (size_t)(base + q) * NVEC + p));
                    epi.row_long(p, row, tot, lid, acc);
                }
                A.counters[lid] = 0;
            }
        }
    }
}

template <int ITEMS, int WARPS, int NVEC, class V, class T, class Epi>
__global__ void __launch_bounds__(WARPS * 32)
    k_tiles(CsrView<V, T> A, VecSet<T, NVEC> xs, Epi epi) {
    __shared__ T prod[WARPS][32 * ITEMS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int task = blockIdx.x * WARPS + w;
    typename Epi::Acc acc;
    epi.init(acc);
    if (task < A.ntasks) tile_task<ITEMS, NVEC>(A, xs, epi, acc, task, lane, prod[w]);
    epi.finish(acc);
}

constexpr int TILE_WARPS = 8;

template <int NVEC, class V, class T, class Epi>
void launch_tiles(const TilePlan& plan, const CsrView<V, T>& view, const VecSet<T, NVEC>& xs,
                  const Epi& epi, cudaStream_t s) {
    if (plan.ntasks == 0) return;
    const unsigned grid = (unsigned)((plan.ntasks + TILE_WARPS - 1) / TILE_WARPS);
    switch (plan.items) {
        case 4: k_tiles<4, TILE_WARPS, NVEC, V, T, Epi><<<grid, TILE_WARPS * 32, 0, s>>>(view, xs, epi); break;
        case 8: k_tiles<8, TILE_WARPS, NVEC, V, T, Epi><<<grid, TILE_WARPS * 32, 0, s>>>(view, xs, epi); break;
        default: k_tiles<16, TILE_WARPS, NVEC, V, T, Epi><<<grid, TILE_WARPS * 32, 0, s>>>(view, xs, epi); break;
    }
    CK_LAUNCH();
}

inline unsigned tiles_grid(const TilePlan& plan) {
    return (unsigned)((plan.ntasks + TILE_WARPS - 1) / TILE_WARPS);
}

// ---- block reduction of per-thread FP64 accumulators -------------------------
// Every thread of a TILE_WARPS*32 block calls it; thread 0..Q-1 of the block
// write the block's sums to out[blockIdx.x * Q + q].
template <int Q>
__device__ __forceinline__ void block_reduce_store(const double (&v)[Q], double* out) {
    __shared__ double red[TILE_WARPS][Q];
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
        for (int ww = 0; ww < TILE_WARPS; ww++) s += red[ww][threadIdx.x];
        out[(size_t)blockIdx.x * Q + threadIdx.x] = s;
    }
}

// Sums `nblocks` rows of Q partials (plus `nextra` extra rows) into out[Q], in
// a fixed order: one block, thread-strided then tree.
void reduce_partials(const double* partials, int64_t nrows, int q, double* out, cudaStream_t s);

}  // namespace cpdlp
