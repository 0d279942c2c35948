// tiles.cu -- host side of the warp-tile partition and the partial reduction.
#include "tiles.cuh"

namespace cpdlp {

int choose_items(int64_t nnz, int64_t rows, int requested_tile_nnz) {
    if (requested_tile_nnz > 0) {
        if (requested_tile_nnz <= 128) return 4;
        if (requested_tile_nnz <= 256) return 8;
        return 16;
    }
    // Autotuner default: the tile should hold many short rows (so that row
    // sums are sequential and the lanes stay busy) while a warp issues enough
    // independent loads; 512 nonzeros per warp for typical LPs, smaller tiles
    // for very sparse matrices so that the grid still fills 152 SMs.
    double mean = rows > 0 ? (double)nnz / (double)rows : 0.0;
    if (nnz < 152LL * 8 * 128) return 4;
    if (mean < 2.0 || nnz < 152LL * 8 * 512 * 2) return 8;
    return 16;
}

void build_tile_plan(const std::vector<int32_t>& ptr, int32_t rows, int items, TilePlan& plan,
                     cudaStream_t s, const std::vector<int64_t>* seg_rows,
                     std::vector<int32_t>* seg_tasks, std::vector<int32_t>* seg_ltasks,
                     std::vector<int32_t>* seg_lids, int max_rows) {
    if (max_rows < 32 || max_rows > MAX_TILE_ROWS || max_rows % 32 != 0)
        fail(CPDLP_ERR_ARGUMENT, "tile row cap must be a multiple of 32 up to 128");
    plan.rows = rows;
    plan.items = items;
    const int tile = 32 * items;
    // rows of LONG_ROW+1 .. tile nonzeros stay in short tiles (summed by the
    // whole warp); with the default row cap their tiles hold at most 64 rows
    bool medium = false;
    for (int32_t r = 0; r < rows && !medium; r++) {
        const int32_t len = ptr[r + 1] - ptr[r];
        medium = len > LONG_ROW && len <= tile;
    }
    if (medium && max_rows == MAX_TILE_ROWS) max_rows = 64;
    plan.medium = medium;
    plan.rpl = max_rows / 32;
    std::vector<int4> longs, shorts;
    plan.long_rows.clear();
    int32_t slot = 0;
    const std::vector<int64_t> whole = {0, (int64_t)rows};
    const std::vector<int64_t>& segs = seg_rows ? *seg_rows : whole;
    const size_t nseg = segs.size() - 1;
    if (seg_tasks) seg_tasks->assign(nseg + 1, 0);
    if (seg_ltasks) seg_ltasks->assign(nseg + 1, 0);
    if (seg_lids) seg_lids->assign(nseg + 1, 0);
    for (size_t k = 0; k < nseg; k++) {
        if (seg_tasks) (*seg_tasks)[k] = (int32_t)shorts.size();
        if (seg_ltasks) (*seg_ltasks)[k] = (int32_t)longs.size();
        if (seg_lids) (*seg_lids)[k] = (int32_t)plan.long_rows.size();
        const int32_t end = (int32_t)segs[k + 1];
        int32_t r = (int32_t)segs[k];
        while (r < end) {
            int32_t len = ptr[r + 1] - ptr[r];
            if (len > tile) {
                // warp path: one piece per TILE nonzeros; only multi-piece rows use slots
                int32_t lid = (int32_t)plan.long_rows.size();
                int32_t np = (len + tile - 1) / tile;
                for (int32_t p = 0; p < np; p++) longs.push_back(make_int4(r, -(p + 1), lid, slot));
                plan.long_rows.push_back(r);
                if (np > 1) slot += np;
                r++;
                continue;
            }
            int32_t r0 = r, nz = 0;
            while (r < end && r - r0 < max_rows) {
                int32_t l = ptr[r + 1] - ptr[r];
                if (l > tile || nz + l > tile) break;
                nz += l;
                r++;
            }
            shorts.push_back(make_int4(r0, r, ptr[r0], ptr[r]));
        }
    }
    if (seg_tasks) (*seg_tasks)[nseg] = (int32_t)shorts.size();
    if (seg_ltasks) (*seg_ltasks)[nseg] = (int32_t)longs.size();
    if (seg_lids) (*seg_lids)[nseg] = (int32_t)plan.long_rows.size();
    plan.nlong = (int32_t)plan.long_rows.size();
    plan.npieces = slot;
    plan.nshort = (int32_t)shorts.size();
    plan.ntasks = (int32_t)shorts.size();
    plan.nltasks = (int32_t)longs.size();
    plan.tasks.alloc(shorts.size() ? shorts.size() : 1);
    plan.ltasks.alloc(longs.size() ? longs.size() : 1);
    if (!shorts.empty())
        CK(cudaMemcpyAsync(plan.tasks.p, shorts.data(), sizeof(int4) * shorts.size(),
                           cudaMemcpyHostToDevice, s));
    if (!longs.empty())
        CK(cudaMemcpyAsync(plan.ltasks.p, longs.data(), sizeof(int4) * longs.size(),
                           cudaMemcpyHostToDevice, s));
    plan.counters.alloc(plan.nlong ? (size_t)plan.nlong : 1);
    CK(cudaMemsetAsync(plan.counters.p, 0, sizeof(int32_t) * plan.counters.n, s));
    CK(cudaStreamSynchronize(s));
}

namespace {
constexpr int RED_MAX_Q = 12;
// block b reduces segment b: rows [b*nrows, (b+1)*nrows) -> out[b*q + j].
// Each thread adds whole rows (q contiguous values) in row order, then the
// block sums its threads' values in a fixed tree: the result depends only on
// the data and the block size.
__global__ void k_reduce_partials(const double* __restrict__ part, int64_t nrows, int q,
                                  double* __restrict__ out) {
    __shared__ double red[32][RED_MAX_Q];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    part += (size_t)blockIdx.x * nrows * q;
    out += (size_t)blockIdx.x * q;
    double acc[RED_MAX_Q];
#pragma unroll
    for (int j = 0; j < RED_MAX_Q; j++) acc[j] = 0.0;
    for (int64_t r = threadIdx.x; r < nrows; r += blockDim.x) {
        const double* row = part + r * q;
#pragma unroll
        for (int j = 0; j < RED_MAX_Q; j++)
            if (j < q) acc[j] += row[j];
    }
#pragma unroll
    for (int j = 0; j < RED_MAX_Q; j++) {
        if (j >= q) break;
        double x = acc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[w][j] = x;
    }
    __syncthreads();
    if (threadIdx.x < q) {
        double t = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) t += red[ww][threadIdx.x];
        out[threadIdx.x] = t;
    }
}
}  // namespace

void reduce_partials(const double* partials, int64_t nrows, int q, double* out, cudaStream_t s,
                     int nseg) {
    if (q < 1 || q > RED_MAX_Q) fail(CPDLP_ERR_ARGUMENT, "reduce_partials: 1..12 values per row");
    // fewer threads for short inputs (the launch cost dominates there)
    const int threads = nrows >= 8192 ? 1024 : nrows >= 1024 ? 256 : 64;
    k_reduce_partials<<<nseg, threads, 0, s>>>(partials, nrows, q, out);
    CK_LAUNCH();
}

}  // namespace cpdlp
