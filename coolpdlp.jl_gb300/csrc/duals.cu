// duals.cu -- the reduced costs and the dual objective the MOI wrapper reports
// (src/moi.jl:215-227), on the device:
//   z = proj_multiplier.(c .- A'y, lv, uv)
//   dual objective = sum safeprod_left(lc, y+) - sum safeprod_left(uc, y-)
//                  + sum safeprod_left(lv, z+) - sum safeprod_left(uv, z-)
// in FP64 from the LP's original (unscaled) data.  (A'y)_j runs over column j
// of A in its row order, the order of the reference's CSC product At * y.
#include "duals.cuh"

#include "tiles.cuh"

namespace cpdlp {
namespace {

constexpr int DU_THREADS = TILE_WARPS * 32;

// one thread per variable j: z_j and its dual-objective terms
__global__ void __launch_bounds__(DU_THREADS)
    k_reduced_costs(const int64_t* __restrict__ colptr1, const int64_t* __restrict__ rowval1,
                    const double* __restrict__ nzval, const double* __restrict__ y,
                    const double* __restrict__ c, const double* __restrict__ lv,
                    const double* __restrict__ uv, int64_t n, double* __restrict__ z,
                    double* __restrict__ part) {
    double acc[1] = {0.0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        double s = 0.0;
        for (int64_t k = colptr1[j] - 1; k < colptr1[j + 1] - 1; k++)
            s = __dadd_rn(s, __dmul_rn(nzval[k], y[rowval1[k] - 1]));
        const double zj = proj_multiplier(__dsub_rn(c[j], s), lv[j], uv[j]);
        z[j] = zj;
        acc[0] += __dsub_rn(safeprod_left(lv[j], pos_part(zj)), safeprod_left(uv[j], neg_part(zj)));
    }
    block_reduce_store<1>(acc, part);
}
// the constraint rows' terms
__global__ void __launch_bounds__(DU_THREADS)
    k_row_terms(const double* __restrict__ y, const double* __restrict__ lc,
                const double* __restrict__ uc, int64_t m, double* __restrict__ part) {
    double acc[1] = {0.0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
        acc[0] += __dsub_rn(safeprod_left(lc[i], pos_part(y[i])), safeprod_left(uc[i], neg_part(y[i])));
    block_reduce_store<1>(acc, part);
}

}  // namespace

void reduced_costs(Handle& h, const cpdlp_lp* lp, const double* y, double* z_out,
                   double* dual_objective) {
    if (!lp || !y) fail(CPDLP_ERR_ARGUMENT, "null lp or y");
    const int64_t m = lp->m, n = lp->n, nnz = lp->nnz;
    if (m < 0 || n < 0 || nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative problem size");
    if (n > 0 && (!lp->colptr || !lp->c || !lp->lv || !lp->uv))
        fail(CPDLP_ERR_ARGUMENT, "null variable arrays");
    if (m > 0 && (!lp->lc || !lp->uc)) fail(CPDLP_ERR_ARGUMENT, "null constraint bounds");
    if (nnz > 0 && (!lp->rowval || !lp->nzval)) fail(CPDLP_ERR_ARGUMENT, "null matrix arrays");
    if (n > 0 && (lp->colptr[0] != 1 || lp->colptr[n] - 1 != nnz))
        fail(CPDLP_ERR_DIMENSION, "colptr does not describe nnz entries");
    for (int64_t k = 0; k < nnz; k++)
        if (lp->rowval[k] < 1 || lp->rowval[k] > m)
            fail(CPDLP_ERR_ARGUMENT, "row index outside 1..m");
    cudaStream_t s = h.stream;
    const size_t nz = (size_t)std::max<int64_t>(n, 1), mz = (size_t)std::max<int64_t>(m, 1);
    DBuf<int64_t> cp(nz + 1), rv((size_t)std::max<int64_t>(nnz, 1));
    DBuf<double> v((size_t)std::max<int64_t>(nnz, 1)), dy(mz), dc(nz), dlv(nz), duv(nz), dlc(mz),
        duc(mz), dz(nz);
    const int64_t gmax = (int64_t)(h.num_sms > 0 ? h.num_sms : 152) * 4;
    const unsigned gn = (unsigned)std::max<int64_t>(1, std::min<int64_t>(gmax, (n + DU_THREADS - 1) / DU_THREADS));
    const unsigned gm = (unsigned)std::max<int64_t>(1, std::min<int64_t>(gmax, (m + DU_THREADS - 1) / DU_THREADS));
    DBuf<double> part((size_t)gn + gm), out(2);
    auto up = [&](void* d, const void* hsrc, size_t bytes) {
        if (bytes) CK(cudaMemcpyAsync(d, hsrc, bytes, cudaMemcpyHostToDevice, s));
    };
    if (n > 0) {
        up(cp.p, lp->colptr, sizeof(int64_t) * (n + 1));
        up(dc.p, lp->c, sizeof(double) * n);
        up(dlv.p, lp->lv, sizeof(double) * n);
        up(duv.p, lp->uv, sizeof(double) * n);
    }
    up(rv.p, lp->rowval, sizeof(int64_t) * nnz);
    up(v.p, lp->nzval, sizeof(double) * nnz);
    if (m > 0) {
        up(dy.p, y, sizeof(double) * m);
        up(dlc.p, lp->lc, sizeof(double) * m);
        up(duc.p, lp->uc, sizeof(double) * m);
    }
    k_reduced_costs<<<gn, DU_THREADS, 0, s>>>(cp.p, rv.p, v.p, dy.p, dc.p, dlv.p, duv.p, n, dz.p,
                                              part.p);
    k_row_terms<<<gm, DU_THREADS, 0, s>>>(dy.p, dlc.p, duc.p, m, part.p + gn);
    CK_LAUNCH();
    reduce_partials(part.p, (int64_t)gn + gm, 1, out.p, s);
    double total = 0.0;
    CK(cudaMemcpyAsync(&total, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (z_out && n > 0) CK(cudaMemcpyAsync(z_out, dz.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (dual_objective) *dual_objective = total;
}

}  // namespace cpdlp
