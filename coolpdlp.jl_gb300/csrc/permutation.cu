// permutation.cu -- sort_rows_columns(milp) (src/components/permutation.jl:1-46):
// the LP with its variables in order of increasing column length and its
// constraints in order of increasing row length.  Host code: the reference
// runs it on the CPU before conversion, and the solver never calls it.
#include <algorithm>
#include <numeric>
#include <utility>
#include <vector>

#include "cpdlp_common.cuh"
#include "permutation.cuh"

namespace cpdlp {

namespace {

// increasing_column_order (permutation.jl:1-4): sortperm of the lengths.
// Julia's sortperm is stable, so equal lengths keep their index order.
std::vector<int64_t> stable_order(const std::vector<int64_t>& len) {
    std::vector<int64_t> p(len.size());
    std::iota(p.begin(), p.end(), int64_t(0));
    std::stable_sort(p.begin(), p.end(),
                     [&](int64_t a, int64_t b) { return len[(size_t)a] < len[(size_t)b]; });
    return p;
}

void check_csc(const cpdlp_lp& lp) {
    if (lp.m < 0 || lp.n < 0 || lp.nnz < 0) fail(CPDLP_ERR_DIMENSION, "negative size");
    if (!lp.colptr) fail(CPDLP_ERR_ARGUMENT, "null colptr");
    if (lp.nnz > 0 && (!lp.rowval || !lp.nzval)) fail(CPDLP_ERR_ARGUMENT, "null rowval / nzval");
    if (lp.colptr[0] != 1 || lp.colptr[lp.n] != lp.nnz + 1)
        fail(CPDLP_ERR_ARGUMENT, "colptr must start at 1 and end at nnz + 1");
    for (int64_t j = 0; j < lp.n; j++) {
        const int64_t a = lp.colptr[j] - 1, b = lp.colptr[j + 1] - 1;
        if (b < a) fail(CPDLP_ERR_ARGUMENT, "colptr must be nondecreasing");
        for (int64_t k = a; k < b; k++) {
            const int64_t r = lp.rowval[k];
            if (r < 1 || r > lp.m) fail(CPDLP_ERR_ARGUMENT, "row index out of range");
            if (k > a && r <= lp.rowval[k - 1])
                fail(CPDLP_ERR_ARGUMENT, "row indices must be strictly ascending in each column");
        }
    }
}

}  // namespace

void sort_rows_columns(const cpdlp_lp& lp, int64_t* perm_var, int64_t* perm_cons,
                       int64_t* colptr_out, int64_t* rowval_out, double* nzval_out, double* c_out,
                       double* lv_out, double* uv_out, double* lc_out, double* uc_out) {
    check_csc(lp);
    const int64_t m = lp.m, n = lp.n;
    std::vector<int64_t> collen((size_t)n), rowlen((size_t)m, 0);
    for (int64_t j = 0; j < n; j++) collen[(size_t)j] = lp.colptr[j + 1] - lp.colptr[j];
    for (int64_t k = 0; k < lp.nnz; k++) rowlen[(size_t)(lp.rowval[k] - 1)]++;
    // perm_var = increasing_column_order(A), perm_cons = increasing_column_order(At)
    const std::vector<int64_t> pv = stable_order(collen), pc = stable_order(rowlen);
    std::vector<int64_t> inv_cons((size_t)m);
    for (int64_t k = 0; k < m; k++) inv_cons[(size_t)pc[(size_t)k]] = k;
    if (perm_var)
        for (int64_t k = 0; k < n; k++) perm_var[k] = pv[(size_t)k] + 1;
    if (perm_cons)
        for (int64_t k = 0; k < m; k++) perm_cons[k] = pc[(size_t)k] + 1;
    // permute_rows_columns (permutation.jl:6-14): B = A[perm_cons, perm_var],
    // column k of B is column perm_var[k] of A with its rows relabelled by the
    // inverse constraint permutation and sorted again
    if (colptr_out || rowval_out || nzval_out) {
        std::vector<std::pair<int64_t, double>> col;
        int64_t pos = 0;
        if (colptr_out) colptr_out[0] = 1;
        for (int64_t k = 0; k < n; k++) {
            const int64_t j = pv[(size_t)k];
            const int64_t a = lp.colptr[j] - 1, b = lp.colptr[j + 1] - 1;
            col.clear();
            for (int64_t e = a; e < b; e++)
                col.emplace_back(inv_cons[(size_t)(lp.rowval[e] - 1)], lp.nzval[e]);
            std::sort(col.begin(), col.end(),
                      [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
                          return x.first < y.first;
                      });
            for (const auto& rv : col) {
                if (rowval_out) rowval_out[pos] = rv.first + 1;
                if (nzval_out) nzval_out[pos] = rv.second;
                pos++;
            }
            if (colptr_out) colptr_out[k + 1] = pos + 1;
        }
    }
    auto gather = [](const double* in, const std::vector<int64_t>& p, double* out) {
        if (!out) return;
        if (!in) fail(CPDLP_ERR_ARGUMENT, "null input vector for a requested output");
        for (size_t k = 0; k < p.size(); k++) out[k] = in[p[k]];
    };
    gather(lp.c, pv, c_out);
    gather(lp.lv, pv, lv_out);
    gather(lp.uv, pv, uv_out);
    gather(lp.lc, pc, lc_out);
    gather(lp.uc, pc, uc_out);
}

}  // namespace cpdlp
