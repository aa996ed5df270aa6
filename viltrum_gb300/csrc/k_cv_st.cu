/* control variates + residual Monte Carlo, rule pair (3 nodes, 2 nodes); see k_cv.cuh */
#include "k_cv.cuh"

namespace vcu {
int run_cv_st(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
              const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
              uint32_t& launches) {
    return run_cv_pair<3, 2>(ctx, p, g, n, iterations, cv, d_replay, d_bins, d_approx, d_regions, launches);
}
int run_tol_st(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, float tol,
               uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches) {
    return run_tol_pair<3, 2>(ctx, p, g, n, tol, max_regions, d_bins, nregions, nleaves, launches);
}
}  // namespace vcu
