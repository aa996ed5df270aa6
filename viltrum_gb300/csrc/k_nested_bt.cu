/* per-bin adaptive nested quadrature, rule pair (5 nodes, 2 nodes); see k_nested.cuh */
#include "k_nested.cuh"

namespace vcu {
int run_nested_bt(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                     float* d_bins, int32_t* d_trace, uint32_t& launches) {
    return run_nested_pair<5, 2>(ctx, p, g, n, iterations, d_bins, d_trace, launches);
}
}  // namespace vcu
