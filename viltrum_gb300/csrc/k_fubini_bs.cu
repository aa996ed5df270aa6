/* integrator_fubini<2> over per-bin adaptive nested quadrature, rule pair (5 nodes, 3 nodes); also
 * the per-bin Monte Carlo first integrator (st unit only); see k_fubini.cuh */
#include "k_fubini.cuh"

namespace vcu {
int run_fubini_bs(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini& fb, const FubiniPlan& plan, const BinGrid& g,
                  float* d_bins, uint32_t& launches) {
    return run_fubini_pair<5, 3>(ctx, p, fb, plan, g, d_bins, launches);
}
}  // namespace vcu
