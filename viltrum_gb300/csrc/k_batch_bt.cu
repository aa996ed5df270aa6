/* batched independent integrals, nested rule pair (5-node high rule over 2-node low rule) */
#include "k_batch.cuh"

namespace vcu {
int run_batch_bt(vcu_ctx* ctx, int kind, const vcu_nested& n, const vcu_batch_item* items, uint64_t count,
                 uint32_t& launches) {
    return run_batch_pair<5, 2>(ctx, kind, n, items, count, launches);
}
}  // namespace vcu
