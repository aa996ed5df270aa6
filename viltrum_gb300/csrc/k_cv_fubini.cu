/* control variates whose regions span the first two dimensions, the others integrated by Monte Carlo
 * inside every evaluation (a Fubini tail), rule pair (3 nodes, 2 nodes); see k_cv.cuh */
#include "k_cv.cuh"

namespace vcu {
int run_cv_fubini(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                  const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                  uint32_t& launches) {
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        if constexpr (F::DIM < 3 && !is_unbounded<F>::value) {
            return fail(ctx, VCU_UNSUPPORTED, "a Fubini tail needs an integrand of 3 or more dimensions");
        } else {
            cv_detail::TailMC<F, 2> t{};
            t.f = f;
            t.full_dim = p->dim;
            t.k = cv.tail_samples;
            /* integrator_crespo2021_infinite seeds its tail Monte Carlo with 2*seed+1 (integrator-crespo2021.h:34) */
            const uint64_t key = cv.seed * 2 + 1;
            t.k0 = (uint32_t)key;
            t.k1 = (uint32_t)(key >> 32);
            t.tag = 0xF0B10000u;
            if constexpr (is_unbounded<F>::value) t.f.k1 ^= (uint32_t)key; /* its own stream, keyed by the call too */
            float vol = 1.0f; /* Range<Float, DIM-N>::volume(), a float product (range.h) */
            for (int d = 2; d < p->dim; ++d) {
                t.tmin[d] = p->range_min[d];
                t.tlen[d] = vsub(p->range_max[d], p->range_min[d]);
                vol = vmul(vol, t.tlen[d]);
            }
            t.vol = (double)vol;
            t.factor = (double)vol / (double)cv.tail_samples;
            return cv_detail::cv_launch<2, 3, 2>(ctx, t, p, g, n, iterations, cv, d_replay, d_bins, d_approx, d_regions,
                                                 launches);
        }
    });
}
}  // namespace vcu
