/*
 * k_fubini.cuh -- integrator_fubini<2>(per-bin integrator, monte_carlo(K)) with an optional
 * integrator_reorder in front (src/combination/fubini.h:75-95, reorder.h:15-58), on the device.
 *
 * The integrand is wrapped twice: Permuted (the reorder's index map, identity without reordering)
 * and TailMC<., 2> (the Monte Carlo integral of the dimensions after the first two in every
 * evaluation); the per-bin Monte Carlo kernel (k_mc.cuh) or the per-bin adaptive nested kernel
 * (k_nested.cuh) then runs unchanged on the 2-D functor over the first two dimensions of the
 * reordered range.
 */
#pragma once
#include "k_mc.cuh"
#include "k_nested.cuh"
#include "vcu_tail.cuh"

namespace vcu {

/* the problem after reordering: range permuted on the host, index map for the device */
struct FubiniPlan {
    int src[VCU_MAX_DIM];
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
};

inline int fubini_plan(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini& fb, FubiniPlan& plan) {
    if (fb.n_order < 0 || fb.n_order > VCU_REORDER_MAX_PAIRS) return fail(ctx, VCU_INVALID_ARG, "n_order must be 0..6");
    if (fb.n_order == 0) {
        for (int i = 0; i < p->dim; ++i) plan.src[i] = i;
    } else if (!reorder_map(p->dim, fb.order, fb.n_order, plan.src)) {
        return fail(ctx, VCU_INVALID_ARG, "reorder pairs must stay within the integrand's dimensions");
    }
    /* reorder(range.min(), 0) and reorder(range.max(), 1) (reorder.h:55) */
    for (int i = 0; i < p->dim; ++i) {
        plan.rmin[i] = plan.src[i] >= 0 ? p->range_min[plan.src[i]] : 0.0f;
        plan.rmax[i] = plan.src[i] >= 0 ? p->range_max[plan.src[i]] : 1.0f;
    }
    return VCU_OK;
}

/* method 0: per-bin Monte Carlo; SH/SL: the nested rule pair of method 1 */
template <int SH, int SL>
int run_fubini_pair(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini& fb, const FubiniPlan& plan,
                    const BinGrid& g, float* d_bins, uint32_t& launches) {
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        if constexpr (F::DIM < 3 && !is_unbounded<F>::value) {
            return fail(ctx, VCU_UNSUPPORTED, "a Fubini tail needs an integrand of 3 or more dimensions");
        } else {
            using P = std::conditional_t<is_unbounded<F>::value, F, Permuted<F>>;
            cv_detail::TailMC<P, 2> t{};
            if constexpr (is_unbounded<F>::value) {
                if (fb.n_order) return fail(ctx, VCU_UNSUPPORTED, "an integrand of unbounded dimension is not reordered");
                t.f = f;
                t.f.k1 ^= (uint32_t)fb.tail_seed; /* its own stream, keyed by the call too */
            } else {
                t.f.f = f;
                t.f.n = p->dim;
                for (int i = 0; i < VCU_MAX_DIM; ++i) t.f.src[i] = (int8_t)(i < p->dim ? plan.src[i] : -1);
            }
            t.full_dim = p->dim;
            t.k = fb.tail_samples;
            t.k0 = (uint32_t)fb.tail_seed;
            t.k1 = (uint32_t)(fb.tail_seed >> 32);
            t.tag = 0xF0B20000u;
            float vol = 1.0f; /* Range<Float, DIM-N>::volume(), a float product (range.h:24-25) */
            for (int d = 2; d < p->dim; ++d) {
                t.tmin[d] = plan.rmin[d];
                t.tlen[d] = vsub(plan.rmax[d], plan.rmin[d]);
                vol = vmul(vol, t.tlen[d]);
            }
            t.vol = (double)vol;
            t.factor = (double)vol / (double)fb.tail_samples;
            using T = cv_detail::TailMC<P, 2>;
            if (fb.method == VCU_FUBINI_MONTE_CARLO) {
                using namespace mc_detail;
                const unsigned blocks = (unsigned)((g.nbins + MC_WARPS - 1) / MC_WARPS);
                k_per_bin_mc<T, 2, false, false><<<blocks, MC_WARPS * 32, 0, ctx->stream>>>(
                    t, g, fb.samples_per_bin, (uint32_t)fb.seed, (uint32_t)(fb.seed >> 32), nullptr, d_bins,
                    ctx->d_status, 1.0f);
                ++launches;
                VCU_CUDA(ctx, cudaGetLastError());
                return VCU_OK;
            } else {
                return nc_detail::launch<2, SH, SL>(ctx, t, g, fb.nested, (int)fb.iterations, d_bins, nullptr,
                                                    launches);
            }
        }
    });
}

}  // namespace vcu
