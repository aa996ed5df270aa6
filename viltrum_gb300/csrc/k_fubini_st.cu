/* integrator_fubini<2> over per-bin adaptive nested quadrature, rule pair (3 nodes, 2 nodes); also
 * the per-bin Monte Carlo first integrator (st unit only); see k_fubini.cuh */
#include "k_fubini.cuh"

namespace vcu {
int run_fubini_st(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini& fb, const FubiniPlan& plan, const BinGrid& g,
                  float* d_bins, uint32_t& launches) {
    return run_fubini_pair<3, 2>(ctx, p, fb, plan, g, d_bins, launches);
}
}  // namespace vcu

namespace vcu {
int run_fubini_bs(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini& fb, const FubiniPlan& plan, const BinGrid& g,
                  float* d_bins, uint32_t& launches);
}  // namespace vcu

using namespace vcu;

extern "C" int vcu_per_bin_fubini(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini* fb, float* bins,
                                  vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    if (!p || !fb || !bins) return fail(ctx, VCU_INVALID_ARG, "null problem, Fubini options or bins");
    BinGrid full;
    int rc = make_grid(ctx, p, full);
    if (rc) return rc;
    if (fb->dims != 2) return fail(ctx, VCU_UNSUPPORTED, "the per-bin Fubini form is built for 2 leading dimensions");
    if (p->dimbins > 2) return fail(ctx, VCU_INVALID_ARG, "the bins take at most the Fubini dimensions");
    if (fb->tail_samples == 0) return fail(ctx, VCU_INVALID_ARG, "tail_samples must be >= 1");
    if (fb->method == VCU_FUBINI_MONTE_CARLO) {
        if (fb->samples_per_bin == 0 || fb->samples_per_bin > 0xffffffffull)
            return fail(ctx, VCU_INVALID_ARG, "samples per bin must be 1..2^32-1");
    } else if (fb->method == VCU_FUBINI_NESTED) {
        if (fb->iterations > 62) return fail(ctx, VCU_UNSUPPORTED, "per-bin region budget is limited to 62 splits");
        if ((rc = check_per_bin_nested(ctx, fb->nested))) return rc;
        const bool st = fb->nested.rule_hi == VCU_RULE_SIMPSON && fb->nested.rule_lo == VCU_RULE_TRAPEZOIDAL;
        const bool bs = fb->nested.rule_hi == VCU_RULE_BOOLE && fb->nested.rule_lo == VCU_RULE_SIMPSON;
        if (!st && !bs)
            return fail(ctx, VCU_UNSUPPORTED, "the per-bin Fubini form takes nested(simpson, trapezoidal) or nested(boole, simpson)");
    } else {
        return fail(ctx, VCU_INVALID_ARG, "unknown Fubini method");
    }
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    FubiniPlan plan;
    if ((rc = fubini_plan(ctx, p, *fb, plan))) return rc;
    /* the per-bin integrator's own problem: the first 2 dimensions of the reordered range */
    vcu_problem p2 = *p;
    p2.dim = 2;
    for (int d = 0; d < VCU_MAX_DIM; ++d) {
        p2.range_min[d] = d < p->dim ? plan.rmin[d] : 0.0f;
        p2.range_max[d] = d < p->dim ? plan.rmax[d] : 0.0f;
    }
    BinGrid g;
    if ((rc = make_grid(ctx, &p2, g))) return rc;
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    const size_t bbytes = g.nbins * ch * 4;
    float* dbins = bins;
    if (p->mem == VCU_MEM_HOST) {
        if ((rc = ensure(ctx, ctx->out, bbytes))) return rc;
        dbins = static_cast<float*>(ctx->out.ptr);
    }
    const bool bs = fb->method == VCU_FUBINI_NESTED && fb->nested.rule_hi == VCU_RULE_BOOLE;
    rc = bs ? run_fubini_bs(ctx, p, *fb, plan, g, dbins, scope.launches)
            : run_fubini_st(ctx, p, *fb, plan, g, dbins, scope.launches);
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST)
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
    uint64_t per_bin = fb->samples_per_bin;
    if (fb->method == VCU_FUBINI_NESTED) {
        const uint64_t S = (uint64_t)fb->nested.rule_hi;
        per_bin = S * S + fb->iterations * (S - 1) * S;
    }
    return scope.end(g.nbins * per_bin * fb->tail_samples, fb->method == VCU_FUBINI_NESTED ? g.nbins * (fb->iterations + 1) : 0);
}
