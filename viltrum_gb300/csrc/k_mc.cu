/*
 * k_mc.cu -- per-bin Monte Carlo on the device, and device evaluation of an integrand.
 *
 * Replaces the per-bin loop of integrator_per_bin_parallel(monte_carlo(samples, seed))
 * (src/integrator-per-bin-parallel.h:17-35, src/monte-carlo/monte-carlo.h:39-63) and of
 * monte_carlo_per_bin_parallel (src/monte-carlo/monte-carlo-per-bin-parallel.h:40-71).
 *
 * One warp per bin: lanes take samples j = lane, lane+32, ...; sample j of bin b reads its
 * coordinates from Philox4x32-10 (key = seed, counter = (j, b_lo, b_hi, block)) -- or, in replay
 * mode, from a caller-supplied point array -- maps them into the bin as u*(max-min)+min (the
 * reference's uniform_real_distribution arithmetic), evaluates the integrand and accumulates it
 * with a Kahan-compensated FP32 sum (integrands that evaluate two points at once take samples j and
 * j+32 together, as two independent dependency chains, and add them in sample order).  The 32 lane sums are combined by warp shuffles in FP64,
 * scaled by prod(res)*volume(bin)/samples, staged in shared memory and written with coalesced
 * stores (float4 when a block's run of bins is 16-byte aligned).
 *
 * The accumulating flavour (ACCUM) is monte_carlo_per_bin_parallel's arithmetic
 * (monte-carlo-per-bin-parallel.h:45,69): the sum is scaled by volume(range)/samples -- the whole
 * range's float volume, not prod(res)*volume(bin) -- and ADDED to the bin's current value in FP64
 * before the one rounding to float (the reference rounds after every sample).
 */
#include "k_mc.cuh"

namespace vcu {

namespace {

using namespace mc_detail;

template <class F, int DIM>
__global__ void k_eval(const __grid_constant__ F f, const float* __restrict__ x, int64_t npts, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    float xi[F::DIM];
#pragma unroll
    for (int d = 0; d < F::DIM; ++d) xi[d] = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) xi[d] = x[i * DIM + d];
    float v[F::CH];
    f(xi, v);
#pragma unroll
    for (int c = 0; c < F::CH; ++c) out[i * F::CH + c] = v[c];
}

template <class F, class Body> int by_arity(vcu_ctx* ctx, int dim, Body&& body) {
    if constexpr (F::DIM == 6) {
        switch (dim) {
        case 2: return body(std::integral_constant<int, 2>{});
        case 3: return body(std::integral_constant<int, 3>{});
        case 4: return body(std::integral_constant<int, 4>{});
        case 5: return body(std::integral_constant<int, 5>{});
        case 6: return body(std::integral_constant<int, 6>{});
        default: return fail(ctx, VCU_INVALID_ARG, "half-space dimension must be 2..6");
        }
    } else {
        return body(std::integral_constant<int, F::DIM>{});
    }
}

}  // namespace

int run_mc(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, uint64_t spp, uint64_t seed, const float* points,
           float* d_bins, bool accumulate, uint32_t& launches) {
    /* Range::volume() (range.h:24-25): the float product of the widths */
    float range_volume = 1.0f;
    for (int d = 0; d < p->dim; ++d) range_volume *= (p->range_max[d] - p->range_min[d]);
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        return by_arity<F>(ctx, p->dim, [&](auto dimc) -> int {
            constexpr int DIM = decltype(dimc)::value;
            const unsigned blocks = (unsigned)((g.nbins + MC_WARPS - 1) / MC_WARPS);
            const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
            if (points && accumulate)
                k_per_bin_mc<F, DIM, true, true><<<blocks, MC_WARPS * 32, 0, ctx->stream>>>(
                    f, g, spp, k0, k1, points, d_bins, ctx->d_status, range_volume);
            else if (points)
                k_per_bin_mc<F, DIM, true, false><<<blocks, MC_WARPS * 32, 0, ctx->stream>>>(
                    f, g, spp, k0, k1, points, d_bins, ctx->d_status, range_volume);
            else if (accumulate)
                k_per_bin_mc<F, DIM, false, true><<<blocks, MC_WARPS * 32, 0, ctx->stream>>>(
                    f, g, spp, k0, k1, nullptr, d_bins, ctx->d_status, range_volume);
            else
                k_per_bin_mc<F, DIM, false, false><<<blocks, MC_WARPS * 32, 0, ctx->stream>>>(
                    f, g, spp, k0, k1, nullptr, d_bins, ctx->d_status, range_volume);
            ++launches;
            VCU_CUDA(ctx, cudaGetLastError());
            return VCU_OK;
        });
    });
}

int run_eval(vcu_ctx* ctx, const vcu_integrand& fi, int dim, const float* d_x, int64_t npts, float* d_out,
             uint32_t& launches) {
    return with_integrand(ctx, fi, dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        return by_arity<F>(ctx, dim, [&](auto dimc) -> int {
            constexpr int DIM = decltype(dimc)::value;
            if (npts == 0) return VCU_OK;
            const unsigned blocks = (unsigned)((npts + 255) / 256);
            k_eval<F, DIM><<<blocks, 256, 0, ctx->stream>>>(f, d_x, npts, d_out);
            ++launches;
            VCU_CUDA(ctx, cudaGetLastError());
            return VCU_OK;
        });
    });
}

}  // namespace vcu
