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
#include "vcu_internal.cuh"

namespace vcu {

namespace {

constexpr int MC_WARPS = 8;

template <class F, int DIM, bool REPLAY, bool ACCUM>
__global__ void __launch_bounds__(MC_WARPS * 32)
    k_per_bin_mc(const __grid_constant__ F f, const BinGrid g, uint64_t spp, uint32_t k0, uint32_t k1,
                 const float* __restrict__ points, float* __restrict__ bins, uint32_t* __restrict__ status,
                 float range_volume) {
    constexpr int CH = F::CH;
    __shared__ float stage[MC_WARPS * CH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t first = (uint64_t)blockIdx.x * MC_WARPS;
    const uint64_t bin = first + warp;
    float sum[CH], comp[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) sum[c] = comp[c] = 0.0f;
    float vol = 1.0f;
    if (bin < g.nbins) {
        float lo[DIM], w[DIM];
        uint64_t rem = bin;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            float a = g.rmin[d], b = g.rmax[d];
            if (d < g.dimbins) {
                const uint32_t pos = (uint32_t)(rem % g.res[d]);
                rem /= g.res[d];
                a = vadd(g.rmin[d], vmul((float)pos, g.drange[d]));
                b = vadd(g.rmin[d], vmul((float)(pos + 1), g.drange[d]));
            }
            lo[d] = a;
            w[d] = vsub(b, a);
            vol = vmul(vol, w[d]);
        }
        const uint32_t blo = (uint32_t)bin, bhi = (uint32_t)(bin >> 32);
        auto point = [&](uint64_t s, float* x) {
#pragma unroll
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
            if constexpr (REPLAY) {
                const float* pt = points + (bin * spp + s) * DIM;
#pragma unroll
                for (int d = 0; d < DIM; ++d) x[d] = __ldg(pt + d);
            } else {
#pragma unroll
                for (int blk = 0; blk < (DIM + 3) / 4; ++blk) {
                    const U4 r = philox4x32_10(U4{(uint32_t)s, blo, bhi, (uint32_t)blk}, k0, k1);
                    const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int d = blk * 4 + k;
                        if (d < DIM) x[d] = vadd(vmul(u01(rr[k]), w[d]), lo[d]);
                    }
                }
            }
        };
        auto kahan = [&](const float* v) {
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                const float y = vsub(v[c], comp[c]);
                const float t = vadd(sum[c], y);
                comp[c] = vsub(vsub(t, sum[c]), y);
                sum[c] = t;
            }
        };
        if constexpr (has_pair<F>::value) {
            /* samples s and s+32 of this lane as two independent chains, added in sample order */
            for (uint64_t s = lane; s < spp; s += 64) {
                const bool two = s + 32 < spp;
                float x0[F::DIM], x1[F::DIM], v0[CH], v1[CH];
                point(s, x0);
                point(two ? s + 32 : s, x1);
                f.pair(x0, x1, v0, v1);
                kahan(v0);
                if (two) kahan(v1);
            }
        } else {
            for (uint64_t s = lane; s < spp; s += 32) {
                float x[F::DIM], v[CH];
                point(s, x);
                f(x, v);
                kahan(v);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < CH; ++c) {
        double t = (double)sum[c] - (double)comp[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if (lane == 0) {
            double est;
            if constexpr (ACCUM)
                est = (bin < g.nbins ? (double)bins[bin * CH + c] : 0.0) + (double)range_volume / (double)spp * t;
            else
                est = (double)g.factor * (double)vol / (double)spp * t;
            const float e = (float)est;
            if (bin < g.nbins && isnan(e)) atomicOr(status, VCU_FLAG_NAN);
            stage[warp * CH + c] = e;
        }
    }
    __syncthreads();
    /* coalesced write of this block's MC_WARPS*CH consecutive floats */
    const uint64_t base = first * CH;
    const uint64_t total = g.nbins * CH;
    const int nvals = MC_WARPS * CH;
    if (base + nvals <= total && (((uintptr_t)(bins + base)) & 15) == 0 && (nvals % 4) == 0) {
        if (threadIdx.x < nvals / 4)
            reinterpret_cast<float4*>(bins + base)[threadIdx.x] = reinterpret_cast<const float4*>(stage)[threadIdx.x];
    } else if (threadIdx.x < nvals && base + threadIdx.x < total) {
        bins[base + threadIdx.x] = stage[threadIdx.x];
    }
}

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
