/*
 * k_mc.cuh -- the per-bin Monte Carlo kernel template (see k_mc.cu for the method), in a header so
 * that it can be instantiated for any integrand functor: the library's built-in ones (k_mc.cu) and a
 * caller's own (include/viltrum_cuda_device.cuh).
 */
#pragma once
#include "vcu_internal.cuh"

namespace vcu {
namespace mc_detail {

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
            /* with Philox points (inside the bin) an integrand that can cull its terms to the bin's
             * box of the first two coordinates evaluates only those -- the same bits */
            [[maybe_unused]] typename cull_box_of<F>::type cl{};
            if constexpr (has_pair_cull<F>::value && !REPLAY && DIM >= 2) {
                float clo[F::DIM], chi[F::DIM];
                for (int d = 0; d < F::DIM; ++d) clo[d] = chi[d] = 0.0f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    clo[d] = lo[d];
                    chi[d] = vadd(lo[d], w[d]);
                }
                cl = f.cull_box(clo, chi);
            }
            /* samples s and s+32 of this lane as two independent chains, added in sample order */
            for (uint64_t s = lane; s < spp; s += 64) {
                const bool two = s + 32 < spp;
                float x0[F::DIM], x1[F::DIM], v0[CH], v1[CH];
                point(s, x0);
                point(two ? s + 32 : s, x1);
                if constexpr (has_pair_cull<F>::value && !REPLAY && DIM >= 2) f.pair_culled(cl, x0, x1, v0, v1);
                else f.pair(x0, x1, v0, v1);
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

}  // namespace mc_detail
}  // namespace vcu
