/*
 * k_cv.cuh -- piecewise-polynomial control variates with residual Monte Carlo on the device.
 *
 * Replaces integrator_region_based(regions_generator_adaptive_heap(nested(H,L), heuristic, iters),
 * regions_integrator_parallel_variance_reduction(rr_uniform_region(), weight, region_sampling_uniform(),
 * std::mt19937(seed), spp)) -- integrator_crespo2021 when nested = (simpson, trapezoidal) with
 * error_heuristic_size(error_metric_relative(), 1e-5) (src/control-variates/integrator-crespo2021.h:7-22).
 *
 * Three stages:
 *  1. The global region heap over the whole range, exactly as
 *     src/nested/regions-generator-adaptive-heap.h:18-45 builds it (same split choices: error
 *     estimates with the reference's rounding, libstdc++ heap order).  From 128 splits on, in waves
 *     (wave_launch, below): the regions of largest bottleneck error are split together, one warp per
 *     region, the waves decided on the device, and the host replays the heap sequence on their
 *     errors (HeapReplay, overlapping the next waves).  Below that, or when the waves
 *     give up (NaN errors, a pool overflow from masses of equal errors), k_cv_generate: ONE
 *     cooperative thread block splitting in order, the heap in shared memory (up to ~28k regions) or
 *     global memory, each split's new nodes and both children's error folds evaluated by the block
 *     in parallel.  Node values, ranges and volumes of every region built live in a global pool (a
 *     region's slot never moves; the heap holds pool ids).
 *  2. k_cv_lists (count, then fill) / k_cv_scan_* / k_cv_sort: per-bin region lists.  Every region,
 *     in heap order, is appended to the bins pixels_in_region gives (src/newton-cotes/region.h:454-463,
 *     the 0.99 rule),
 *     as the reference's stratification does (regions-integrator-parallel-variance-reduction.h:49-57):
 *     count per bin, exclusive scan, fill, then sort each bin's list by heap position so the order
 *     is the reference's sequential order.
 *  3. k_cv_residual: one warp per bin computes the control-variate integral
 *     sum_i prod(res) * integral over (bin n region_i) (:77-88), then the residual: sample j picks a
 *     region uniformly (rr_uniform_region, weight n) and a uniform point in bin n region (weight
 *     volume), pushes f*w and g*w (g = the region polynomial, region.h:103-112) into the
 *     cv_optimize_weight / cv_fixed_weight estimator (weight-strategy.h:7-110); sums in FP32 (Kahan
 *     per lane, float-float across lanes), moments FP32 per lane and float-float across lanes, the
 *     final recombination (sum_f - a*sum_g)/n + a*approximation in float-float.  Up to 3 dimensions a
 *     sample's polynomial starts from the first-fold coefficients k_cv_coef precomputes per listed
 *     region; uniform points are drawn and evaluated in pairs where the integrand has a two-point culled
 *     form.  Sample j of bin b draws from
 *     Philox4x32-10 (key = seed, counter = (j, b_lo, b_hi, 0xC0DE0000 | block)), or replays given
 *     (chosen list index, point) records.
 */
#pragma once
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "vcu_heap.h"
#include "vcu_tail.cuh"
#include "vcu_internal.cuh"
#include "vcu_pdf.cuh"
#include "vcu_rules.cuh"

namespace vcu {
namespace cv_detail {

__host__ __device__ constexpr int ipow(int b, int e) { return e <= 0 ? 1 : b * ipow(b, e - 1); }

constexpr int GEN_THREADS = 256;
constexpr int RES_WARPS = 4;
constexpr int RES_CHUNK = 128; /* region integrals staged per warp before the ordered sum */

struct GenCfg {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
    int32_t iters;
    int32_t heap_in_smem;
    int32_t heuristic, relative;
    float min_val_f;
    double size_weight, min_size;
};

template <int DIM, int S>
__device__ __forceinline__ int node_index(int d, int J, int pos) {
    int idx = 0, rem = J;
#pragma unroll
    for (int e = 0; e < DIM; ++e) {
        if (e == d) {
            idx += pos * ipow(S, e);
        } else {
            idx += (rem % S) * ipow(S, e);
            rem /= S;
        }
    }
    return idx;
}

/* the functor the residual samples with: itself, or a Fubini tail of one sample */
template <class F> F residual_functor(const F& f) { return f; }
template <class F, int N> TailMC<F, N> residual_functor(const TailMC<F, N>& g) {
    TailMC<F, N> r = g;
    r.k = 1;
    r.factor = g.vol;
    r.tag = g.tag ^ 0x00010000u;
    return r;
}

/* ---------------------------------------------------------------- stage 1: global region heap */
template <class F, int DIM, int SH, int SL>
__global__ void __launch_bounds__(GEN_THREADS, 1)
    k_cv_generate(const __grid_constant__ F f, const GenCfg cfg, float* __restrict__ vals, float* __restrict__ rmin,
                  float* __restrict__ rmax, float* __restrict__ vol, float* __restrict__ heap_key,
                  int* __restrict__ heap_pay, uint32_t* __restrict__ status) {
    constexpr int S = SH;
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    constexpr int NL = ipow(S, DIM - 1);
    constexpr int NNEW = (S - 1) * NL;
    extern __shared__ float smem[];
    /* up to two splits per round: the top region's and, speculatively, the region the sequential
     * algorithm pops next if the first split's children do not overtake it */
    __shared__ float CO[2][DIM * S], CN[2][S - 1];
    __shared__ float LN[4 * DIM * NL], LF[(4 * DIM * NL + S - 1) / S];
    __shared__ float EC[4 * DIM];
    __shared__ float VC[4][SD * CH]; /* the children of the round's splits, on chip */
    __shared__ int s_top[2], s_nspec, s_adv;
    const int nheap = cfg.iters + 1;
    float* HE = cfg.heap_in_smem ? smem : heap_key;
    int* HS = cfg.heap_in_smem ? reinterpret_cast<int*>(smem + nheap) : heap_pay;
    const int tid = threadIdx.x;

    /* error estimates of the regions whose node values are R0 (and R1) into EC[r*DIM + d]
     * (region.h:379-418): line metrics with compile-time strides, then the folds level by level */
    auto errors = [&](int nreg, const int* rid) {
        static_for<DIM>([&](auto dc) {
            constexpr int d = decltype(dc)::value;
            constexpr int PD = ipow(S, d);
            for (int t = tid; t < nreg * NL; t += GEN_THREADS) {
                const int r = t / NL;
                const int J = t - r * NL;
                const float* RV = VC[r] + (J % PD + (J / PD) * (PD * S)) * CH;
                float m = 0.0f;
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    float line[S], low[SL];
#pragma unroll
                    for (int i = 0; i < S; ++i) line[i] = RV[i * PD * CH + c];
#pragma unroll
                    for (int i = 0; i < SL; ++i) low[i] = line[i * (S - 1) / (SL - 1)];
                    float H, L;
                    if constexpr (CH == 1) {
                        H = RefRule<S>::scalar(line);
                        L = RefRule<SL>::scalar(low);
                    } else {
                        H = RefRule<S>::rgb(line);
                        L = RefRule<SL>::rgb(low);
                    }
                    const float mv = metric_value(cfg.relative, cfg.min_val_f, H, L);
                    m = (c == 0) ? mv : vadd(m, mv);
                }
                LN[(r * DIM + d) * NL + J] = m;
            }
        });
        __syncthreads();
        float* src = LN;
        float* dst = LF;
        static_for<DIM - 1>([&](auto lc) {
            constexpr int n = NL / ipow(S, decltype(lc)::value), m = n / S;
            for (int t = tid; t < nreg * DIM * m; t += GEN_THREADS) {
                const int rd = t / m, i = t - rd * m;
                float tmp[S];
#pragma unroll
                for (int j = 0; j < S; ++j) tmp[j] = src[rd * n + i * S + j];
                dst[rd * m + i] = RefRule<S>::scalar(tmp);
            }
            __syncthreads();
            float* sw = src;
            src = dst;
            dst = sw;
        });
        if (tid < nreg * DIM) EC[tid] = vmul(vol[rid[tid / DIM]], src[tid]);
        __syncthreads();
    };
    auto heuristic = [&](int r, int id, float& err_out, int& dim_out) {
        const float* e = EC + r * DIM;
        if (cfg.heuristic == VCU_HEUR_DEFAULT) {
            float max_err = 0.0f;
            int max_dim = 0;
            for (int d = 0; d < DIM; ++d)
                if (e[d] > max_err) {
                    max_err = e[d];
                    max_dim = d;
                }
            err_out = max_err;
            dim_out = max_dim;
            return;
        }
        float w = vsub(rmax[id * DIM], rmin[id * DIM]);
        float max_err;
        if ((double)w < cfg.min_size || isnan(w)) max_err = 0.0f;
        else max_err = __double2float_rn(__dadd_rn((double)e[0], __dmul_rn(cfg.size_weight, (double)fabsf(w))));
        int max_dim = 0;
        for (int d = 1; d < DIM; ++d) {
            w = vsub(rmax[id * DIM + d], rmin[id * DIM + d]);
            float err = __double2float_rn(__dadd_rn((double)e[d], __dmul_rn(cfg.size_weight, (double)fabsf(w))));
            if ((double)w < cfg.min_size) err = 0.0f;
            if (err >= max_err) {
                max_err = err;
                max_dim = d;
            }
        }
        err_out = max_err;
        dim_out = max_dim;
    };

    /* root region: the whole range (regions-generator-adaptive-heap.h:27) */
    if (tid == 0) {
        float v = 1.0f;
        for (int d = 0; d < DIM; ++d) {
            rmin[d] = cfg.rmin[d];
            rmax[d] = cfg.rmax[d];
            v = vmul(v, vsub(cfg.rmax[d], cfg.rmin[d]));
        }
        vol[0] = v;
    }
    for (int t = tid; t < DIM * S; t += GEN_THREADS) {
        const int d = t / S, j = t % S;
        CO[0][t] = node_coord(node_pos<S>(j), vsub(cfg.rmax[d], cfg.rmin[d]), cfg.rmin[d]);
    }
    __syncthreads();
    for (int t = tid; t < SD; t += GEN_THREADS) {
        float x[F::DIM];
        for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
        int rem = t;
        for (int d = 0; d < DIM; ++d) {
            x[d] = CO[0][d * S + rem % S];
            rem /= S;
        }
        float v[CH];
        f(x, v);
        for (int c = 0; c < CH; ++c) {
            vals[t * CH + c] = v[c];
            VC[0][t * CH + c] = v[c];
        }
    }
    __syncthreads();
    {
        const int rid0[1] = {0};
        errors(1, rid0);
    }
    if (tid == 0) {
        float e;
        int dm;
        heuristic(0, 0, e, dm);
        HE[0] = e;
        HS[0] = 0 | (dm << 24);
    }
    constexpr int TB = NNEW + S * NL; /* tasks of one split's children */
    int it = 0;
    while (it < cfg.iters) {
        __syncthreads();
        if (tid == 0) {
            const int n = it + 1; /* heap size */
            s_top[0] = HS[0];
            int nspec = 1;
            if (it + 1 < cfg.iters && n >= 2) {
                /* the element libstdc++'s pop moves to the root: the right child unless it is less */
                const int c = (n >= 3 && !(HE[2] < HE[1])) ? 2 : 1;
                s_top[1] = HS[c];
                nspec = 2;
            }
            s_nspec = nspec;
        }
        __syncthreads();
        const int nspec = s_nspec;
        for (int t = tid; t < nspec * (DIM * S + (S - 1)); t += GEN_THREADS) {
            const int q = t / (DIM * S + (S - 1)), u = t - q * (DIM * S + (S - 1));
            const int P = s_top[q] & 0xffffff, dd = s_top[q] >> 24;
            const float* pmin = rmin + (size_t)P * DIM;
            const float* pmax = rmax + (size_t)P * DIM;
            if (u < DIM * S) {
                const int d = u / S, j = u % S;
                CO[q][u] = node_coord(node_pos<S>(j), vsub(pmax[d], pmin[d]), pmin[d]);
            } else {
                const int k = u - DIM * S;
                CN[q][k] = node_coord(mid_pos<S>(k), vsub(pmax[dd], pmin[dd]), pmin[dd]);
            }
        }
        __syncthreads();
        /* new nodes at the odd positions, parent nodes at the even (region.h:345-359, split.h:13-49),
         * built on chip and copied to the pool (split q writes pool ids 2(it+q)+1, 2(it+q)+2); one
         * instance per split dimension */
        auto build_children = [&](auto ddc, int q, int u) {
            constexpr int DD = decltype(ddc)::value;
            constexpr int PD = ipow(S, DD);
            const int P = s_top[q] & 0xffffff;
            const float* VP = vals + (size_t)P * SD * CH;
            float* V0 = vals + (size_t)(2 * (it + q) + 1) * SD * CH;
            float* V1 = vals + (size_t)(2 * (it + q) + 2) * SD * CH;
            const bool fresh = u < NNEW;
            const int w = fresh ? u : u - NNEW;
            const int k = w / NL, J = w - k * NL;
            const int base = J % PD + (J / PD) * (PD * S);
            float v[CH];
            int i;
            if (fresh) {
                float x[F::DIM];
#pragma unroll
                for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
                static_for<DIM>([&](auto ec) {
                    constexpr int e = decltype(ec)::value;
                    if constexpr (e != DD) {
                        constexpr int pe = e < DD ? ipow(S, e) : ipow(S, e - 1);
                        x[e] = CO[q][e * S + (J / pe) % S];
                    }
                });
                x[DD] = CN[q][k];
                f(x, v);
                i = 2 * k + 1;
            } else {
#pragma unroll
                for (int c = 0; c < CH; ++c) v[c] = VP[(base + k * PD) * CH + c];
                i = 2 * k;
            }
            if (i <= S - 1) {
                const int n0 = (base + i * PD) * CH;
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    VC[2 * q][n0 + c] = v[c];
                    V0[n0 + c] = v[c];
                }
            }
            if (i >= S - 1) {
                const int n1 = (base + (i - (S - 1)) * PD) * CH;
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    VC[2 * q + 1][n1 + c] = v[c];
                    V1[n1 + c] = v[c];
                }
            }
        };
        for (int t = tid; t < nspec * TB; t += GEN_THREADS) {
            const int q = t / TB, u = t - q * TB;
            const int dd = s_top[q] >> 24;
            static_for<DIM>([&](auto dc) {
                if (dd == decltype(dc)::value) build_children(dc, q, u);
            });
        }
        if (tid == 0) {
            for (int q = 0; q < nspec; ++q) {
                const int P = s_top[q] & 0xffffff, dd = s_top[q] >> 24;
                const int C0 = 2 * (it + q) + 1, C1 = 2 * (it + q) + 2;
                const float* pmin = rmin + (size_t)P * DIM;
                const float* pmax = rmax + (size_t)P * DIM;
                const float pmn = pmin[dd], pmx = pmax[dd];
                const float half = vmul(vsub(pmx, pmn), 0.5f); /* = (max - min) / 2.0, exactly */
                const float mid = vadd(pmn, vmul(half, 1.0f));
                float v0 = 1.0f, v1 = 1.0f;
                for (int d = 0; d < DIM; ++d) {
                    const float mn = pmin[d], mx = pmax[d];
                    const float mx0 = (d == dd) ? mid : mx;
                    const float mn1 = (d == dd) ? mid : mn;
                    rmin[(size_t)C0 * DIM + d] = mn;
                    rmax[(size_t)C0 * DIM + d] = mx0;
                    rmin[(size_t)C1 * DIM + d] = mn1;
                    rmax[(size_t)C1 * DIM + d] = mx;
                    v0 = vmul(v0, vsub(mx0, mn));
                    v1 = vmul(v1, vsub(mx, mn1));
                }
                vol[C0] = v0;
                vol[C1] = v1;
            }
        }
        __syncthreads();
        {
            const int rid[4] = {2 * it + 1, 2 * it + 2, 2 * it + 3, 2 * it + 4};
            errors(2 * nspec, rid);
        }
        if (tid == 0) {
            /* commit the first split; commit the second only if the heap now really has it on top
             * (same entry), which is exactly what the sequential algorithm would pop next */
            int adv = 0;
            for (int q = 0; q < nspec; ++q) {
                if (q == 1 && HS[0] != s_top[1]) break;
                const int C0 = 2 * (it + q) + 1, C1 = 2 * (it + q) + 2;
                float e0, e1;
                int d0, d1;
                heuristic(2 * q, C0, e0, d0);
                heuristic(2 * q + 1, C1, e1, d1);
                const int n = it + q + 1;
                heap_pop(HE, HS, n);
                HE[n - 1] = e0;
                HS[n - 1] = C0 | (d0 << 24);
                heap_push(HE, HS, n);
                HE[n] = e1;
                HS[n] = C1 | (d1 << 24);
                heap_push(HE, HS, n + 1);
                ++adv;
            }
            s_adv = adv;
        }
        __syncthreads();
        it += s_adv;
    }
    __syncthreads();
    if (cfg.heap_in_smem)
        for (int t = tid; t < nheap; t += GEN_THREADS) {
            heap_key[t] = HE[t];
            heap_pay[t] = HS[t];
        }
}

/* ---------------------------------------------------------------- stage 2: per-bin lists */
struct ListCfg {
    float rmin[VCU_MAX_DIMBINS], rmax[VCU_MAX_DIMBINS];
    uint32_t res[VCU_MAX_DIMBINS];
    int32_t dim, dimbins, nheap;
};

/* bins [st, en) a region covers along the binned dims (pixels_in_region, region.h:454-463) */
__device__ __forceinline__ void region_bins(const ListCfg& c, const float* rmn, const float* rmx, uint32_t* st,
                                            uint32_t* en) {
    for (int i = 0; i < c.dimbins; ++i) {
        const float w = vsub(c.rmax[i], c.rmin[i]);
        const float a = vdiv(vmul((float)c.res[i], vsub(rmn[i], c.rmin[i])), w);
        const float b = vadd(0.99f, vdiv(vmul((float)c.res[i], vsub(rmx[i], c.rmin[i])), w));
        const uint32_t s = a > 0.0f ? (uint32_t)a : 0u;
        uint32_t e = b > 0.0f ? (uint32_t)b : 0u;
        if (e > c.res[i]) e = c.res[i];
        if (e < s + 1) e = s + 1;
        st[i] = s;
        en[i] = e;
    }
}

/* one warp per heap position: count (mode 0) or fill (mode 1) the bins of its region */
static __global__ void k_cv_lists(const ListCfg c, const int* __restrict__ heap_pay, const float* __restrict__ rmin,
                           const float* __restrict__ rmax, uint32_t* __restrict__ counts,
                           const uint32_t* __restrict__ offsets, uint32_t* __restrict__ cursor,
                           uint32_t* __restrict__ lists, int mode) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= c.nheap) return;
    const int id = heap_pay[warp] & 0xffffff;
    uint32_t st[VCU_MAX_DIMBINS], en[VCU_MAX_DIMBINS];
    region_bins(c, rmin + (size_t)id * c.dim, rmax + (size_t)id * c.dim, st, en);
    uint64_t area = 1;
    for (int i = 0; i < c.dimbins; ++i) area *= (en[i] - st[i]);
    for (uint64_t q = lane; q < area; q += 32) {
        uint64_t rem = q, bin = 0, mul = 1;
        for (int i = 0; i < c.dimbins; ++i) {
            const uint32_t ext = en[i] - st[i];
            bin += (st[i] + rem % ext) * mul;
            rem /= ext;
            mul *= c.res[i];
        }
        if (mode == 0) atomicAdd(&counts[bin], 1u);
        else lists[offsets[bin] + atomicAdd(&cursor[bin], 1u)] = (uint32_t)warp;
    }
}

/* exclusive scan of the bin counts into the list offsets, in three coalesced passes: per block of
 * SCAN_TILE counts a block-local scan and the block's total (k_cv_scan_tiles), one block scanning the
 * totals (k_cv_scan_totals, which also writes offsets[n] and flags a total beyond 32 bits), and the
 * tiles' bases added (k_cv_scan_add) */
constexpr int SCAN_THREADS = 256, SCAN_PER = 4, SCAN_TILE = SCAN_THREADS * SCAN_PER;

/* inclusive scan of v over the block's threads (warp shuffles, then the warp totals) */
__device__ __forceinline__ uint64_t block_inclusive_scan(uint64_t v, uint64_t* warp_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint64_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    return v + (warp ? warp_tot[warp - 1] : 0);
}

static __global__ void __launch_bounds__(SCAN_THREADS)
    k_cv_scan_tiles(const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets, uint64_t n,
                    uint64_t* __restrict__ tile_tot) {
    __shared__ uint64_t wt[32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_PER;
    uint32_t c[SCAN_PER];
    uint64_t sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        c[k] = base + k < n ? counts[base + k] : 0u;
        sum += c[k];
    }
    const uint64_t incl = block_inclusive_scan(sum, wt);
    uint64_t acc = incl - sum; /* exclusive within the tile */
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        if (base + k < n) offsets[base + k] = (uint32_t)acc;
        acc += c[k];
    }
    if (threadIdx.x == SCAN_THREADS - 1) tile_tot[blockIdx.x] = incl;
}

static __global__ void __launch_bounds__(SCAN_THREADS)
    k_cv_scan_totals(uint64_t* __restrict__ tile_tot, uint64_t ntiles, uint32_t* __restrict__ offsets, uint64_t n,
                     uint32_t* __restrict__ status) {
    __shared__ uint64_t wt[32];
    uint64_t carry = 0;
    for (uint64_t b = 0; b < ntiles; b += SCAN_THREADS) {
        const uint64_t i = b + threadIdx.x;
        const uint64_t v = i < ntiles ? tile_tot[i] : 0;
        const uint64_t incl = block_inclusive_scan(v, wt);
        if (i < ntiles) tile_tot[i] = carry + incl - v; /* exclusive base of tile i */
        __syncthreads();
        if (threadIdx.x == SCAN_THREADS - 1) wt[0] = incl; /* this chunk's total */
        __syncthreads();
        carry += wt[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (carry > 0xffffffffull) atomicOr(status, VCU_FLAG_OVERFLOW);
        offsets[n] = (uint32_t)carry;
    }
}

static __global__ void k_cv_scan_add(uint32_t* __restrict__ offsets, uint64_t n, const uint64_t* __restrict__ tile_tot) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) offsets[i] += (uint32_t)tile_tot[i / SCAN_TILE];
}

/* sort each bin's list by heap position (rank sort by one warp per bin) */
static __global__ void k_cv_sort(const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ in,
                          uint32_t* __restrict__ out, uint64_t nbins) {
    const uint64_t bin = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (bin >= nbins) return;
    const uint32_t a = offsets[bin], n = offsets[bin + 1] - a;
    for (uint32_t i = lane; i < n; i += 32) {
        const uint32_t v = in[a + i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) rank += (in[a + j] < v) ? 1u : 0u;
        out[a + rank] = v;
    }
}

/* ---------------------------------------------------------------- stage 3: CV integral + residual */
struct ResCfg {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
    float drange[VCU_MAX_DIMBINS];
    uint32_t res[VCU_MAX_DIMBINS];
    int32_t dimbins;
    uint64_t nbins;
    double factor; /* prod(res) */
    uint64_t spp;
    uint32_t k0, k1;
    int32_t weight; /* VCU_CV_OPTIMIZE / VCU_CV_FIXED */
    double alpha;
    const float* approx_init; /* nullable: the approximation starts from these bin values */
    int32_t factor_f32;       /* prod(res) < 2^24: it converts to float exactly */
    int32_t rr;               /* VCU_RR_UNIFORM / VCU_RR_INTEGRAL / VCU_RR_ERROR / VCU_RR_PDF */
    int32_t sampling;         /* VCU_RS_UNIFORM / VCU_RS_IMPORTANCE / VCU_RS_RUSSIAN_ROULETTE / VCU_RS_MIS */
    float rr_factor;          /* VCU_RR_PDF: floor of the weights, a fraction of their mean */
    uint32_t rec_w;           /* floats per replayed sample */
    double mis_power, mis_cutoff;
    const float* rerr;        /* VCU_RR_ERROR: norm of each heap region's error estimate */
    double* cdf;              /* importance choice, per list entry: cumulative probability */
    double* rrf;              /* importance choice, per list entry: 1 / probability */
    float* var_out;           /* nullable: per bin, the estimated variance of the estimate */
};

/* rr_error_region weighs a region by norm(error()), error() = volume * (fold_all(H) - fold_all(low))
 * (region.h:422-426, nested.h:17-24, norm.h:11-24), folded from dimension 0 with the reference's
 * rounding; one thread per heap region */
template <int DIM, int SH, int SL, int CH>
__global__ void k_cv_region_error(const int* __restrict__ heap_pay, const float* __restrict__ vals,
                                  const float* __restrict__ rvol, int nheap, float* __restrict__ rerr) {
    constexpr int SD = ipow(SH, DIM);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nheap) return;
    const int id = heap_pay[k] & 0xffffff;
    const float* V = vals + (size_t)id * SD * CH;
    float nrm = 0.0f;
    for (int c = 0; c < CH; ++c) {
        float hb[SD / SH], lb[SD / SH];
        for (int i = 0; i < SD / SH; ++i) {
            float line[SH], low[SL];
#pragma unroll
            for (int j = 0; j < SH; ++j) line[j] = V[(i * SH + j) * CH + c];
#pragma unroll
            for (int j = 0; j < SL; ++j) low[j] = line[j * (SH - 1) / (SL - 1)];
            hb[i] = (CH == 1) ? RefRule<SH>::scalar(line) : RefRule<SH>::rgb(line);
            lb[i] = (CH == 1) ? RefRule<SL>::scalar(low) : RefRule<SL>::rgb(low);
        }
        for (int n = SD / SH; n > 1; n /= SH) {
            for (int i = 0; i < n / SH; ++i) {
                float line[SH], low[SL];
#pragma unroll
                for (int j = 0; j < SH; ++j) line[j] = hb[i * SH + j];
#pragma unroll
                for (int j = 0; j < SL; ++j) low[j] = lb[i * SH + j * (SH - 1) / (SL - 1)];
                hb[i] = (CH == 1) ? RefRule<SH>::scalar(line) : RefRule<SH>::rgb(line);
                lb[i] = (CH == 1) ? RefRule<SL>::scalar(low) : RefRule<SL>::rgb(low);
            }
        }
        const float e = vabs(vmul(rvol[id], vsub(hb[0], lb[0])));
        nrm = (c == 0) ? e : vadd(nrm, e);
    }
    rerr[k] = nrm;
}

template <int DIM, int S, int CH>
__device__ float poly_subrange(const float* V, int c, const float* A, const float* B) {
    constexpr int SD = ipow(S, DIM);
    constexpr int inner = SD / S;
    float buf[inner > 0 ? inner : 1];
    for (int i = 0; i < inner; ++i) {
        float line[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = V[(i + j * inner) * CH + c];
        buf[i] = (CH == 1) ? subrange_ref<S>(A[DIM - 1], B[DIM - 1], line) : Rule<S>::subrange(A[DIM - 1], B[DIM - 1], line);
    }
    int n = inner;
    for (int d = DIM - 2; d >= 0; --d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i + j * m];
            buf[i] = (CH == 1) ? subrange_ref<S>(A[d], B[d], line) : Rule<S>::subrange(A[d], B[d], line);
        }
        n = m;
    }
    return buf[0];
}

/* approximation_at (region.h:86-112): the region's polynomial at the normalised point p, folded
 * from dimension 0 with Horner's at() (rules.h:85-89, 282-286).  The first fold's S^(DIM-1) lines
 * take their power-basis coefficients from C (k_cv_coef: the same floats at() computes from the
 * node values), so a sample spends its arithmetic on the Horner steps. */
template <int DIM, int S, int CH>
__device__ float poly_at_coef(const float* C, int c, const float* p) {
    constexpr int SD = ipow(S, DIM);
    constexpr int UNROLL = SD / S <= 9 ? SD / S : 4; /* 3-D Boole: 25 lines, unrolled by 4 */
    float buf[SD / S > 0 ? SD / S : 1];
    int n = SD / S;
#pragma unroll UNROLL
    for (int i = 0; i < n; ++i) {
        float cc[S];
#pragma unroll
        for (int j = 0; j < S; ++j) cc[j] = C[(i * S + j) * CH + c];
        buf[i] = Rule<S>::horner_at(cc, p[0]);
    }
    for (int d = 1; d < DIM; ++d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i * S + j];
            buf[i] = Rule<S>::at(p[d], line);
        }
        n = m;
    }
    return vmul(buf[0], 1.0f);
}

/* the same from the node values (at() forms each line's coefficients): for more than 3 dimensions,
 * where the first fold has 81 lines, the precomputed coefficients measured no faster (2326 against
 * 2309 ms for a 5-D scene at 1024x1024 bins and 4096 samples; 3-D RGB: 5.62 against 5.72 ms) */
template <int DIM, int S, int CH>
__device__ float poly_at_nodes(const float* V, int c, const float* p) {
    constexpr int SD = ipow(S, DIM);
    float buf[SD / S > 0 ? SD / S : 1];
    int n = SD / S;
    for (int i = 0; i < n; ++i) {
        float line[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = V[(i * S + j) * CH + c];
        buf[i] = Rule<S>::at(p[0], line);
    }
    for (int d = 1; d < DIM; ++d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i * S + j];
            buf[i] = Rule<S>::at(p[d], line);
        }
        n = m;
    }
    return vmul(buf[0], 1.0f);
}
template <int DIM> __host__ __device__ constexpr bool cv_coef_pass() { return DIM <= 3; }

/* the first-fold coefficients of every listed region: coef[(k*SD + i*S + j)*CH + c] is coefficient j
 * of line i (nodes i*S .. i*S+S-1 along dimension 0) of channel c of heap entry k's region */
template <int S, int CH>
__global__ void k_cv_coef(const int* __restrict__ heap_pay, const float* __restrict__ vals, int sd, size_t nheap,
                          float* __restrict__ coef) {
    const size_t lines = (size_t)(sd / S) * CH;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nheap * lines;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t k = t / lines;
        const int r = (int)(t - k * lines), i = r / CH, c = r - i * CH;
        const size_t id = (size_t)(heap_pay[k] & 0xffffff);
        float line[S], cc[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = vals[(id * sd + i * S + j) * CH + c];
        Rule<S>::coefficients(line, cc);
#pragma unroll
        for (int j = 0; j < S; ++j) coef[(k * sd + i * S + j) * CH + c] = cc[j];
    }
}

__device__ __forceinline__ float norm1(const float* v, int ch) {
    float s = vabs(v[0]);
    for (int c = 1; c < ch; ++c) s = vadd(s, vabs(v[c]));
    return s;
}

/* float-float numbers: value = h + l with |l| <= ulp(h)/2, about 48 significant bits from FP32
 * operations (two-sum / two-product with an exact FMA; division by one Newton-style correction) */
namespace ffn {
struct FF {
    float h, l;
};
__device__ __forceinline__ FF make(float a) { return FF{a, 0.0f}; }
__device__ __forceinline__ FF norm(float s, float e) { /* |s| >= |e| */
    const float h = vadd(s, e);
    return FF{h, vsub(e, vsub(h, s))};
}
__device__ __forceinline__ FF add(FF a, FF b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    return norm(s, vadd(e, vadd(a.l, b.l)));
}
__device__ __forceinline__ FF sub(FF a, FF b) { return add(a, FF{-b.h, -b.l}); }
__device__ __forceinline__ FF mul(FF a, FF b) {
    float p, e;
    two_prod(a.h, b.h, p, e);
    return norm(p, vfma(a.h, b.l, vfma(a.l, b.h, e)));
}
__device__ __forceinline__ FF div(FF a, FF b) {
    const float q1 = vdiv(a.h, b.h);
    const FF r = sub(a, mul(b, make(q1)));
    return norm(q1, vdiv(r.h, b.h));
}
__device__ __forceinline__ FF shfl_down(FF a, int off) {
    return FF{__shfl_down_sync(0xffffffffu, a.h, off), __shfl_down_sync(0xffffffffu, a.l, off)};
}
__device__ __forceinline__ double to_double(FF a) { return (double)a.h + (double)a.l; }
}  // namespace ffn

template <class F, int DIM, int S, bool PDF>
__global__ void __launch_bounds__(RES_WARPS * 32, (!PDF && DIM <= 3) ? 6 : 1)
    k_cv_residual(const __grid_constant__ F f, const ResCfg cfg, const uint32_t* __restrict__ offsets,
                  const uint32_t* __restrict__ lists, const int* __restrict__ heap_pay, const float* __restrict__ vals,
                  const float* __restrict__ coef, const float* __restrict__ rmin, const float* __restrict__ rmax,
                  const float* __restrict__ rvol, const float* __restrict__ replay, float* __restrict__ bins,
                  float* __restrict__ approx_out, uint32_t* __restrict__ status) {
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    static_assert(!PDF || S == 3, "the pdf of a region exists for Simpson's rule only");
    __shared__ float stage[RES_WARPS][RES_CHUNK][CH];
    /* the pdf of region id over bin n region [A,B] (region.h:267-290), and at an absolute point x
     * (pdf_subrange, region.h:326-331); NV holds 3^DIM node norms, overwritten */
    float NV[PDF ? SD : 1], MV[PDF ? SD / 3 + 1 : 1];
    auto load_norms = [&](int id) {
        if constexpr (PDF) {
#pragma unroll 1
            for (int i = 0; i < SD; ++i) NV[i] = norm1(vals + ((size_t)id * SD + i) * CH, CH);
        }
    };
    auto pdf_integral = [&](int id, const float* A, const float* B) -> float {
        if constexpr (PDF) {
            load_norms(id);
            return vmul(rvol[id], pdf3::Region<DIM>::integral(NV, A, B));
        } else {
            return 0.0f;
        }
    };
    auto pdf_at = [&](int id, const float* A, const float* B, const float* x) -> float {
        if constexpr (PDF) {
            float P[DIM];
            for (int d = 0; d < DIM; ++d) {
                const float rmn = rmin[(size_t)id * DIM + d], rmx = rmax[(size_t)id * DIM + d];
                P[d] = (rmn >= rmx) ? rmn : vdiv(vsub(x[d], rmn), vsub(rmx, rmn));
            }
            load_norms(id);
            const float at = pdf3::Region<DIM>::at(NV, P);
            return vdiv(at, pdf_integral(id, A, B));
        } else {
            return 0.0f;
        }
    };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t bin = (uint64_t)blockIdx.x * RES_WARPS + warp;
    if (bin >= cfg.nbins) return;
    /* bin range (regions-integrator-parallel-variance-reduction.h:71-73) */
    float bmin[DIM], bmax[DIM];
    {
        uint64_t rem = bin;
        for (int d = 0; d < DIM; ++d) {
            bmin[d] = cfg.rmin[d];
            bmax[d] = cfg.rmax[d];
            if (d < cfg.dimbins) {
                const uint32_t pos = (uint32_t)(rem % cfg.res[d]);
                rem /= cfg.res[d];
                bmin[d] = vadd(cfg.rmin[d], vmul((float)pos, cfg.drange[d]));
                bmax[d] = vadd(cfg.rmin[d], vmul((float)(pos + 1), cfg.drange[d]));
            }
        }
    }
    const uint32_t off = offsets[bin];
    const uint32_t n = offsets[bin + 1] - off;
    /* the integrand's terms that can be non-zero in the bin (points drawn here lie in it; replayed
     * points are the caller's, so they are evaluated in full) */
    [[maybe_unused]] typename cull_box_of<F>::type cl{};
    if constexpr ((has_eval_cull<F>::value || has_pair_cull<F>::value) && F::DIM == DIM) {
        if (!replay) cl = f.cull_box(bmin, bmax);
    }
    auto isect = [&](int id, float* a, float* b, float* A, float* B, float& v, bool& empty) {
        empty = false;
        v = 1.0f;
        for (int d = 0; d < DIM; ++d) {
            const float rmn = rmin[(size_t)id * DIM + d], rmx = rmax[(size_t)id * DIM + d];
            a[d] = smax(bmin[d], rmn);
            b[d] = smax(a[d], smin(bmax[d], rmx));
            empty = empty || (a[d] >= b[d]);
            v = vmul(v, vsub(b[d], a[d]));
            A[d] = (rmn >= rmx) ? rmn : vdiv(vsub(a[d], rmn), vsub(rmx, rmn));
            B[d] = (rmn >= rmx) ? rmn : vdiv(vsub(b[d], rmn), vsub(rmx, rmn));
        }
    };
    /* control-variate integral, summed in list order as the reference does */
    float approx[CH];
    for (int c = 0; c < CH; ++c) approx[c] = cfg.approx_init ? cfg.approx_init[bin * CH + c] : 0.0f;
    for (uint32_t base = 0; base < n; base += RES_CHUNK) {
        const uint32_t m = (n - base < RES_CHUNK) ? n - base : RES_CHUNK;
        for (uint32_t i = lane; i < m; i += 32) {
            const int id = heap_pay[lists[off + base + i]] & 0xffffff;
            float a[DIM], b[DIM], A[DIM], B[DIM], v;
            bool empty;
            isect(id, a, b, A, B, v, empty);
            for (int c = 0; c < CH; ++c)
                stage[warp][i][c] = empty ? __int_as_float(0x7fc00001)
                                          : vmul(rvol[id], poly_subrange<DIM, S, CH>(vals + (size_t)id * SD * CH, c, A, B));
            if (cfg.rr == VCU_RR_INTEGRAL) /* norm(integral over bin n region); an empty one integrates to 0 */
                cfg.cdf[off + base + i] = empty ? 0.0 : (double)norm1(stage[warp][i], CH);
            else if (cfg.rr == VCU_RR_ERROR) /* norm(error) * volume(bin n region) / volume(region) */
                cfg.cdf[off + base + i] = (double)vdiv(vmul(cfg.rerr[lists[off + base + i]], v), rvol[id]);
            else if (cfg.rr == VCU_RR_PDF) /* the pdf's integral over bin n region */
                cfg.cdf[off + base + i] = empty ? 0.0 : (double)pdf_integral(id, A, B);
        }
        __syncwarp();
        if (lane == 0)
            for (uint32_t i = 0; i < m; ++i) {
                if (__float_as_int(stage[warp][i][0]) == 0x7fc00001) continue;
                for (int c = 0; c < CH; ++c) {
                    if (CH == 1) /* float += double(factor) * float */
                        approx[c] = __double2float_rn((double)approx[c] + cfg.factor * (double)stage[warp][i][c]);
                    else /* 3-channel value type: double scale rounded per channel (a float product when
                          * prod(res) is an exact float), then float add */
                        approx[c] = vadd(approx[c], cfg.factor_f32
                                                        ? vmul(stage[warp][i][c], (float)cfg.factor)
                                                        : __double2float_rn(cfg.factor * (double)stage[warp][i][c]));
                }
            }
        __syncwarp();
    }
    for (int c = 0; c < CH; ++c) {
        approx[c] = __shfl_sync(0xffffffffu, approx[c], 0);
    }
    /* importance choice among the bin's regions (region-russian-roulette.h:30-149): weights floored at
     * 1% (rr_pdf_region: its factor) of their mean (all 1 when they sum to <= 0), then
     * std::discrete_distribution's normalised
     * probabilities and their running sum, the last set to 1.  The sums are warp-parallel in FP64, so
     * they can differ from the sequential ones in the last bits. */
    if (cfg.rr != VCU_RR_UNIFORM && n > 0) {
        double* W = cfg.cdf + off;
        auto warp_sum = [&](double x) {
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            return __shfl_sync(0xffffffffu, x, 0);
        };
        double s1 = 0.0;
        for (uint32_t i = lane; i < n; i += 32) s1 += W[i];
        s1 = warp_sum(s1);
        const double floor_w = (cfg.rr == VCU_RR_PDF ? (double)cfg.rr_factor : 0.01) * s1 / (double)n;
        auto clamped = [&](double w) { return (s1 <= 0.0) ? 1.0 : (w < floor_w ? floor_w : w); };
        double s2 = 0.0;
        for (uint32_t i = lane; i < n; i += 32) s2 += clamped(W[i]);
        s2 = warp_sum(s2);
        double carry = 0.0;
        for (uint32_t b0 = 0; b0 < n; b0 += 32) {
            const uint32_t i = b0 + lane;
            const double pi = (i < n) ? clamped(W[i]) / s2 : 0.0;
            double x = pi;
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            __syncwarp();
            if (i < n) {
                W[i] = (i == n - 1) ? 1.0 : carry + x;
                cfg.rrf[off + i] = (n == 1) ? 1.0 : 1.0 / pi;
            }
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
    }
    /* residual samples */
    /* per lane, in FP32: Kahan sums of the weighted samples, and the covariance moments of the
     * sample norms (weight-strategy.h:187-208) by Welford's update.  Across lanes the sums merge as
     * float-float pairs (two-sum, FP32) and the moments by Chan's formulas in float-float, as is the
     * recombination -- FP64 runs at a small fraction of the FP32 rate here */
    float sf32[CH], cf32[CH], sa32[CH], ca32[CH];
    for (int c = 0; c < CH; ++c) sf32[c] = cf32[c] = sa32[c] = ca32[c] = 0.0f;
    float wn32 = 0.0f, mf32 = 0.0f, ma32 = 0.0f, m2a32 = 0.0f, cfa32 = 0.0f, m2f32 = 0.0f;
    const uint32_t blo = (uint32_t)bin, bhi = (uint32_t)(bin >> 32);
    /* one sample's draw: its region of the bin's list, its point, the point's weight (volume(bin n
     * region) for a uniform point, else 1/pdf) */
    auto draw = [&](uint64_t j, uint32_t& chosen, float* x, float& sfac) {
        float a[DIM], b[DIM], A[DIM], B[DIM], v;
        bool empty;
        /* region_sampling_mis's weight from the importance point's pdf (region-sampling.h:93-135);
         * also whether the uniform point is taken for a draw rr_u */
        auto mis_weight = [&](float pdf_imp, float vol, float rr_u, bool& uniform) -> float {
            const float pdf_uni = vdiv(1.0f, vol);
            float mis_imp = __double2float_rn(pow((double)pdf_imp, cfg.mis_power));
            float mis_uni = __double2float_rn(pow((double)pdf_uni, cfg.mis_power));
            float mis_sum = vadd(mis_imp, mis_uni);
            if ((double)mis_imp < cfg.mis_cutoff * (double)mis_sum) {
                mis_imp = 0.0f;
                mis_sum = mis_uni;
            }
            if ((double)mis_uni < cfg.mis_cutoff * (double)mis_sum) {
                mis_uni = 0.0f;
                mis_sum = mis_imp;
            }
            const float p_imp = ((double)pdf_imp > 1.e-10) ? vdiv(mis_imp, pdf_imp) : 0.0f;
            const float p_uni = vmul(mis_uni, vol);
            const float p_sum = vadd(p_imp, p_uni);
            uniform = rr_u < vdiv(p_uni, p_sum);
            return vdiv(p_sum, mis_sum);
        };
        auto inv_pdf = [&](float pdf, double eps) -> float {
            return ((double)pdf < eps) ? 0.0f : __double2float_rn(__ddiv_rn(1.0, (double)pdf));
        };
        if (replay) {
            const float* rec = replay + (bin * cfg.spp + j) * cfg.rec_w;
            chosen = (uint32_t)rec[0];
            if (chosen >= n) {
                atomicOr(status, VCU_FLAG_OVERFLOW);
                chosen = n - 1;
            }
            const int id = heap_pay[lists[off + chosen]] & 0xffffff;
            isect(id, a, b, A, B, v, empty);
            for (int d = 0; d < DIM; ++d) x[d] = rec[1 + d];
            sfac = v;
            if constexpr (PDF) {
                if (cfg.sampling == VCU_RS_IMPORTANCE) {
                    if (!((double)v < 1.e-5)) sfac = inv_pdf(pdf_at(id, A, B, x), 1.e-5);
                } else if (cfg.sampling == VCU_RS_RUSSIAN_ROULETTE) {
                    sfac = inv_pdf(rec[1 + DIM] != 0.0f ? pdf_at(id, A, B, x) : vdiv(1.0f, v), 1.e-10);
                } else if (cfg.sampling == VCU_RS_MIS) {
                    bool uni;
                    sfac = mis_weight(pdf_at(id, A, B, rec + 2 + DIM), v, 0.0f, uni);
                }
            }
        } else {
            const U4 r0 = philox4x32_10(U4{(uint32_t)j, blo, bhi, 0xC0DE0000u}, cfg.k0, cfg.k1);
            if (cfg.rr == VCU_RR_UNIFORM) {
                chosen = (uint32_t)(((uint64_t)r0.x * n) >> 32); /* uniform index in [0, n) */
            } else {
                /* the first running probability >= u, u uniform in [0, 1) with 53 random bits */
                const U4 r2 = philox4x32_10(U4{(uint32_t)j, blo, bhi, 0xC0DE1000u}, cfg.k0, cfg.k1);
                const double u = (double)(((uint64_t)(r2.x >> 11) << 32) | r2.y) * 0x1p-53;
                uint32_t lo = 0, hi = n - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (cfg.cdf[off + mid] < u) lo = mid + 1;
                    else hi = mid;
                }
                chosen = lo;
            }
            const int id = heap_pay[lists[off + chosen]] & 0xffffff;
            isect(id, a, b, A, B, v, empty);
            const uint32_t rr[3] = {r0.y, r0.z, r0.w};
            float u[DIM];
            for (int d = 0; d < DIM; ++d) {
                uint32_t bits;
                if (d < 3) bits = rr[d];
                else {
                    const U4 r1 = philox4x32_10(U4{(uint32_t)j, blo, bhi, 0xC0DE0001u + (uint32_t)((d - 3) / 4)},
                                                cfg.k0, cfg.k1);
                    const uint32_t q[4] = {r1.x, r1.y, r1.z, r1.w};
                    bits = q[(d - 3) % 4];
                }
                u[d] = u01(bits);
                x[d] = vadd(vmul(u[d], vsub(b[d], a[d])), a[d]);
            }
            sfac = v;
            if constexpr (PDF) {
                if (cfg.sampling != VCU_RS_UNIFORM) {
                    const int id = heap_pay[lists[off + chosen]] & 0xffffff;
                    const float rr_u =
                        u01(philox4x32_10(U4{(uint32_t)j, blo, bhi, 0xC0DE1000u}, cfg.k0, cfg.k1).z);
                    /* a point drawn from the region's pdf over bin n region (region.h:241-257) */
                    auto importance_point = [&](float* xx) {
                        float sol[DIM];
                        load_norms(id);
                        pdf3::Region<DIM>::sample(NV, MV, u, A, B, sol);
                        for (int d = 0; d < DIM; ++d) {
                            const float rmn = rmin[(size_t)id * DIM + d], rmx = rmax[(size_t)id * DIM + d];
                            xx[d] = vadd(vmul(sol[d], vsub(rmx, rmn)), rmn);
                        }
                    };
                    auto uniform_point = [&]() {
                        for (int d = 0; d < DIM; ++d) x[d] = vadd(a[d], vmul(u[d], vsub(b[d], a[d])));
                    };
                    if (cfg.sampling == VCU_RS_IMPORTANCE) { /* region-sampling.h:22-43 */
                        if (!((double)v < 1.e-5)) {
                            importance_point(x);
                            sfac = inv_pdf(pdf_at(id, A, B, x), 1.e-5);
                        }
                    } else if (cfg.sampling == VCU_RS_RUSSIAN_ROULETTE) { /* :47-81 */
                        const float pdf_imp = pdf_integral(id, A, B);
                        float pdf;
                        if (rr_u < vdiv(pdf_imp, vadd(pdf_imp, v))) {
                            importance_point(x);
                            pdf = pdf_at(id, A, B, x);
                        } else {
                            uniform_point();
                            pdf = vdiv(1.0f, v);
                        }
                        sfac = inv_pdf(pdf, 1.e-10);
                    } else { /* region_sampling_mis, :84-135 */
                        importance_point(x);
                        bool uni;
                        sfac = mis_weight(pdf_at(id, A, B, x), v, rr_u, uni);
                        if (uni) uniform_point();
                    }
                }
            }
        }
    };
    /* one sample's polynomial value, weights and moments, in sample order */
    auto accumulate = [&](uint32_t chosen, const float* x, const float* fv, float sfac) {
        const int id = heap_pay[lists[off + chosen]] & 0xffffff;
        float gv[CH], p[DIM];
        for (int d = 0; d < DIM; ++d) {
            const float rmn = rmin[(size_t)id * DIM + d], rmx = rmax[(size_t)id * DIM + d];
            p[d] = (rmn >= rmx) ? rmn : vdiv(vsub(x[d], rmn), vsub(rmx, rmn));
        }
        if constexpr (cv_coef_pass<DIM>()) {
            const float* C = coef + (size_t)lists[off + chosen] * SD * CH;
            for (int c = 0; c < CH; ++c) gv[c] = poly_at_coef<DIM, S, CH>(C, c, p);
        } else {
            for (int c = 0; c < CH; ++c) gv[c] = poly_at_nodes<DIM, S, CH>(vals + (size_t)id * SD * CH, c, p);
        }
        /* sample weights: prod(res) * 1/P(region) (n for the uniform choice) * the point's weight */
        const double rrf = (cfg.rr == VCU_RR_UNIFORM) ? (double)n : cfg.rrf[off + chosen];
        float fs[CH], as[CH];
        for (int c = 0; c < CH; ++c) {
            if (CH == 1) {
                fs[c] = __double2float_rn((double)fv[c] * cfg.factor * rrf * (double)sfac);
                as[c] = __double2float_rn((double)gv[c] * cfg.factor * rrf * (double)sfac);
            } else if (cfg.rr == VCU_RR_UNIFORM && cfg.factor_f32) {
                /* per channel each scale rounds to float once; with prod(res) and n integers below 2^24
                 * the double product of a float and either is exact, so the float products equal them */
                fs[c] = vmul(vmul(vmul(fv[c], (float)cfg.factor), (float)n), sfac);
                as[c] = vmul(vmul(vmul(gv[c], (float)cfg.factor), (float)n), sfac);
            } else { /* per channel: scales by double rounded to float, then the float point weight */
                fs[c] = vmul(__double2float_rn((double)__double2float_rn((double)fv[c] * cfg.factor) * rrf), sfac);
                as[c] = vmul(__double2float_rn((double)__double2float_rn((double)gv[c] * cfg.factor) * rrf), sfac);
            }
            float y = vsub(fs[c], cf32[c]);
            float t = vadd(sf32[c], y);
            cf32[c] = vsub(vsub(t, sf32[c]), y);
            sf32[c] = t;
            y = vsub(as[c], ca32[c]);
            t = vadd(sa32[c], y);
            ca32[c] = vsub(vsub(t, sa32[c]), y);
            sa32[c] = t;
        }
        const float nf = norm1(fs, CH), na = norm1(as, CH);
        wn32 = vadd(wn32, 1.0f);
        const float inv = vdiv(1.0f, wn32);
        const float df = vsub(nf, mf32);
        mf32 = vfma(df, inv, mf32);
        const float da = vsub(na, ma32);
        ma32 = vfma(da, inv, ma32);
        const float da2 = vsub(na, ma32);
        m2a32 = vfma(da, da2, m2a32);
        cfa32 = vfma(df, da2, cfa32);
        if (cfg.var_out) m2f32 = vfma(df, vsub(nf, mf32), m2f32);
    };
    bool paired = false;
    if constexpr (has_pair_cull<F>::value && F::DIM == DIM && !PDF) {
        if (!replay) {
            /* a lane's samples j and j + 32 drawn, evaluated together (pair_culled: the kept terms'
             * loops shared, two independent chains), then accumulated in order */
            paired = true;
            for (uint64_t j = lane; j < cfg.spp && n > 0; j += 64) {
                const bool two = j + 32 < cfg.spp;
                uint32_t c0, c1;
                float x0[F::DIM], x1[F::DIM], s0, s1;
                for (int d = 0; d < F::DIM; ++d) x0[d] = x1[d] = 0.0f;
                draw(j, c0, x0, s0);
                if (two) {
                    draw(j + 32, c1, x1, s1);
                } else {
                    c1 = c0;
                    s1 = s0;
                    for (int d = 0; d < F::DIM; ++d) x1[d] = x0[d];
                }
                float f0[CH], f1[CH];
                f.pair_culled(cl, x0, x1, f0, f1);
                accumulate(c0, x0, f0, s0);
                if (two) accumulate(c1, x1, f1, s1);
            }
        }
    }
    if (!paired)
        for (uint64_t j = lane; j < cfg.spp && n > 0; j += 32) {
            uint32_t chosen;
            float x[F::DIM];
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
            float sfac;
            draw(j, chosen, x, sfac);
            float fv[CH];
            if constexpr (has_eval_cull<F>::value && F::DIM == DIM) {
                if (!replay) f.eval_culled(cl, x, fv);
                else f(x, fv);
            } else {
                f(x, fv);
            }
            accumulate(chosen, x, fv, sfac);
        }
    /* lanes merged in FP32: each Kahan sum as the float-float pair (sum, -compensation) added with
     * two-sum, the moments by Chan's pairwise formulas (one division per step) */
    float sfh[CH], sfl[CH], sah[CH], sal[CH];
    for (int c = 0; c < CH; ++c) {
        sfh[c] = sf32[c];
        sfl[c] = -cf32[c];
        sah[c] = sa32[c];
        sal[c] = -ca32[c];
    }
    auto ff_add = [](float& h, float& l, float bh, float bl) {
        float s_, e_;
        two_sum(h, bh, s_, e_);
        e_ = vadd(e_, vadd(l, bl));
        two_sum(s_, e_, h, l);
    };
    /* the moments merge in float-float (~48 bits): alpha = cov/var can sit where a last-bit change
     * of FP32 moments moves the estimate (large sample weights whose f and g terms cancel), and FP64
     * runs at a small fraction of the FP32 rate here */
    ffn::FF mf = ffn::make(mf32), ma = ffn::make(ma32), m2a = ffn::make(m2a32), cfa = ffn::make(cfa32);
    float m2f = m2f32; /* only for the variance report: FP32 is enough */
    float wn = wn32;
    for (int off2 = 16; off2 > 0; off2 >>= 1) {
        for (int c = 0; c < CH; ++c) {
            const float bh = __shfl_down_sync(0xffffffffu, sfh[c], off2), bl = __shfl_down_sync(0xffffffffu, sfl[c], off2);
            const float ch_ = __shfl_down_sync(0xffffffffu, sah[c], off2), cl = __shfl_down_sync(0xffffffffu, sal[c], off2);
            ff_add(sfh[c], sfl[c], bh, bl);
            ff_add(sah[c], sal[c], ch_, cl);
        }
        const float nb = __shfl_down_sync(0xffffffffu, wn, off2);
        const ffn::FF mfb = ffn::shfl_down(mf, off2), mab = ffn::shfl_down(ma, off2);
        const ffn::FF m2b = ffn::shfl_down(m2a, off2), cb = ffn::shfl_down(cfa, off2);
        const float m2fb = __shfl_down_sync(0xffffffffu, m2f, off2);
        const float nt = vadd(wn, nb); /* counts: exact */
        if (nb > 0.0f && nt > 0.0f) {
            const ffn::FF r = ffn::div(ffn::make(nb), ffn::make(nt));
            const ffn::FF dfm = ffn::sub(mfb, mf), dam = ffn::sub(mab, ma);
            const ffn::FF w = ffn::mul(ffn::make(wn), r);
            m2f = m2f + m2fb + dfm.h * dfm.h * w.h;
            mf = ffn::add(mf, ffn::mul(dfm, r));
            ma = ffn::add(ma, ffn::mul(dam, r));
            m2a = ffn::add(m2a, ffn::add(m2b, ffn::mul(ffn::mul(dam, dam), w)));
            cfa = ffn::add(cfa, ffn::add(cb, ffn::mul(ffn::mul(dfm, dam), w)));
            wn = nt;
        }
    }
    if (lane != 0) return;
    /* the recombination (sum_f - a sum_g)/n + a approximation (weight-strategy.h:94-101) in
     * float-float too: each FP64 instruction costs the whole warp's issue slots many times over on
     * this part, and ~48 bits leave the float result unchanged but for rare last-bit ties */
    using ffn::FF;
    auto exact_ff = [](double v) { /* v's nearest float-float */
        const float h = __double2float_rn(v);
        return FF{h, __double2float_rn(v - (double)h)};
    };
    const FF N = (n > 0) ? exact_ff((double)cfg.spp) : ffn::make(0.0f);
    FF alpha = ffn::make(1.0f);
    bool use_approx = (n == 0 || cfg.spp == 0); /* no residual samples: the approximation alone */
    if (cfg.weight == VCU_CV_FIXED) {
        alpha = exact_ff(cfg.alpha);
    } else {
        use_approx = use_approx || N.h < 2.0f;
        if (!use_approx) {
            const FF nm1 = ffn::sub(N, ffn::make(1.0f));
            const FF cov = ffn::div(cfa, nm1), var = ffn::div(m2a, nm1);
            const FF vv = var.h > 0.0f ? var : ffn::make(0.0f);
            if (vv.h > 0.0f) {
                const FF cc = cov.h > 0.0f ? cov : ffn::make(0.0f);
                const bool lt = cc.h < vv.h || (cc.h == vv.h && cc.l < vv.l);
                alpha = ffn::div(lt ? cc : vv, vv);
            }
        }
    }
    FF out[CH];
    for (int c = 0; c < CH; ++c) {
        const FF ap = ffn::make(approx[c]);
        if (use_approx) {
            out[c] = ap;
        } else {
            const FF sf = FF{sfh[c], sfl[c]}, sa = FF{sah[c], sal[c]};
            out[c] = ffn::add(ffn::div(ffn::sub(sf, ffn::mul(alpha, sa)), N), ffn::mul(alpha, ap));
        }
    }
    bool nan = false;
    for (int c = 0; c < CH; ++c) {
        const float o = vadd(out[c].h, out[c].l);
        nan = nan || isnan(o);
        bins[bin * CH + c] = o;
        if (approx_out) approx_out[bin * CH + c] = approx[c];
    }
    if (cfg.var_out) {
        /* variance of the estimate, Var(norm f - alpha norm g) / n from the sample moments of the
         * weighted norms (exact for a non-negative scalar integrand); infinite without 2 samples */
        float var = __int_as_float(0x7f800000);
        if (!use_approx && cfg.spp >= 2) {
            const float nn = (float)cfg.spp, a = vadd(alpha.h, alpha.l);
            const float m2 = vfma(vmul(a, a), m2a.h, vfma(vmul(-2.0f, a), cfa.h, m2f));
            var = m2 > 0.0f ? vdiv(m2, vmul(nn, vsub(nn, 1.0f))) : 0.0f;
        }
        cfg.var_out[bin] = var;
    }
    if (nan) atomicOr(status, VCU_FLAG_NAN);
}

}  // namespace cv_detail

/* host driver for one rule pair */
template <int SH, int SL>
int run_cv_pair(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, int iterations,
                const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                uint32_t& launches);

}  // namespace vcu

namespace vcu {
namespace cv_detail {

static __global__ void k_cv_regions_out(const int* __restrict__ heap_pay, const float* __restrict__ rmin,
                                 const float* __restrict__ rmax, int dim, int nheap, float* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nheap) return;
    const int id = heap_pay[k] & 0xffffff;
    for (int d = 0; d < dim; ++d) {
        out[(size_t)k * 2 * dim + d] = rmin[(size_t)id * dim + d];
        out[(size_t)k * 2 * dim + dim + d] = rmax[(size_t)id * dim + d];
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

/* stages 2 and 3 over a finished set of regions: hp[0..nheap) are pool ids (low 24 bits) in the
 * order the reference integrates them (heap order, or depth-first order for the tolerance-driven
 * form); cnt/off/cur are per-bin scratch of nbins, nbins+1, nbins words */
template <class F, int DIM, int SH, int SL>
int regions_into_bins(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_cv& cv,
                      const float* vals, const float* rmin, const float* rmax, const float* vol, const int* hp,
                      size_t nheap, uint32_t* cnt, uint32_t* off, uint32_t* cur, const float* d_replay, float* d_bins,
                      float* d_approx, float* d_regions, uint32_t& launches) {
    constexpr int S = SH;
    int rc = VCU_OK;
    /* stage 2 */
    ListCfg lc{};
    for (int d = 0; d < p->dimbins; ++d) {
        lc.rmin[d] = p->range_min[d];
        lc.rmax[d] = p->range_max[d];
        lc.res[d] = g.res[d];
    }
    lc.dim = DIM;
    lc.dimbins = p->dimbins;
    lc.nheap = (int)nheap;
    VCU_CUDA(ctx, cudaMemsetAsync(cnt, 0, g.nbins * 4, ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(cur, 0, g.nbins * 4, ctx->stream));
    const unsigned lblocks = (unsigned)((nheap * 32 + 255) / 256);
    k_cv_lists<<<lblocks, 256, 0, ctx->stream>>>(lc, hp, rmin, rmax, cnt, nullptr, nullptr, nullptr, 0);
    {
        const uint64_t ntiles = (g.nbins + SCAN_TILE - 1) / SCAN_TILE;
        /* the tile totals live in cur (256-byte aligned, nbins words, at least 256 bytes: room for
         * ntiles = nbins / 1024 eight-byte totals), which is zeroed again before the fill uses it */
        uint64_t* tt = reinterpret_cast<uint64_t*>(cur);
        k_cv_scan_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, ctx->stream>>>(cnt, off, g.nbins, tt);
        k_cv_scan_totals<<<1, SCAN_THREADS, 0, ctx->stream>>>(tt, ntiles, off, g.nbins, ctx->d_status);
        k_cv_scan_add<<<(unsigned)((g.nbins + 255) / 256), 256, 0, ctx->stream>>>(off, g.nbins, tt);
        VCU_CUDA(ctx, cudaMemsetAsync(cur, 0, g.nbins * 4, ctx->stream));
        launches += 4;
    }
    VCU_CUDA(ctx, cudaGetLastError());
    uint32_t total = 0;
    VCU_CUDA(ctx, cudaMemcpyAsync(&total, off + g.nbins, 4, cudaMemcpyDeviceToHost, ctx->stream));
    VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    /* aux: unsorted and sorted lists; for an importance choice also the per-entry running
     * probabilities and inverse probabilities (FP64) and, for rr_error, each heap region's error norm */
    const bool importance = cv.rr != VCU_RR_UNIFORM;
    const size_t o_cdf = align256((size_t)total * 8 + 512);
    const size_t o_rrf = align256(o_cdf + (size_t)total * 8);
    const size_t o_rerr = align256(o_rrf + (size_t)total * 8);
    const size_t aux_lists = importance ? o_rerr + nheap * 4 : (size_t)total * 8 + 512;
    /* the listed regions' first-fold coefficients, for the residual's polynomial values */
    const bool sampled = cv_coef_pass<DIM>() && (cv.samples_per_bin > 0 || d_replay != nullptr);
    const size_t o_coef = align256(aux_lists);
    const size_t aux_bytes = sampled ? o_coef + nheap * (size_t)ipow(S, DIM) * F::CH * 4 : aux_lists;
    if ((rc = ensure(ctx, ctx->aux, aux_bytes))) return rc;
    uint32_t* lists_u = static_cast<uint32_t*>(ctx->aux.ptr);
    uint32_t* lists = lists_u + total + 64;
    char* aux = static_cast<char*>(ctx->aux.ptr);
    float* coef = sampled ? reinterpret_cast<float*>(aux + o_coef) : nullptr;
    if (sampled) {
        const size_t nt = nheap * (size_t)ipow(S, DIM - 1) * F::CH;
        const unsigned cblocks = (unsigned)std::min<size_t>((nt + 255) / 256, (size_t)ctx->sm_count * 16);
        k_cv_coef<S, F::CH><<<cblocks, 256, 0, ctx->stream>>>(hp, vals, ipow(S, DIM), nheap, coef);
        ++launches;
    }
    k_cv_lists<<<lblocks, 256, 0, ctx->stream>>>(lc, hp, rmin, rmax, nullptr, off, cur, lists_u, 1);
    k_cv_sort<<<(unsigned)((g.nbins * 32 + 255) / 256), 256, 0, ctx->stream>>>(off, lists_u, lists, g.nbins);
    launches += 2;
    VCU_CUDA(ctx, cudaGetLastError());

    /* stage 3 */
    ResCfg rcfg{};
    for (int d = 0; d < DIM; ++d) {
        rcfg.rmin[d] = p->range_min[d];
        rcfg.rmax[d] = p->range_max[d];
    }
    for (int d = 0; d < p->dimbins; ++d) {
        rcfg.res[d] = g.res[d];
        rcfg.drange[d] = g.drange[d];
    }
    rcfg.dimbins = p->dimbins;
    rcfg.nbins = g.nbins;
    rcfg.factor = (double)g.factor;
    rcfg.factor_f32 = g.factor < (1ull << 24);
    rcfg.spp = cv.samples_per_bin;
    rcfg.k0 = (uint32_t)cv.seed;
    rcfg.k1 = (uint32_t)(cv.seed >> 32);
    rcfg.weight = cv.weight;
    rcfg.alpha = cv.alpha;
    /* reserved == 1 (set only by vcu_adaptive_iterations_global): accumulate into the bins' values */
    rcfg.approx_init = cv.reserved == 1 ? d_bins : nullptr;
    rcfg.rr = cv.rr;
    if (importance) {
        rcfg.cdf = reinterpret_cast<double*>(aux + o_cdf);
        rcfg.rrf = reinterpret_cast<double*>(aux + o_rrf);
        if (cv.rr == VCU_RR_ERROR) {
            float* rerr = reinterpret_cast<float*>(aux + o_rerr);
            k_cv_region_error<DIM, SH, SL, F::CH>
                <<<(unsigned)((nheap + 127) / 128), 128, 0, ctx->stream>>>(hp, vals, vol, (int)nheap, rerr);
            ++launches;
            rcfg.rerr = rerr;
        }
    }
    rcfg.sampling = cv.sampling;
    rcfg.rr_factor = cv.rr_factor;
    rcfg.mis_power = cv.mis_power;
    rcfg.mis_cutoff = cv.mis_cutoff;
    rcfg.rec_w = (uint32_t)vcu_cv_replay_width(DIM, cv.sampling);
    rcfg.var_out = cv.variance;
    const unsigned rblocks = (unsigned)((g.nbins + RES_WARPS - 1) / RES_WARPS);
    const bool pdf = cv.rr == VCU_RR_PDF || cv.sampling != VCU_RS_UNIFORM;
    if constexpr (S == 3) {
        if (pdf)
            k_cv_residual<F, DIM, S, true><<<rblocks, RES_WARPS * 32, 0, ctx->stream>>>(
                f, rcfg, off, lists, hp, vals, coef, rmin, rmax, vol, d_replay, d_bins, d_approx, ctx->d_status);
        else
            k_cv_residual<F, DIM, S, false><<<rblocks, RES_WARPS * 32, 0, ctx->stream>>>(
                f, rcfg, off, lists, hp, vals, coef, rmin, rmax, vol, d_replay, d_bins, d_approx, ctx->d_status);
    } else {
        if (pdf) return fail(ctx, VCU_UNSUPPORTED, "the pdf strategies need a Simpson high rule");
        k_cv_residual<F, DIM, S, false><<<rblocks, RES_WARPS * 32, 0, ctx->stream>>>(
            f, rcfg, off, lists, hp, vals, coef, rmin, rmax, vol, d_replay, d_bins, d_approx, ctx->d_status);
    }
    ++launches;
    if (d_regions) {
        k_cv_regions_out<<<(unsigned)((nheap + 255) / 256), 256, 0, ctx->stream>>>(hp, rmin, rmax, DIM, (int)nheap,
                                                                                  d_regions);
        ++launches;
    }
    VCU_CUDA(ctx, cudaGetLastError());
    return VCU_OK;
}

template <int DIM, int SH, int SL, class F>
int wave_launch(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, int iters,
                const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                uint32_t& launches);

/* which generator builds the heap: the waves from 128 splits on (VCU_CV_GENERATOR=wave|sequential
 * overrides), the single-block sequential one below that or when the waves give up */
inline bool use_waves(int iters) {
    const char* e = std::getenv("VCU_CV_GENERATOR");
    if (e && std::strcmp(e, "sequential") == 0) return false;
    if (e && std::strcmp(e, "wave") == 0) return iters > 0;
    return iters >= 128;
}

template <int DIM, int SH, int SL, class F>
int cv_launch(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, int iters,
              const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
              uint32_t& launches) {
    if (use_waves(iters)) {
        const int rc = wave_launch<DIM, SH, SL>(ctx, f, p, g, nst, iters, cv, d_replay, d_bins, d_approx, d_regions,
                                                launches);
        if (rc != -1) return rc; /* -1: the waves gave up, build the heap sequentially */
    }
    constexpr int S = SH;
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    const size_t npool = 2 * (size_t)iters + 1, nheap = (size_t)iters + 1;
    /* scratch layout: region pool, heap, per-bin counts/offsets/cursors */
    size_t o = 0;
    const size_t o_vals = o;
    o = align256(o + npool * SD * CH * 4);
    const size_t o_rmin = o;
    o = align256(o + npool * DIM * 4);
    const size_t o_rmax = o;
    o = align256(o + npool * DIM * 4);
    const size_t o_vol = o;
    o = align256(o + npool * 4);
    const size_t o_hk = o;
    o = align256(o + nheap * 4);
    const size_t o_hp = o;
    o = align256(o + nheap * 4);
    const size_t o_cnt = o;
    o = align256(o + g.nbins * 4);
    const size_t o_off = o;
    o = align256(o + (g.nbins + 1) * 4);
    const size_t o_cur = o;
    o = align256(o + g.nbins * 4);
    int rc = ensure(ctx, ctx->scratch, o);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->scratch.ptr);
    float* vals = reinterpret_cast<float*>(base + o_vals);
    float* rmin = reinterpret_cast<float*>(base + o_rmin);
    float* rmax = reinterpret_cast<float*>(base + o_rmax);
    float* vol = reinterpret_cast<float*>(base + o_vol);
    float* hk = reinterpret_cast<float*>(base + o_hk);
    int* hp = reinterpret_cast<int*>(base + o_hp);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(base + o_cnt);
    uint32_t* off = reinterpret_cast<uint32_t*>(base + o_off);
    uint32_t* cur = reinterpret_cast<uint32_t*>(base + o_cur);

    /* stage 1 */
    GenCfg gc{};
    for (int d = 0; d < DIM; ++d) {
        gc.rmin[d] = p->range_min[d];
        gc.rmax[d] = p->range_max[d];
    }
    gc.iters = iters;
    gc.heuristic = nst.heuristic;
    gc.relative = nst.metric == VCU_METRIC_RELATIVE;
    float mv = (float)nst.min_val;
    if ((double)mv < nst.min_val) mv = nextafterf(mv, INFINITY);
    gc.min_val_f = mv;
    gc.size_weight = nst.size_weight;
    gc.min_size = nst.min_size;
    auto gen = k_cv_generate<F, DIM, SH, SL>;
    cudaFuncAttributes attr;
    VCU_CUDA(ctx, cudaFuncGetAttributes(&attr, gen));
    const size_t heap_bytes = nheap * 8;
    gc.heap_in_smem = (heap_bytes + attr.sharedSizeBytes + 1024 <= ctx->smem_optin) ? 1 : 0;
    const size_t dsmem = gc.heap_in_smem ? heap_bytes : 0;
    if (dsmem) VCU_CUDA(ctx, cudaFuncSetAttribute(gen, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
    gen<<<1, GEN_THREADS, dsmem, ctx->stream>>>(f, gc, vals, rmin, rmax, vol, hk, hp, ctx->d_status);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());

    return regions_into_bins<F, DIM, SH, SL>(ctx, residual_functor(f), p, g, cv, vals, rmin, rmax, vol, hp, nheap, cnt,
                                             off, cur, d_replay, d_bins, d_approx, d_regions, launches);
}


/* ---------------------------------------------------------------- tolerance-driven adaptive
 * integrator_adaptive_tolerance (src/nested/integrator-adaptive-tolerance.h:9-56): the reference
 * recurses depth first -- a region whose heuristic error is below the tolerance is integrated into
 * the bins, any other is split and its halves visited in order.  Nothing is sequential but the order
 * the leaves are added into a bin, so the tree is built breadth first, one kernel per level, one
 * warp per region (errors, decision, and the split's new nodes), with every level's regions in
 * parallel.  Afterwards the leaves are ranked in depth-first order (leaf counts bottom up, offsets
 * top down) and stages 2-3 add them into the bins in that order. */
struct TolCfg {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
    int32_t heuristic, relative;
    float min_val_f;
    float tol;
    double size_weight, min_size;
    uint32_t capacity;
};

constexpr int TOL_WARPS = 4;

/* The heuristic error and split dimension of the region whose node values are V, computed by one
 * warp (lane 0 holds the result): per-dimension errors (region.h:379-418) with the reference's
 * rounding, then error_heuristic_default / error_heuristic_size (error-heuristic.h:10-47).  LN holds
 * DIM * S^(DIM-1) floats, EC DIM floats, both private to the warp. */
template <int DIM, int S, int SL, int CH>
__device__ __forceinline__ void warp_heuristic(const TolCfg& cfg, const float* V, float vol, const float* rmn,
                                               const float* rmx, float* LN, float* EC, int lane, float& err,
                                               int& dim) {
    constexpr int NL = ipow(S, DIM - 1);
    for (int t = lane; t < DIM * NL; t += 32) {
        const int d = t / NL, J = t % NL;
        float m = 0.0f;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            float line[S], low[SL];
#pragma unroll
            for (int i = 0; i < S; ++i) line[i] = V[node_index<DIM, S>(d, J, i) * CH + c];
#pragma unroll
            for (int i = 0; i < SL; ++i) low[i] = line[i * (S - 1) / (SL - 1)];
            float H, L;
            if constexpr (CH == 1) {
                H = RefRule<S>::scalar(line);
                L = RefRule<SL>::scalar(low);
            } else {
                H = RefRule<S>::rgb(line);
                L = RefRule<SL>::rgb(low);
            }
            const float mv = metric_value(cfg.relative, cfg.min_val_f, H, L);
            m = (c == 0) ? mv : vadd(m, mv);
        }
        LN[t] = m;
    }
    __syncwarp();
    if (lane < DIM) {
        float buf[NL];
        for (int i = 0; i < NL; ++i) buf[i] = LN[lane * NL + i];
        int n = NL;
        for (int level = 0; level < DIM - 1; ++level) {
            n /= S;
            for (int i = 0; i < n; ++i) buf[i] = RefRule<S>::scalar(buf + i * S);
        }
        EC[lane] = vmul(vol, buf[0]);
    }
    __syncwarp();
    err = 0.0f;
    dim = 0;
    if (lane == 0) {
        const float* e = EC;
        float max_err;
        int max_dim = 0;
        if (cfg.heuristic == VCU_HEUR_DEFAULT) {
            max_err = 0.0f;
            for (int d = 0; d < DIM; ++d)
                if (e[d] > max_err) {
                    max_err = e[d];
                    max_dim = d;
                }
        } else {
            float wd = vsub(rmx[0], rmn[0]);
            if ((double)wd < cfg.min_size || isnan(wd)) max_err = 0.0f;
            else max_err = __double2float_rn(__dadd_rn((double)e[0], __dmul_rn(cfg.size_weight, (double)fabsf(wd))));
            for (int d = 1; d < DIM; ++d) {
                wd = vsub(rmx[d], rmn[d]);
                float er = __double2float_rn(__dadd_rn((double)e[d], __dmul_rn(cfg.size_weight, (double)fabsf(wd))));
                if ((double)wd < cfg.min_size) er = 0.0f;
                if (er >= max_err) {
                    max_err = er;
                    max_dim = d;
                }
            }
        }
        err = max_err;
        dim = max_dim;
    }
}

template <class F, int DIM, int SH>
__global__ void k_tol_root(const __grid_constant__ F f, const TolCfg cfg, float* __restrict__ vals,
                           float* __restrict__ rmin, float* __restrict__ rmax, float* __restrict__ vol) {
    constexpr int S = SH, CH = F::CH, SD = ipow(S, DIM);
    __shared__ float CO[DIM * S];
    for (int t = threadIdx.x; t < DIM * S; t += blockDim.x) {
        const int d = t / S, j = t % S;
        CO[t] = node_coord(node_pos<S>(j), vsub(cfg.rmax[d], cfg.rmin[d]), cfg.rmin[d]);
    }
    if (threadIdx.x == 0) {
        float v = 1.0f;
        for (int d = 0; d < DIM; ++d) {
            rmin[d] = cfg.rmin[d];
            rmax[d] = cfg.rmax[d];
            v = vmul(v, vsub(cfg.rmax[d], cfg.rmin[d]));
        }
        vol[0] = v;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < SD; t += blockDim.x) {
        float x[F::DIM];
        for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
        int rem = t;
        for (int d = 0; d < DIM; ++d) {
            x[d] = CO[d * S + rem % S];
            rem /= S;
        }
        float v[CH];
        f(x, v);
        for (int c = 0; c < CH; ++c) vals[t * CH + c] = v[c];
    }
}

/* Split region id along dd into pool slots C0 (lower half) and C0+1 (upper half), one warp: the new
 * nodes at the odd positions are evaluated, the parent's nodes fill the even ones (region.h:345-359,
 * split.h:13-49), and the children's ranges and volumes are written.  CO (DIM*S floats) and CN (S-1)
 * are the warp's scratch. */
template <class F, int DIM, int S>
__device__ __forceinline__ void warp_split(const F& f, const float* V, int id, int dd, int C0, float* vals, float* rmin,
                                           float* rmax, float* vol, float* CO, float* CN, int lane) {
    constexpr int CH = F::CH, SD = ipow(S, DIM), NL = ipow(S, DIM - 1), NNEW = (S - 1) * NL;
    const int C1 = C0 + 1;
    const float* pmin = rmin + (size_t)id * DIM;
    const float* pmax = rmax + (size_t)id * DIM;
    for (int t = lane; t < DIM * S + (S - 1); t += 32) {
        if (t < DIM * S) {
            const int d = t / S, j = t % S;
            CO[t] = node_coord(node_pos<S>(j), vsub(pmax[d], pmin[d]), pmin[d]);
        } else {
            const int k = t - DIM * S;
            CN[k] = node_coord(mid_pos<S>(k), vsub(pmax[dd], pmin[dd]), pmin[dd]);
        }
    }
    __syncwarp();
    float* V0 = vals + (size_t)C0 * SD * CH;
    float* V1 = vals + (size_t)C1 * SD * CH;
    for (int t = lane; t < NNEW + S * NL; t += 32) {
        const bool fresh = t < NNEW;
        const int u = fresh ? t : t - NNEW;
        const int k = u / NL, J = u % NL;
        float v[CH];
        int i;
        if (fresh) {
            float x[F::DIM];
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
            int rem = J;
            for (int e = 0; e < DIM; ++e) {
                if (e == dd) continue;
                x[e] = CO[e * S + rem % S];
                rem /= S;
            }
            x[dd] = CN[k];
            f(x, v);
            i = 2 * k + 1;
        } else {
#pragma unroll
            for (int c = 0; c < CH; ++c) v[c] = V[node_index<DIM, S>(dd, J, k) * CH + c];
            i = 2 * k;
        }
        if (i <= S - 1) {
            const int n0 = node_index<DIM, S>(dd, J, i) * CH;
#pragma unroll
            for (int c = 0; c < CH; ++c) V0[n0 + c] = v[c];
        }
        if (i >= S - 1) {
            const int n1 = node_index<DIM, S>(dd, J, i - (S - 1)) * CH;
#pragma unroll
            for (int c = 0; c < CH; ++c) V1[n1 + c] = v[c];
        }
    }
    if (lane == 0) {
        const float pmn = pmin[dd], pmx = pmax[dd];
        const float half = vmul(vsub(pmx, pmn), 0.5f); /* = (max - min) / 2.0, exactly */
        const float mid = vadd(pmn, vmul(half, 1.0f));
        float v0 = 1.0f, v1 = 1.0f;
        for (int d = 0; d < DIM; ++d) {
            const float mn = pmin[d], mx = pmax[d];
            const float mx0 = (d == dd) ? mid : mx;
            const float mn1 = (d == dd) ? mid : mn;
            rmin[(size_t)C0 * DIM + d] = mn;
            rmax[(size_t)C0 * DIM + d] = mx0;
            rmin[(size_t)C1 * DIM + d] = mn1;
            rmax[(size_t)C1 * DIM + d] = mx;
            v0 = vmul(v0, vsub(mx0, mn));
            v1 = vmul(v1, vsub(mx, mn1));
        }
        vol[C0] = v0;
        vol[C1] = v1;
    }
}

/* one level: counters[0] = pool slots used, counters[1] = regions of the next level */
template <class F, int DIM, int SH, int SL>
__global__ void __launch_bounds__(TOL_WARPS * 32)
    k_tol_level(const __grid_constant__ F f, const TolCfg cfg, const int* __restrict__ cur, int ncur,
                int* __restrict__ next, uint32_t* __restrict__ counters, float* __restrict__ vals,
                float* __restrict__ rmin, float* __restrict__ rmax, float* __restrict__ vol, int* __restrict__ child,
                uint32_t* __restrict__ status) {
    constexpr int S = SH, CH = F::CH, SD = ipow(S, DIM), NL = ipow(S, DIM - 1);
    __shared__ float LN[TOL_WARPS][DIM * NL];
    __shared__ float EC[TOL_WARPS][DIM];
    __shared__ float CO[TOL_WARPS][DIM * S], CN[TOL_WARPS][S - 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * TOL_WARPS + warp;
    if (w >= ncur) return;
    const int id = cur[w];
    const float* V = vals + (size_t)id * SD * CH;
    float max_err;
    int max_dim;
    warp_heuristic<DIM, S, SL, CH>(cfg, V, vol[id], rmin + (size_t)id * DIM, rmax + (size_t)id * DIM, LN[warp], EC[warp],
                                   lane, max_err, max_dim);
    int split_dim = 0, c0 = -1;
    if (lane == 0) {
        if (max_err < cfg.tol) {
            child[id] = -1; /* leaf */
        } else {
            const uint32_t c = atomicAdd(&counters[0], 2u);
            if (c + 2 > cfg.capacity) {
                atomicOr(status, VCU_FLAG_OVERFLOW);
                child[id] = -1;
            } else {
                child[id] = (int)c;
                const uint32_t k = atomicAdd(&counters[1], 2u);
                next[k] = (int)c;
                next[k + 1] = (int)c + 1;
                c0 = (int)c;
                split_dim = max_dim;
            }
        }
    }
    c0 = __shfl_sync(0xffffffffu, c0, 0);
    split_dim = __shfl_sync(0xffffffffu, split_dim, 0);
    if (c0 < 0) return;
    warp_split<F, DIM, S>(f, V, id, split_dim, c0, vals, rmin, rmax, vol, CO[warp], CN[warp], lane);
}

/* leaf counts of the subtrees of one level's regions (deepest level first) */
static __global__ void k_tol_count(const int* __restrict__ lvl, int n, const int* __restrict__ child,
                                   uint32_t* __restrict__ leaves) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = lvl[i], c = child[id];
    leaves[id] = c < 0 ? 1u : leaves[c] + leaves[c + 1];
}

/* depth-first offsets (root level first): children inherit the parent's offset, the second after the
 * first's leaves; a leaf's offset is its depth-first rank */
static __global__ void k_tol_rank(const int* __restrict__ lvl, int n, const int* __restrict__ child,
                                  const uint32_t* __restrict__ leaves, uint32_t* __restrict__ first,
                                  int* __restrict__ order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = lvl[i], c = child[id];
    const uint32_t o = first[id];
    if (c < 0) {
        order[o] = id;
    } else {
        first[c] = o;
        first[c + 1] = o + leaves[c];
    }
}

template <int DIM, int SH, int SL, class F>
int tol_launch(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, float tol,
               uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches) {
    constexpr int S = SH;
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    /* pool capacity: the caller's, else what 4 GiB of region storage holds */
    const size_t per_region = (size_t)SD * CH * 4 + 2 * DIM * 4 + 4 + 4 + 4 + 4 + 4 + 4;
    size_t cap = max_regions ? (size_t)max_regions : ((size_t)4 << 30) / per_region;
    if (cap > (1u << 24) - 2) cap = (1u << 24) - 2;
    if (cap < 1) cap = 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    const size_t o_vals = take(cap * SD * CH * 4), o_rmin = take(cap * DIM * 4), o_rmax = take(cap * DIM * 4),
                 o_vol = take(cap * 4), o_child = take(cap * 4), o_lvl = take(cap * 4), o_leaves = take(cap * 4),
                 o_first = take(cap * 4), o_order = take(cap * 4), o_ctr = take(64), o_cnt = take(g.nbins * 4),
                 o_off = take((g.nbins + 1) * 4), o_cur = take(g.nbins * 4);
    int rc = ensure(ctx, ctx->scratch, o);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->scratch.ptr);
    float* vals = reinterpret_cast<float*>(base + o_vals);
    float* rmin = reinterpret_cast<float*>(base + o_rmin);
    float* rmax = reinterpret_cast<float*>(base + o_rmax);
    float* vol = reinterpret_cast<float*>(base + o_vol);
    int* child = reinterpret_cast<int*>(base + o_child);
    int* lvl = reinterpret_cast<int*>(base + o_lvl);
    uint32_t* leaves = reinterpret_cast<uint32_t*>(base + o_leaves);
    uint32_t* first = reinterpret_cast<uint32_t*>(base + o_first);
    int* order = reinterpret_cast<int*>(base + o_order);
    uint32_t* ctr = reinterpret_cast<uint32_t*>(base + o_ctr);

    TolCfg tc{};
    for (int d = 0; d < DIM; ++d) {
        tc.rmin[d] = p->range_min[d];
        tc.rmax[d] = p->range_max[d];
    }
    tc.heuristic = nst.heuristic;
    tc.relative = nst.metric == VCU_METRIC_RELATIVE;
    float mv = (float)nst.min_val;
    if ((double)mv < nst.min_val) mv = nextafterf(mv, INFINITY);
    tc.min_val_f = mv;
    tc.tol = tol;
    tc.size_weight = nst.size_weight;
    tc.min_size = nst.min_size;
    tc.capacity = (uint32_t)cap;
    k_tol_root<F, DIM, SH><<<1, 256, 0, ctx->stream>>>(f, tc, vals, rmin, rmax, vol);
    const uint32_t init[2] = {1u, 0u};
    const int zero = 0;
    VCU_CUDA(ctx, cudaMemcpyAsync(ctr, init, 8, cudaMemcpyHostToDevice, ctx->stream));
    VCU_CUDA(ctx, cudaMemcpyAsync(lvl, &zero, 4, cudaMemcpyHostToDevice, ctx->stream));
    ++launches;
    /* breadth first: level L's regions are lvl[starts[L] .. starts[L+1]) */
    std::vector<size_t> starts{0, 1};
    constexpr int MAX_LEVELS = 256;
    for (int L = 0;; ++L) {
        const size_t a = starts[L], n = starts[L + 1] - starts[L];
        if (L >= MAX_LEVELS) return fail(ctx, VCU_QUEUE_OVERFLOW, "tolerance not reached within 256 levels of subdivision");
        VCU_CUDA(ctx, cudaMemsetAsync(ctr + 1, 0, 4, ctx->stream));
        k_tol_level<F, DIM, SH, SL><<<(unsigned)((n + TOL_WARPS - 1) / TOL_WARPS), TOL_WARPS * 32, 0, ctx->stream>>>(
            f, tc, lvl + a, (int)n, lvl + a + n, ctr, vals, rmin, rmax, vol, child, ctx->d_status);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
        uint32_t host[2];
        VCU_CUDA(ctx, cudaMemcpyAsync(host, ctr, 8, cudaMemcpyDeviceToHost, ctx->stream));
        VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        uint32_t flags = 0;
        VCU_CUDA(ctx, cudaMemcpy(&flags, ctx->d_status, 4, cudaMemcpyDeviceToHost));
        if (flags & VCU_FLAG_OVERFLOW)
            return fail(ctx, VCU_QUEUE_OVERFLOW, "tolerance needs more than " + std::to_string(cap) + " regions");
        if (host[1] == 0) break;
        starts.push_back(starts.back() + host[1]);
    }
    const int levels = (int)starts.size() - 1;
    nregions = starts.back();
    /* depth-first ranks of the leaves */
    for (int L = levels - 1; L >= 0; --L) {
        const size_t n = starts[L + 1] - starts[L];
        k_tol_count<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(lvl + starts[L], (int)n, child, leaves);
        ++launches;
    }
    VCU_CUDA(ctx, cudaMemsetAsync(first, 0, 4, ctx->stream));
    for (int L = 0; L < levels; ++L) {
        const size_t n = starts[L + 1] - starts[L];
        k_tol_rank<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(lvl + starts[L], (int)n, child, leaves, first,
                                                                         order);
        ++launches;
    }
    VCU_CUDA(ctx, cudaGetLastError());
    uint32_t nl = 0;
    VCU_CUDA(ctx, cudaMemcpyAsync(&nl, leaves, 4, cudaMemcpyDeviceToHost, ctx->stream));
    VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    nleaves = nl;
    /* stages 2-3: the leaves into the bins in depth-first order, accumulating */
    vcu_cv cv{};
    cv.samples_per_bin = 0;
    cv.weight = VCU_CV_FIXED;
    cv.reserved = 1;
    cv.alpha = 1.0;
    return regions_into_bins<F, DIM, SH, SL>(ctx, f, p, g, cv, vals, rmin, rmax, vol, order, nl,
                                         reinterpret_cast<uint32_t*>(base + o_cnt), reinterpret_cast<uint32_t*>(base + o_off),
                                         reinterpret_cast<uint32_t*>(base + o_cur), nullptr, d_bins, nullptr, nullptr,
                                         launches);
}

/* ---------------------------------------------------------------- the heap's regions in waves
 * regions_generator_adaptive_heap (regions-generator-adaptive-heap.h:18-45) pops the region of
 * largest error and pushes its two halves, `iterations` times.  Which regions it splits can be found
 * without following it step by step: a region is split before any region whose path from the root
 * holds a smaller error, so the split set is (ties aside) the `iterations` regions of largest
 * bottleneck b(v) = min of the errors from the root to v.  Waves expand the unsplit regions of
 * largest b together (one warp per region: its new nodes, then its halves' errors), until the
 * regions already split with b >= the largest b left unsplit number `iterations`.  The host then
 * replays the reference's exact heap sequence (libstdc++ push/pop, vcu_heap.h) on the computed
 * errors, which fixes the final heap order (the order regions are integrated in) and resolves ties
 * exactly; a region that sequence pops but no wave split sends the waves further.  The result is the
 * sequential generator's, region for region and position for position.  Which regions a wave
 * splits (and whether the waves are done) is decided on the device between waves (k_wave_decide),
 * so waves run back to back and the host reads the loop's state once every WAVE_CHUNK waves. */
constexpr int WAVE_WARPS = 4;
constexpr int WAVE_SHIFT = 19;                      /* bucket = bits(b) >> 19: 4096 buckets */
constexpr int WAVE_BUCKETS = 1 << (31 - WAVE_SHIFT);
/* counters: */
enum { WC_POOL = 0, WC_NEW = 1, WC_EXPAND = 2, WC_FRONT2 = 3, WC_SPLIT = 4, WC_MAXB = 5, WC_GE = 6, WC_NAN = 7,
       WC_FRONT = 8, WC_OVF = 9, WC_N = 16 };

/* The wave loop's state, decided on the device between waves (k_wave_decide): the host launches
 * waves back to back and reads it back once every WAVE_CHUNK waves. */
struct WaveCtl {
    uint32_t state; /* WAVE_ACTIVE, WAVE_DONE (the split set is complete), WAVE_FAIL (sequential generator) */
    uint32_t thr;   /* this wave's bucket threshold */
    uint32_t cur;   /* the unsplit regions' list: 0 -> the first list, 1 -> the second */
    uint32_t waves; /* waves decided so far */
};
enum : uint32_t { WAVE_ACTIVE = 0, WAVE_DONE = 1, WAVE_FAIL = 2 };
constexpr int WAVE_CHUNK = 8;
constexpr uint32_t WAVE_NO_FORCE = 0xffffffffu;

__device__ __forceinline__ uint32_t wave_bits(float b) {
    const uint32_t u = __float_as_uint(b);
    return (u & 0x80000000u) ? 0u : u; /* errors are >= 0; -0 counts as 0 */
}

/* errors of the listed regions; b = min(b(parent), error) */
template <class F, int DIM, int SH, int SL>
__global__ void __launch_bounds__(WAVE_WARPS * 32)
    k_wave_eval(const TolCfg cfg, const int* __restrict__ list, const uint32_t* __restrict__ nlist,
                const float* __restrict__ vals, const float* __restrict__ rmin, const float* __restrict__ rmax,
                const float* __restrict__ vol, const int* __restrict__ parent, float* __restrict__ key,
                int* __restrict__ kdim, float* __restrict__ bneck, uint32_t* __restrict__ ctr,
                const WaveCtl* __restrict__ ctl) {
    constexpr int S = SH, CH = F::CH, SD = ipow(S, DIM), NL = ipow(S, DIM - 1);
    __shared__ float LN[WAVE_WARPS][DIM * NL];
    __shared__ float EC[WAVE_WARPS][DIM];
    if (ctl->state != WAVE_ACTIVE) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t n = *nlist;
    for (uint32_t w = blockIdx.x * WAVE_WARPS + warp; w < n; w += gridDim.x * WAVE_WARPS) {
        const int id = list[w];
        float e;
        int dm;
        warp_heuristic<DIM, S, SL, CH>(cfg, vals + (size_t)id * SD * CH, vol[id], rmin + (size_t)id * DIM,
                                       rmax + (size_t)id * DIM, LN[warp], EC[warp], lane, e, dm);
        if (lane == 0) {
            key[id] = e;
            kdim[id] = dm;
            const int par = parent[id];
            const float bp = par < 0 ? e : bneck[par];
            bneck[id] = (e < bp) ? e : bp;
            if (isnan(e)) atomicOr(&ctr[WC_NAN], 1u);
        }
        __syncwarp();
    }
}

/* the largest b of the unsplit regions, and their histogram of b; the count of split regions with
 * b >= that largest b comes next (k_wave_count) */
static __global__ void k_wave_stats(const int* __restrict__ fa, const int* __restrict__ fb,
                                    const uint32_t* __restrict__ nfront, const float* __restrict__ bneck,
                                    uint32_t* __restrict__ ctr, uint32_t* __restrict__ hist,
                                    const WaveCtl* __restrict__ ctl) {
    __shared__ uint32_t h[WAVE_BUCKETS];
    if (ctl->state != WAVE_ACTIVE) return;
    const int* __restrict__ front = ctl->cur ? fb : fa;
    for (int i = threadIdx.x; i < WAVE_BUCKETS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint32_t n = *nfront;
    uint32_t mx = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t u = wave_bits(bneck[front[i]]);
        mx = u > mx ? u : mx;
        atomicAdd(&h[u >> WAVE_SHIFT], 1u);
    }
    atomicMax(&ctr[WC_MAXB], mx);
    __syncthreads();
    for (int i = threadIdx.x; i < WAVE_BUCKETS; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

static __global__ void k_wave_count(const int* __restrict__ split, const uint32_t* __restrict__ nsplit,
                                    const float* __restrict__ bneck, uint32_t* __restrict__ ctr,
                                    const WaveCtl* __restrict__ ctl) {
    if (ctl->state != WAVE_ACTIVE) return;
    const uint32_t n = *nsplit, m = ctr[WC_MAXB];
    uint32_t c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += wave_bits(bneck[split[i]]) >= m;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&ctr[WC_GE], c);
}

/* the unsplit regions whose b lies in bucket >= thr are split this wave (and recorded as split);
 * the others stay unsplit */
static __global__ void k_wave_select(int* __restrict__ fa, int* __restrict__ fb, const uint32_t* __restrict__ nfront,
                                     const float* __restrict__ bneck, int* __restrict__ expand,
                                     int* __restrict__ split, uint32_t* __restrict__ ctr,
                                     const WaveCtl* __restrict__ ctl) {
    if (ctl->state != WAVE_ACTIVE) return;
    const int* __restrict__ front = ctl->cur ? fb : fa;
    int* __restrict__ front2 = ctl->cur ? fa : fb;
    const uint32_t thr = ctl->thr;
    const uint32_t n = *nfront;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int id = front[i];
        if ((wave_bits(bneck[id]) >> WAVE_SHIFT) >= thr) {
            expand[atomicAdd(&ctr[WC_EXPAND], 1u)] = id;
            split[atomicAdd(&ctr[WC_SPLIT], 1u)] = id;
        } else {
            front2[atomicAdd(&ctr[WC_FRONT2], 1u)] = id;
        }
    }
}

/* The host loop's decision between two waves, on the device (one block of 1024 threads): stop when
 * the pool overflowed or an error is NaN (the sequential generator takes over), or when the split set
 * is complete (no unsplit region, or `iters` split regions with b >= the largest unsplit b, unless a
 * forced bucket is still above it); otherwise split the unsplit regions of the top buckets, as many
 * as still needed -- the bucket where the count from the top reaches them -- but none more than two
 * octaves below the largest b, nor above a forced bucket. */
constexpr int DECIDE_THREADS = 1024;
static __global__ void __launch_bounds__(DECIDE_THREADS)
    k_wave_decide(uint32_t* __restrict__ ctr, const uint32_t* __restrict__ hist, WaveCtl* __restrict__ ctl,
                  uint32_t iters, uint32_t capacity, uint32_t force) {
    constexpr int PER = WAVE_BUCKETS / DECIDE_THREADS;
    __shared__ uint32_t part[DECIDE_THREADS];
    __shared__ uint32_t best;
    if (ctl->state != WAVE_ACTIVE) return;
    const int t = threadIdx.x;
    const uint32_t nfront = ctr[WC_FRONT], ge = ctr[WC_GE], maxb = ctr[WC_MAXB] >> WAVE_SHIFT;
    const bool forced = force != WAVE_NO_FORCE && maxb >= force;
    const bool fail = ctr[WC_OVF] != 0u || ctr[WC_NAN] != 0u || ctl->waves > 100000u;
    const bool done = nfront == 0u || (ge >= iters && !forced);
    if (fail || done) {
        __syncthreads();
        if (t == 0) ctl->state = fail ? WAVE_FAIL : WAVE_DONE;
        return;
    }
    const uint32_t need = ge >= iters ? 1u : iters - ge;
    /* suffix counts: part[t] = this thread's buckets, then the count above them */
    uint32_t local[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        local[k] = hist[t * PER + k];
        sum += local[k];
    }
    part[t] = sum;
    if (t == 0) best = 0u;
    __syncthreads();
    for (int off = 1; off < DECIDE_THREADS; off <<= 1) { /* inclusive suffix scan over threads */
        const uint32_t v = (t + off < DECIDE_THREADS) ? part[t + off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t suffix = part[t] - sum; /* buckets above this thread's */
    uint32_t cand = 0u;
    bool found = false;
#pragma unroll
    for (int k = PER - 1; k >= 0; --k) {
        suffix += local[k];
        if (!found && suffix >= need) {
            found = true;
            cand = (uint32_t)(t * PER + k);
        }
    }
    if (found) atomicMax(&best, cand);
    __syncthreads();
    if (t == 0) {
        uint32_t thr = best; /* 0 when the unsplit regions number fewer than needed */
        const uint32_t octave2 = 2u * (1u << (23 - WAVE_SHIFT));
        const uint32_t floor_bkt = maxb > octave2 ? maxb - octave2 : 0u;
        if (thr < floor_bkt) thr = floor_bkt;
        if (forced && force < thr) thr = force;
        ctl->thr = thr;
        ctl->waves += 1u;
    }
    __syncthreads();
    /* the regions this wave splits: the unsplit ones in buckets >= thr (the suffix count at thr) */
    const uint32_t thr = ctl->thr;
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k)
        if ((uint32_t)(t * PER + k) >= thr) acc += local[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __syncthreads();
    if ((t & 31) == 0) part[t >> 5] = acc;
    __syncthreads();
    if (t == 0) {
        uint64_t total = 0;
        for (int w = 0; w < DECIDE_THREADS / 32; ++w) total += part[w];
        if ((uint64_t)ctr[WC_POOL] + 2ull * total > capacity) {
            ctl->state = WAVE_FAIL;
        } else {
            ctr[WC_NEW] = 0u;
            ctr[WC_EXPAND] = 0u;
            ctr[WC_FRONT2] = 0u;
        }
    }
}

/* after a wave: the new unsplit list becomes the current one */
static __global__ void k_wave_swap(uint32_t* __restrict__ ctr, WaveCtl* __restrict__ ctl) {
    if (ctl->state != WAVE_ACTIVE) return;
    ctr[WC_FRONT] = ctr[WC_FRONT2];
    ctl->cur ^= 1u;
}

/* split the selected regions along their heuristic dimension; the halves join the unsplit list
 * and the list whose errors are computed next */
template <class F, int DIM, int SH>
__global__ void __launch_bounds__(WAVE_WARPS * 32)
    k_wave_split(const __grid_constant__ F f, const int* __restrict__ expand, const uint32_t* __restrict__ nexpand,
                 const int* __restrict__ kdim, uint32_t capacity, float* __restrict__ vals, float* __restrict__ rmin,
                 float* __restrict__ rmax, float* __restrict__ vol, int* __restrict__ child, int* __restrict__ parent,
                 int* __restrict__ fresh, int* __restrict__ fa, int* __restrict__ fb, uint32_t* __restrict__ ctr,
                 const WaveCtl* __restrict__ ctl) {
    constexpr int S = SH, CH = F::CH, SD = ipow(S, DIM);
    __shared__ float CO[WAVE_WARPS][DIM * S], CN[WAVE_WARPS][S - 1];
    if (ctl->state != WAVE_ACTIVE) return;
    int* __restrict__ front2 = ctl->cur ? fa : fb;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t n = *nexpand;
    for (uint32_t w = blockIdx.x * WAVE_WARPS + warp; w < n; w += gridDim.x * WAVE_WARPS) {
    const int id = expand[w];
    int c0 = -1;
    if (lane == 0) {
        const uint32_t c = atomicAdd(&ctr[WC_POOL], 2u);
        if (c + 2 > capacity) {
            atomicOr(&ctr[WC_OVF], 1u);
        } else {
            c0 = (int)c;
            child[id] = c0;
            parent[c0] = id;
            parent[c0 + 1] = id;
            child[c0] = -1;
            child[c0 + 1] = -1;
            const uint32_t k = atomicAdd(&ctr[WC_NEW], 2u);
            fresh[k] = c0;
            fresh[k + 1] = c0 + 1;
            const uint32_t q = atomicAdd(&ctr[WC_FRONT2], 2u);
            front2[q] = c0;
            front2[q + 1] = c0 + 1;
        }
    }
    c0 = __shfl_sync(0xffffffffu, c0, 0);
    if (c0 < 0) continue;
    warp_split<F, DIM, S>(f, vals + (size_t)id * SD * CH, id, kdim[id], c0, vals, rmin, rmax, vol, CO[warp], CN[warp],
                          lane);
    __syncwarp();
    }
}

template <int DIM, int SH, int SL, class F>
int wave_launch(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, int iters,
                const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                uint32_t& launches) {
    constexpr int S = SH;
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    const size_t N = (size_t)iters;
    /* pool: the split set plus room for the waves' overshoot */
    size_t cap = 6 * N + 4096;
    const size_t per_node = (size_t)SD * CH * 4 + 2 * DIM * 4 + 4 * 4 + 6 * 4;
    if (cap > ((size_t)6 << 30) / per_node) cap = ((size_t)6 << 30) / per_node;
    if (cap > (1u << 24) - 2) cap = (1u << 24) - 2;
    if (cap < 2 * N + 1) return -1; /* too large: the sequential generator */
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    const size_t o_vals = take(cap * SD * CH * 4), o_rmin = take(cap * DIM * 4), o_rmax = take(cap * DIM * 4),
                 o_vol = take(cap * 4), o_key = take(cap * 4), o_kdim = take(cap * 4), o_b = take(cap * 4),
                 o_par = take(cap * 4), o_child = take(cap * 4), o_fa = take(cap * 4), o_fb = take(cap * 4),
                 o_exp = take(cap * 4), o_split = take(cap * 4), o_fresh = take(cap * 4), o_hp = take((N + 1) * 4),
                 o_ctr = take(WC_N * 4), o_ctl = take(sizeof(WaveCtl)), o_hist = take(WAVE_BUCKETS * 4),
                 o_skey = take(cap * 4), o_sdim = take(cap * 4), o_schild = take(cap * 4),
                 o_sctr = take(WC_N * 4 + sizeof(WaveCtl)),
                 o_cnt = take(g.nbins * 4),
                 o_off = take((g.nbins + 1) * 4), o_cur = take(g.nbins * 4);
    int rc = ensure(ctx, ctx->scratch, o);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->scratch.ptr);
    float* vals = reinterpret_cast<float*>(base + o_vals);
    float* rmin = reinterpret_cast<float*>(base + o_rmin);
    float* rmax = reinterpret_cast<float*>(base + o_rmax);
    float* vol = reinterpret_cast<float*>(base + o_vol);
    float* key = reinterpret_cast<float*>(base + o_key);
    int* kdim = reinterpret_cast<int*>(base + o_kdim);
    float* bneck = reinterpret_cast<float*>(base + o_b);
    int* parent = reinterpret_cast<int*>(base + o_par);
    int* child = reinterpret_cast<int*>(base + o_child);
    int* fa = reinterpret_cast<int*>(base + o_fa);
    int* fb = reinterpret_cast<int*>(base + o_fb);
    int* expand = reinterpret_cast<int*>(base + o_exp);
    int* split = reinterpret_cast<int*>(base + o_split);
    int* fresh = reinterpret_cast<int*>(base + o_fresh);
    int* hp = reinterpret_cast<int*>(base + o_hp);
    uint32_t* ctr = reinterpret_cast<uint32_t*>(base + o_ctr);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + o_hist);

    TolCfg tc{};
    for (int d = 0; d < DIM; ++d) {
        tc.rmin[d] = p->range_min[d];
        tc.rmax[d] = p->range_max[d];
    }
    tc.heuristic = nst.heuristic;
    tc.relative = nst.metric == VCU_METRIC_RELATIVE;
    float mv = (float)nst.min_val;
    if ((double)mv < nst.min_val) mv = nextafterf(mv, INFINITY);
    tc.min_val_f = mv;
    tc.size_weight = nst.size_weight;
    tc.min_size = nst.min_size;
    tc.capacity = (uint32_t)cap;

    /* the root, its error; it is the one unsplit region */
    k_tol_root<F, DIM, SH><<<1, 256, 0, ctx->stream>>>(f, tc, vals, rmin, rmax, vol);
    {
        uint32_t init[WC_N] = {};
        init[WC_POOL] = 1;
        init[WC_NEW] = 1;
        init[WC_FRONT] = 1;
        const int root[3] = {0, -1, -1}; /* fresh/front list, parent, child of the root */
        VCU_CUDA(ctx, cudaMemcpyAsync(ctr, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
        VCU_CUDA(ctx, cudaMemcpyAsync(fresh, root, 4, cudaMemcpyHostToDevice, ctx->stream));
        VCU_CUDA(ctx, cudaMemcpyAsync(fa, root, 4, cudaMemcpyHostToDevice, ctx->stream));
        VCU_CUDA(ctx, cudaMemcpyAsync(parent, root + 1, 4, cudaMemcpyHostToDevice, ctx->stream));
        VCU_CUDA(ctx, cudaMemcpyAsync(child, root + 2, 4, cudaMemcpyHostToDevice, ctx->stream));
    }
    WaveCtl* ctl = reinterpret_cast<WaveCtl*>(base + o_ctl);
    {
        const WaveCtl c0{WAVE_ACTIVE, 0u, 0u, 0u};
        VCU_CUDA(ctx, cudaMemcpyAsync(ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, ctx->stream));
    }
    k_wave_eval<F, DIM, SH, SL><<<1, WAVE_WARPS * 32, 0, ctx->stream>>>(tc, fresh, ctr + WC_NEW, vals, rmin, rmax, vol,
                                                                      parent, key, kdim, bneck, ctr, ctl);
    launches += 2;
    std::vector<float> hkey, hb;
    std::vector<int> hdim, hchild;
    std::vector<HeapEntry> H(N + 2);
    std::vector<int> HS(N + 1);
    uint32_t force = WAVE_NO_FORCE; /* after an incomplete replay: split every unsplit b bucket >= force */
    /* fixed grids (the kernels loop over their lists, whose lengths stay on the device) */
    const unsigned gstat = (unsigned)ctx->sm_count * 4;
    const unsigned gsplit = (unsigned)ctx->sm_count * 8, geval = (unsigned)ctx->sm_count * 16;
    auto chunk = [&]() -> int {
        for (int wave = 0; wave < WAVE_CHUNK; ++wave) {
            VCU_CUDA(ctx, cudaMemsetAsync(ctr + WC_MAXB, 0, 8, ctx->stream));
            VCU_CUDA(ctx, cudaMemsetAsync(hist, 0, WAVE_BUCKETS * 4, ctx->stream));
            k_wave_stats<<<gstat, 256, 0, ctx->stream>>>(fa, fb, ctr + WC_FRONT, bneck, ctr, hist, ctl);
            k_wave_count<<<gstat, 256, 0, ctx->stream>>>(split, ctr + WC_SPLIT, bneck, ctr, ctl);
            k_wave_decide<<<1, DECIDE_THREADS, 0, ctx->stream>>>(ctr, hist, ctl, (uint32_t)N, (uint32_t)cap, force);
            k_wave_select<<<gstat, 256, 0, ctx->stream>>>(fa, fb, ctr + WC_FRONT, bneck, expand, split, ctr, ctl);
            k_wave_split<F, DIM, SH><<<gsplit, WAVE_WARPS * 32, 0, ctx->stream>>>(
                f, expand, ctr + WC_EXPAND, kdim, (uint32_t)cap, vals, rmin, rmax, vol, child, parent, fresh, fa, fb,
                ctr, ctl);
            k_wave_eval<F, DIM, SH, SL><<<geval, WAVE_WARPS * 32, 0, ctx->stream>>>(
                tc, fresh, ctr + WC_NEW, vals, rmin, rmax, vol, parent, key, kdim, bneck, ctr, ctl);
            k_wave_swap<<<1, 1, 0, ctx->stream>>>(ctr, ctl);
            launches += 7;
        }
        VCU_CUDA(ctx, cudaGetLastError());
        return VCU_OK;
    };
    /* The heap sequence is replayed on the host while the device runs the next waves: after each
     * chunk the device copies the loop state, the errors, split dimensions and children into snapshot
     * buffers; the next chunk is launched at once (it does nothing once the loop is done), and the
     * copy stream brings the snapshot to the host, where the replay goes on until it meets a region
     * no wave has split yet.  A region's children and their errors come from the same wave, and a
     * snapshot is taken between waves, so every region the replay reads is final. */
    float* skey = reinterpret_cast<float*>(base + o_skey);
    int* sdim = reinterpret_cast<int*>(base + o_sdim);
    int* schild = reinterpret_cast<int*>(base + o_schild);
    uint32_t* sctr = reinterpret_cast<uint32_t*>(base + o_sctr);
    WaveCtl* sctl = reinterpret_cast<WaveCtl*>(sctr + WC_N);
    HeapReplay replay{H.data()};
    int missing = -1;
    auto replay_more = [&]() { missing = replay.run(N, hkey.data(), hdim.data(), hchild.data()); };
    for (int round = 0; round < 8; ++round) {
        /* waves, WAVE_CHUNK at a time without a host round trip: the device decides between waves
         * (k_wave_decide) and every kernel of a wave after the last returns at once */
        if ((rc = chunk())) return rc;
        for (;;) {
            VCU_CUDA(ctx, cudaMemcpyAsync(sctr, ctr, WC_N * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(sctl, ctl, sizeof(WaveCtl), cudaMemcpyDeviceToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(skey, key, cap * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(sdim, kdim, cap * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(schild, child, cap * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaEventRecord(ctx->ev_snap, ctx->stream));
            if ((rc = chunk())) return rc;
            VCU_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_snap, 0));
            uint32_t hctr[WC_N];
            WaveCtl hc{};
            VCU_CUDA(ctx, cudaMemcpyAsync(hctr, sctr, WC_N * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(&hc, sctl, sizeof(hc), cudaMemcpyDeviceToHost, ctx->copy_stream));
            VCU_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
            if (hc.state == WAVE_FAIL) { /* pool too small, or NaN errors: the sequential generator */
                VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                return -1;
            }
            const uint32_t pool = hctr[WC_POOL] < cap ? hctr[WC_POOL] : (uint32_t)cap;
            hkey.resize(pool);
            hdim.resize(pool);
            hchild.resize(pool);
            VCU_CUDA(ctx, cudaMemcpyAsync(hkey.data(), skey, (size_t)pool * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(hdim.data(), sdim, (size_t)pool * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(hchild.data(), schild, (size_t)pool * 4, cudaMemcpyDeviceToHost,
                                          ctx->copy_stream));
            VCU_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
            replay_more();
            if (hc.state == WAVE_DONE) break;
        }
        VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (missing < 0) {
            for (size_t i = 0; i <= N; ++i) HS[i] = H[i].pay;
            VCU_CUDA(ctx, cudaMemcpyAsync(hp, HS.data(), (N + 1) * 4, cudaMemcpyHostToDevice, ctx->stream));
            return regions_into_bins<F, DIM, SH, SL>(ctx, residual_functor(f), p, g, cv, vals, rmin, rmax, vol, hp, N + 1,
                                                     reinterpret_cast<uint32_t*>(base + o_cnt),
                                                     reinterpret_cast<uint32_t*>(base + o_off),
                                                     reinterpret_cast<uint32_t*>(base + o_cur), d_replay, d_bins,
                                                     d_approx, d_regions, launches);
        }
        hb.resize(hkey.size());
        VCU_CUDA(ctx, cudaMemcpyAsync(hb.data(), bneck, hb.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
        VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        /* the sequence needs a region no wave split: split every unsplit region down to its b */
        uint32_t u;
        std::memcpy(&u, &hb[missing], 4);
        if (u & 0x80000000u) u = 0;
        force = u >> WAVE_SHIFT;
        const uint32_t active = WAVE_ACTIVE;
        VCU_CUDA(ctx, cudaMemcpyAsync(&ctl->state, &active, 4, cudaMemcpyHostToDevice, ctx->stream));
    }
    return -1;
}

}  // namespace cv_detail

template <int SH, int SL>
int run_cv_pair(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, int iterations,
                const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                uint32_t& launches) {
    using cv_detail::ipow;
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        auto by_dim = [&](auto dimc) -> int {
            constexpr int DIM = decltype(dimc)::value;
            if constexpr (ipow(SH, DIM) <= 243)
                return cv_detail::cv_launch<DIM, SH, SL>(ctx, f, p, g, nst, iterations, cv, d_replay, d_bins, d_approx,
                                                         d_regions, launches);
            else
                return fail(ctx, VCU_UNSUPPORTED, "control-variate regions are limited to 243 nodes (S^dim)");
        };
        if constexpr (F::DIM == 6) {
            switch (p->dim) {
            case 2: return by_dim(std::integral_constant<int, 2>{});
            case 3: return by_dim(std::integral_constant<int, 3>{});
            case 4: return by_dim(std::integral_constant<int, 4>{});
            case 5: return by_dim(std::integral_constant<int, 5>{});
            default: return fail(ctx, VCU_UNSUPPORTED, "half-space control variates are built for 2-5 dimensions");
            }
        } else {
            return by_dim(std::integral_constant<int, F::DIM>{});
        }
    });
}

/* the tolerance-driven form for one rule pair (same dimension limits as the control variates) */
template <int SH, int SL>
int run_tol_pair(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& nst, float tol,
                 uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches) {
    using cv_detail::ipow;
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        auto by_dim = [&](auto dimc) -> int {
            constexpr int DIM = decltype(dimc)::value;
            if constexpr (ipow(SH, DIM) <= 243)
                return cv_detail::tol_launch<DIM, SH, SL>(ctx, f, p, g, nst, tol, max_regions, d_bins, nregions, nleaves,
                                                          launches);
            else
                return fail(ctx, VCU_UNSUPPORTED, "tolerance-driven regions are limited to 243 nodes (S^dim)");
        };
        if constexpr (F::DIM == 6) {
            switch (p->dim) {
            case 2: return by_dim(std::integral_constant<int, 2>{});
            case 3: return by_dim(std::integral_constant<int, 3>{});
            case 4: return by_dim(std::integral_constant<int, 4>{});
            case 5: return by_dim(std::integral_constant<int, 5>{});
            default: return fail(ctx, VCU_UNSUPPORTED, "half-space regions are built for 2-5 dimensions");
            }
        } else {
            return by_dim(std::integral_constant<int, F::DIM>{});
        }
    });
}

}  // namespace vcu
