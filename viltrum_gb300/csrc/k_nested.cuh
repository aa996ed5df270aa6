/*
 * k_nested.cu -- per-bin adaptive nested Newton-Cotes on the device.
 *
 * Replaces integrator_per_bin_parallel(integrator_adaptive_iterations(nested(H,L), heuristic,
 * iterations)): for every bin, the reference builds a root region over the bin
 * (src/newton-cotes/region.h:74-78), then `iterations` times pops the region of largest error
 * estimate from a std heap, splits it in two along its worst dimension re-using the parent's
 * even nodes (region.h:345-359, src/multiarray/split.h:13-49), estimates the children's errors
 * (region.h:387-418, src/nested/error-heuristic.h) and pushes them
 * (src/nested/regions-generator-adaptive-heap.h:18-45); finally it integrates every region over
 * its intersection with the bin, in heap order (src/newton-cotes/regions-integrator-sequential.h:37-58),
 * and scales by prod(res) (src/integrator-per-bin-parallel.h:33).
 *
 * GB300 mapping: a group of G lanes of a warp owns one bin at a time (grid-stride over bins, a
 * persistent grid sized by occupancy).  All node values of the bin's live regions, their ranges,
 * the heap and the scratch of the error folds live in the group's slice of shared memory; the
 * group evaluates the integrand at a region's new nodes in parallel (Boole 2-D: 20 new nodes per
 * split; with 8 lanes and integrands that evaluate several points as independent chains, one round
 * of up to 3 points per lane), folds the per-line error metrics in parallel, and one lane keeps the
 * heap.  Nothing touches global memory but the integrand parameters (kernel parameter space)
 * and the bin writes.
 */
#pragma once
#include <cstdlib>

#include "vcu_heap.h"
#include "vcu_internal.cuh"
#include "vcu_rules.cuh"

namespace vcu {

namespace nc_detail {

constexpr int NC_THREADS = 128;

__host__ __device__ constexpr int ipow(int b, int e) { return e <= 0 ? 1 : b * ipow(b, e - 1); }

struct NcCfg {
    int32_t iters;
    int32_t nslot;
    int32_t nheap;
    int32_t words_per_group;
    int32_t heuristic, relative;
    float min_val_f;  /* smallest float >= error_metric_relative's min_val */
    double size_weight;
    double min_size;
};

template <int DIM, int S, int CH> struct Layout {
    static constexpr int SD = ipow(S, DIM);
    static constexpr int NL = ipow(S, DIM - 1);
    /* words of one group's slice for a given slot/heap count */
    /* scratch of a split (line metrics, per-dimension errors, node coordinates); the final
     * contributions of the regions reuse it (and extend it if they need more room) */
    static constexpr int SCRATCH = 2 * DIM * NL + 2 * DIM + DIM * S + (S - 1);
    static __host__ __device__ int words(int nslot, int nheap) {
        const int ct = nheap * CH;
        return nslot * SD * CH              /* node values            */
               + nslot * (2 * DIM + 1)      /* ranges + volume        */
               + 2 * nheap                  /* heap keys + payloads   */
               + (ct > SCRATCH ? ct : SCRATCH);
    }
};

/* index of the node with coordinate `pos` along dimension d and the other coordinates given by J
 * (J enumerates the remaining dimensions, dim-0 fastest) */
template <int DIM, int S> __device__ __forceinline__ int node_index(int d, int J, int pos) {
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

template <int DIM, int S>
__device__ float fold_all_errors(const float* lines) {
    /* lines: S^(DIM-1) metric values, dim-0 fastest; fold dimension 0 repeatedly with the high
     * rule (the reference's fold_all(quadrature)) */
    constexpr int NL = ipow(S, DIM - 1);
    if constexpr (DIM == 1) {
        return lines[0];
    } else {
        float buf[NL];
#pragma unroll
        for (int i = 0; i < NL; ++i) buf[i] = lines[i];
        int n = NL;
#pragma unroll
        for (int level = 0; level < DIM - 1; ++level) {
            n /= S;
            for (int i = 0; i < n; ++i) buf[i] = RefRule<S>::scalar(buf + i * S);
        }
        return buf[0];
    }
}

/* integral of one region's polynomial over its intersection [A,B] (normalised), folding the
 * last dimension first (region.h:141-150); values of channel c */
template <int DIM, int S, int CH>
__device__ float region_subrange(const float* V, int c, const float* A, const float* B) {
    constexpr int SD = ipow(S, DIM);
    float buf[SD / S];
    /* first level: fold dimension DIM-1 straight from shared memory */
    constexpr int inner = SD / S;
#pragma unroll
    for (int i = 0; i < inner; ++i) {
        float line[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = V[(i + j * inner) * CH + c];
        buf[i] = Rule<S>::subrange(A[DIM - 1], B[DIM - 1], line);
    }
    int n = inner;
#pragma unroll
    for (int d = DIM - 2; d >= 0; --d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i + j * m];
            buf[i] = Rule<S>::subrange(A[d], B[d], line);
        }
        n = m;
    }
    return buf[0];
}

/* Newton-Cotes weights of an S-node rule on [0, 1]: the exact integral of the interpolant */
/* region_subrange() over the whole region, [0, 1] in every dimension (Rule<S>::subrange01) */
template <int DIM, int S, int CH>
__device__ float region_subrange01(const float* V, int c) {
    constexpr int SD = ipow(S, DIM);
    constexpr int inner = SD / S;
    float buf[inner];
#pragma unroll
    for (int i = 0; i < inner; ++i) {
        float line[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = V[(i + j * inner) * CH + c];
        buf[i] = Rule<S>::subrange01(line);
    }
    int n = inner;
#pragma unroll
    for (int d = DIM - 2; d >= 0; --d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i + j * m];
            buf[i] = Rule<S>::subrange01(line);
        }
        n = m;
    }
    return buf[0];
}

/* culled evaluation when the integrand supports it over the kernel's full dimension */
template <class F, int DIM> constexpr bool use_cull = has_cull<F>::value && DIM == F::DIM;
template <class F, bool = has_cull<F>::value> struct cull_of { using type = int; };
template <class F> struct cull_of<F, true> { using type = typename F::Cull; };

template <int N, int DIM, class F>
__device__ __forceinline__ void eval_points(const F& f, const typename cull_of<F>::type& cl, const float (*xs)[F::DIM],
                                            float (*vs)[F::CH]) {
    if constexpr (use_cull<F, DIM>) f.template multi_cull<N>(cl, xs, vs);
    else f.template multi<N>(xs, vs);
}

template <class F, int DIM, int SH, int SL, int G>
__global__ void __launch_bounds__(NC_THREADS, DIM == 2 ? 6 : 1) k_per_bin_nested(const __grid_constant__ F f, const BinGrid g,
                                                               const NcCfg cfg, float* __restrict__ bins,
                                                               int32_t* __restrict__ trace,
                                                               uint32_t* __restrict__ status) {
    constexpr int S = SH;
    constexpr int CH = F::CH;
    constexpr int SD = ipow(S, DIM);
    constexpr int NL = ipow(S, DIM - 1);
    constexpr int NNEW = (S - 1) * NL;
    extern __shared__ float smem[];

    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const int gib = threadIdx.x / G;
    const int gpb = blockDim.x / G;

    float* V = smem + (size_t)gib * cfg.words_per_group;
    float* RMIN = V + cfg.nslot * SD * CH;
    float* RMAX = RMIN + cfg.nslot * DIM;
    float* VOL = RMAX + cfg.nslot * DIM;
    float* HE = VOL + cfg.nslot;
    int* HS = reinterpret_cast<int*>(HE + cfg.nheap);
    float* LN = reinterpret_cast<float*>(HS + cfg.nheap);
    float* EC = LN + 2 * DIM * NL;
    float* CO = EC + 2 * DIM;
    float* CN = CO + DIM * S;
    float* CT = LN; /* the final contributions reuse the split scratch */

    const uint64_t ngroups = (uint64_t)gridDim.x * gpb;
    const int iters = cfg.iters;

    for (uint64_t bin = (uint64_t)blockIdx.x * gpb + gib; bin < g.nbins; bin += ngroups) {
        /* ---- bin sub-range (integrator-per-bin-parallel.h:30-32) */
        auto bin_box = [&](uint64_t b, float* lo, float* hi) {
            uint64_t rem = b;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                if (d < g.dimbins) {
                    const uint32_t pos = (uint32_t)(rem % g.res[d]);
                    rem /= g.res[d];
                    lo[d] = vadd(g.rmin[d], vmul((float)pos, g.drange[d]));
                    hi[d] = vadd(g.rmin[d], vmul((float)(pos + 1), g.drange[d]));
                } else {
                    lo[d] = g.rmin[d];
                    hi[d] = g.rmax[d];
                }
            }
        };
        float bmin[DIM], bmax[DIM];
        bin_box(bin, bmin, bmax);
        /* terms of the integrand that can be non-zero in the box of the bins of this warp's groups
         * (consecutive bins): one list for the whole warp, so the term loop stays uniform */
        [[maybe_unused]] typename cull_of<F>::type cl{};
        if constexpr (use_cull<F, DIM>) {
            constexpr int GPW = 32 / G;
            const uint64_t w0 = bin - (uint64_t)(gib % GPW);
            float lo[DIM], hi[DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                lo[d] = bmin[d];
                hi[d] = bmax[d];
            }
#pragma unroll 1
            for (int k = 0; k < GPW; ++k) {
                if (w0 + k >= g.nbins) break;
                float l2[DIM], h2[DIM];
                bin_box(w0 + k, l2, h2);
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    lo[d] = fminf(lo[d], l2[d]);
                    hi[d] = fmaxf(hi[d], h2[d]);
                }
            }
            if constexpr (has_cull_terms<F>::value) {
                /* the group's lanes share the per-term tests; one vote per G terms */
                float box[F::kCullBox];
                f.cull_prepare(lo, hi, box);
                uint32_t words[F::kCullWords];
                const int gbase = lane & ~(G - 1);
                constexpr uint32_t gbits = (G == 32) ? 0xffffffffu : ((1u << (G & 31)) - 1u);
#pragma unroll
                for (int k = 0; k < F::kCullWords; ++k) {
                    uint32_t word = 0u;
#pragma unroll
                    for (int q = 0; q < 32 / G; ++q) {
                        const uint32_t b = __ballot_sync(gmask, f.cull_keep(32 * k + G * q + gl, box));
                        word |= ((b >> gbase) & gbits) << (G * q);
                    }
                    words[k] = word;
                }
                cl = F::cull_from_words(words);
            } else {
                cl = f.cull(lo, hi);
            }
        }
        /* ---- root region in slot 0 */
        if (gl == 0) {
            float vol = 1.0f;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                RMIN[d] = bmin[d];
                RMAX[d] = bmax[d];
                vol = vmul(vol, vsub(bmax[d], bmin[d]));
            }
            VOL[0] = vol;
        }
        for (int t = gl; t < DIM * S; t += G) {
            const int d = t / S, j = t % S;
            CO[t] = node_coord(node_pos<S>(j), vsub(bmax[d], bmin[d]), bmin[d]);
        }
        __syncwarp(gmask);
        auto root_x = [&](int t, float* x) {
#pragma unroll
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
            int rem = t;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                x[d] = CO[d * S + rem % S];
                rem /= S;
            }
        };
        if constexpr (has_multi<F>::value) {
            constexpr int NR = (SD + G - 1) / G > 4 ? 4 : (SD + G - 1) / G;
            for (int t = gl; t < SD; t += NR * G) {
                float xs[NR][F::DIM], vs[NR][CH];
#pragma unroll
                for (int q = 0; q < NR; ++q) root_x(t + q * G < SD ? t + q * G : t, xs[q]);
                eval_points<NR, DIM>(f, cl, xs, vs);
#pragma unroll
                for (int q = 0; q < NR; ++q)
                    if (q == 0 || t + q * G < SD) {
#pragma unroll
                        for (int c = 0; c < CH; ++c) V[(t + q * G) * CH + c] = vs[q][c];
                    }
            }
        } else if constexpr (has_pair<F>::value) {
            for (int t = gl; t < SD; t += 2 * G) {
                const int t2 = t + G < SD ? t + G : t;
                float x0[F::DIM], x1[F::DIM], v0[CH], v1[CH];
                root_x(t, x0);
                root_x(t2, x1);
                f.pair(x0, x1, v0, v1);
#pragma unroll
                for (int c = 0; c < CH; ++c) V[t * CH + c] = v0[c];
                if (t2 != t) {
#pragma unroll
                    for (int c = 0; c < CH; ++c) V[t2 * CH + c] = v1[c];
                }
            }
        } else {
            for (int t = gl; t < SD; t += G) {
                float x[F::DIM], v[CH];
                root_x(t, x);
                f(x, v);
#pragma unroll
                for (int c = 0; c < CH; ++c) V[t * CH + c] = v[c];
            }
        }
        __syncwarp(gmask);

        /* ---- error estimates of `nreg` regions (slots s0, s1) into EC[r*DIM + d] */
        auto region_errors = [&](auto nreg_c, int s0, int s1) {
            constexpr int NT = decltype(nreg_c)::value * DIM * NL; /* lines */
            auto line_of = [&](int t, int c, float* line, float* low) {
                const int r = t / (DIM * NL), rr = t % (DIM * NL);
                const int d = rr / NL, J = rr % NL;
                const float* RV = V + (size_t)(r ? s1 : s0) * SD * CH;
#pragma unroll
                for (int i = 0; i < S; ++i) line[i] = RV[node_index<DIM, S>(d, J, i) * CH + c];
#pragma unroll
                for (int i = 0; i < SL; ++i) low[i] = line[i * (S - 1) / (SL - 1)];
            };
            if constexpr (CH == 1) {
                for (int t = gl; t < NT; t += G) {
                    float line[S], low[SL];
                    line_of(t, 0, line, low);
                    LN[t] = metric_value(cfg.relative, cfg.min_val_f, RefRule<S>::scalar(line), RefRule<SL>::scalar(low));
                }
            } else {
                for (int t = gl; t < NT; t += G) {
                    float m = 0.0f;
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        float line[S], low[SL];
                        line_of(t, c, line, low);
                        const float mv =
                            metric_value(cfg.relative, cfg.min_val_f, RefRule<S>::rgb(line), RefRule<SL>::rgb(low));
                        m = (c == 0) ? mv : vadd(m, mv);
                    }
                    LN[t] = m;
                }
            }
            __syncwarp(gmask);
            const int nreg = decltype(nreg_c)::value;
            for (int t = gl; t < nreg * DIM; t += G) {
                const int r = t / DIM;
                const float folded = fold_all_errors<DIM, S>(LN + t * NL);
                EC[t] = vmul(VOL[r ? s1 : s0], folded);
            }
            __syncwarp(gmask);
        };
        /* heuristic over EC[r*DIM ..] for the region in slot s (lane 0 only) */
        auto heuristic = [&](int r, int s, float& err_out, int& dim_out) {
            const float* e = EC + r * DIM;
            if (cfg.heuristic == VCU_HEUR_DEFAULT) {
                float max_err = 0.0f;
                int max_dim = 0;
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    if (e[d] > max_err) {
                        max_err = e[d];
                        max_dim = d;
                    }
                err_out = max_err;
                dim_out = max_dim;
                return;
            }
            float w = vsub(RMAX[s * DIM], RMIN[s * DIM]);
            float max_err;
            if ((double)w < cfg.min_size || isnan(w)) max_err = 0.0f;
            else max_err = __double2float_rn(__dadd_rn((double)e[0], __dmul_rn(cfg.size_weight, (double)fabsf(w))));
            int max_dim = 0;
#pragma unroll
            for (int d = 1; d < DIM; ++d) {
                w = vsub(RMAX[s * DIM + d], RMIN[s * DIM + d]);
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

        region_errors(std::integral_constant<int, 1>{}, 0, 0);
        if (gl == 0) {
            float e;
            int dm;
            heuristic(0, 0, e, dm);
            HE[0] = e;
            HS[0] = 0 | (dm << 8);
        }
        uint64_t freemask = (cfg.nslot >= 64 ? ~0ull : ((1ull << cfg.nslot) - 1ull)) & ~1ull;

        for (int it = 0; it < iters; ++it) {
            __syncwarp(gmask);
            const int top = HS[0];
            const int P = top & 0xff, dd = top >> 8;
            const int C0 = __ffsll((long long)freemask) - 1;
            freemask &= freemask - 1;
            const int C1 = __ffsll((long long)freemask) - 1;
            freemask &= freemask - 1;
            /* node coordinates of the parent (other dimensions) and of the new nodes along dd */
            for (int t = gl; t < DIM * S + (S - 1); t += G) {
                if (t < DIM * S) {
                    const int d = t / S, j = t % S;
                    const float mn = RMIN[P * DIM + d];
                    CO[t] = node_coord(node_pos<S>(j), vsub(RMAX[P * DIM + d], mn), mn);
                } else {
                    const int k = t - DIM * S;
                    const float mn = RMIN[P * DIM + dd];
                    CN[k] = node_coord(mid_pos<S>(k), vsub(RMAX[P * DIM + dd], mn), mn);
                }
            }
            __syncwarp(gmask);
            float* VP = V + (size_t)P * SD * CH;
            float* V0 = V + (size_t)C0 * SD * CH;
            float* V1 = V + (size_t)C1 * SD * CH;
            /* new nodes: odd positions of the 2(S-1)+1 grid along dd; two per lane and round when the
             * integrand can evaluate two points as independent chains */
            auto node_x = [&](int t, float* x) {
                const int k = t / NL, J = t % NL;
#pragma unroll
                for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
                int rem = J;
#pragma unroll
                for (int e = 0; e < DIM; ++e) {
                    if (e == dd) continue;
                    x[e] = CO[e * S + rem % S];
                    rem /= S;
                }
                x[dd] = CN[k];
            };
            auto store_new = [&](int t, const float* v) {
                const int k = t / NL, J = t % NL;
                const int i = 2 * k + 1;
                if (i <= S - 1) {
                    const int n0 = node_index<DIM, S>(dd, J, i);
#pragma unroll
                    for (int c = 0; c < CH; ++c) V0[n0 * CH + c] = v[c];
                }
                if (i >= S - 1) {
                    const int n1 = node_index<DIM, S>(dd, J, i - (S - 1));
#pragma unroll
                    for (int c = 0; c < CH; ++c) V1[n1 * CH + c] = v[c];
                }
            };
            if constexpr (has_multi<F>::value) {
                /* NP points per lane in one pass: all of a split's new nodes in one round when
                 * NNEW <= 4 G */
                constexpr int NP = (NNEW + G - 1) / G > 4 ? 4 : (NNEW + G - 1) / G;
                for (int t = gl; t < NNEW; t += NP * G) {
                    float xs[NP][F::DIM], vs[NP][CH];
#pragma unroll
                    for (int q = 0; q < NP; ++q) node_x(t + q * G < NNEW ? t + q * G : t, xs[q]);
                    eval_points<NP, DIM>(f, cl, xs, vs);
#pragma unroll
                    for (int q = 0; q < NP; ++q)
                        if (q == 0 || t + q * G < NNEW) store_new(t + q * G, vs[q]);
                }
            } else if constexpr (has_pair<F>::value) {
                for (int t = gl; t < NNEW; t += 2 * G) {
                    const int t2 = t + G < NNEW ? t + G : t;
                    float x0[F::DIM], x1[F::DIM], v0[CH], v1[CH];
                    node_x(t, x0);
                    node_x(t2, x1);
                    f.pair(x0, x1, v0, v1);
                    store_new(t, v0);
                    if (t2 != t) store_new(t2, v1);
                }
            } else {
                for (int t = gl; t < NNEW; t += G) {
                    float x[F::DIM], v[CH];
                    node_x(t, x);
                    f(x, v);
                    store_new(t, v);
                }
            }
            /* parent nodes re-used at the even positions */
            for (int t = gl; t < S * NL; t += G) {
                const int m = t / NL, J = t % NL;
                const int i = 2 * m;
                const int src = node_index<DIM, S>(dd, J, m);
                if (i <= S - 1) {
                    const int n0 = node_index<DIM, S>(dd, J, i);
#pragma unroll
                    for (int c = 0; c < CH; ++c) V0[n0 * CH + c] = VP[src * CH + c];
                }
                if (i >= S - 1) {
                    const int n1 = node_index<DIM, S>(dd, J, i - (S - 1));
#pragma unroll
                    for (int c = 0; c < CH; ++c) V1[n1 * CH + c] = VP[src * CH + c];
                }
            }
            if (gl == 0) {
                const float pmn = RMIN[P * DIM + dd], pmx = RMAX[P * DIM + dd];
                const float half = vmul(vsub(pmx, pmn), 0.5f); /* = (max - min) / 2.0, exactly */
                const float mid = vadd(pmn, vmul(half, 1.0f));
                float vol0 = 1.0f, vol1 = 1.0f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const float mn = RMIN[P * DIM + d], mx = RMAX[P * DIM + d];
                    const float mx0 = (d == dd) ? mid : mx;
                    const float mn1 = (d == dd) ? mid : mn;
                    RMIN[C0 * DIM + d] = mn;
                    RMAX[C0 * DIM + d] = mx0;
                    RMIN[C1 * DIM + d] = mn1;
                    RMAX[C1 * DIM + d] = mx;
                    vol0 = vmul(vol0, vsub(mx0, mn));
                    vol1 = vmul(vol1, vsub(mx, mn1));
                }
                VOL[C0] = vol0;
                VOL[C1] = vol1;
            }
            __syncwarp(gmask);
            region_errors(std::integral_constant<int, 2>{}, C0, C1);
            if (gl == 0) {
                float e0, e1;
                int d0, d1;
                heuristic(0, C0, e0, d0);
                heuristic(1, C1, e1, d1);
                if (trace) {
                    trace[((size_t)bin * iters + it) * 2] = dd;
                    trace[((size_t)bin * iters + it) * 2 + 1] = __float_as_int(HE[0]);
                }
                const int n = it + 1; /* heap size before this split */
                heap_pop(HE, HS, n);
                HE[n - 1] = e0;
                HS[n - 1] = C0 | (d0 << 8);
                heap_push(HE, HS, n);
                HE[n] = e1;
                HS[n] = C1 | (d1 << 8);
                heap_push(HE, HS, n + 1);
            }
            freemask |= 1ull << P;
        }
        __syncwarp(gmask);
        /* ---- integrate each region over its intersection with the bin
         * (regions-integrator-sequential.h:37-58 with a single bin: the bin range is the bin's
         * sub-range with dimension 0 rebuilt as min + 1*(max-min)) */
        const int nreg = iters + 1;
        for (int k = gl; k < nreg; k += G) {
            const int s = HS[k] & 0xff;
            float a[DIM], b[DIM];
            bool empty = false, whole = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const float blo = bmin[d];
                const float bhi = (d == 0) ? vadd(bmin[0], vmul(1.0f, vdiv(vsub(bmax[0], bmin[0]), 1.0f))) : bmax[d];
                const float rmn = RMIN[s * DIM + d], rmx = RMAX[s * DIM + d];
                a[d] = smax(blo, rmn);
                b[d] = smax(a[d], smin(bhi, rmx));
                empty = empty || (a[d] >= b[d]);
                whole = whole && a[d] == rmn && b[d] == rmx;
            }
            if (empty) {
                CT[k * CH] = __int_as_float(0x7fc00001); /* marker: skipped region */
            } else if (whole) {
                /* the region lies inside the bin (every region, unless the bin's first upper bound,
                 * rebuilt as min + (max - min), rounds below it): the normalised intersection is
                 * [0, 1] in every dimension, A and B need no division */
#pragma unroll
                for (int c = 0; c < CH; ++c)
                    CT[k * CH + c] = vmul(VOL[s], region_subrange01<DIM, S, CH>(V + (size_t)s * SD * CH, c));
            } else {
                float A[DIM], B[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const float rmn = RMIN[s * DIM + d], rmx = RMAX[s * DIM + d];
                    A[d] = (rmn >= rmx) ? rmn : vdiv(vsub(a[d], rmn), vsub(rmx, rmn));
                    B[d] = (rmn >= rmx) ? rmn : vdiv(vsub(b[d], rmn), vsub(rmx, rmn));
                }
#pragma unroll
                for (int c = 0; c < CH; ++c)
                    CT[k * CH + c] = vmul(VOL[s], region_subrange<DIM, S, CH>(V + (size_t)s * SD * CH, c, A, B));
            }
        }
        __syncwarp(gmask);
        if (gl == 0) {
            float sol[CH];
#pragma unroll
            for (int c = 0; c < CH; ++c) sol[c] = 0.0f;
            for (int k = 0; k < nreg; ++k) {
                if (__float_as_int(CT[k * CH]) == 0x7fc00001) continue;
#pragma unroll
                for (int c = 0; c < CH; ++c) sol[c] = vadd(sol[c], CT[k * CH + c]);
            }
            bool nan = false;
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                const float v = vmul(g.factor, sol[c]);
                nan = nan || isnan(v);
                bins[bin * CH + c] = v;
            }
            if (nan) atomicOr(status, VCU_FLAG_NAN);
        }
        __syncwarp(gmask);
    }
}

template <int DIM, int S> constexpr int lanes_per_bin() {
    /* lanes sharing one bin: enough to cover one split's new nodes in a few rounds */
    return ((S - 1) * ipow(S, DIM - 1) <= 24) ? 4 : (((S - 1) * ipow(S, DIM - 1) <= 64) ? 8 : 32);
}

template <int DIM, int SH, int SL, int G, class F>
int launch_g(vcu_ctx* ctx, const F& f, const BinGrid& g, const vcu_nested& n, int iterations, float* d_bins,
             int32_t* d_trace, uint32_t& launches) {
    using Lay = Layout<DIM, SH, F::CH>;
    NcCfg cfg{};
    cfg.iters = iterations;
    cfg.nslot = iterations + 2;
    cfg.nheap = iterations + 1;
    int w = Lay::words(cfg.nslot, cfg.nheap);
    /* pad so that consecutive groups start G banks apart: conflict-free same-offset accesses */
    while ((w & 31) != (G & 31)) ++w;
    cfg.words_per_group = w;
    cfg.heuristic = n.heuristic;
    cfg.relative = n.metric == VCU_METRIC_RELATIVE;
    float mv = (float)n.min_val;
    if ((double)mv < n.min_val) mv = nextafterf(mv, INFINITY);
    cfg.min_val_f = mv;
    cfg.size_weight = n.size_weight;
    cfg.min_size = n.min_size;
    /* bins per block: as many as fit in shared memory, up to NC_THREADS / G */
    int gpb = NC_THREADS / G;
    while (gpb > 1 && (size_t)gpb * (size_t)w * 4 > ctx->smem_optin) gpb /= 2;
    const size_t smem = (size_t)gpb * (size_t)w * 4;
    if (smem > ctx->smem_optin)
        return fail(ctx, VCU_UNSUPPORTED,
                    "per-bin region storage of " + std::to_string(smem) + " bytes exceeds shared memory");
    const int threads = gpb * G;
    auto kern = k_per_bin_nested<F, DIM, SH, SL, G>;
    VCU_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VCU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    if (per_sm < 1) per_sm = 1;
    const uint64_t need = (g.nbins + gpb - 1) / gpb;
    const uint64_t cap = (uint64_t)ctx->sm_count * per_sm;
    const unsigned blocks = (unsigned)(need < cap ? need : cap);
    kern<<<blocks, threads, smem, ctx->stream>>>(f, g, cfg, d_bins, d_trace, ctx->d_status);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    return VCU_OK;
}

/* Lanes per bin (G) does not change any result -- every value is computed by one lane with the
 * same arithmetic -- only occupancy and lane utilisation.  For 2-D regions three variants are built
 * and the context's autotuner times each once on the caller's problem (first use of a
 * configuration), then reuses the fastest.  VCU_NESTED_LANES=4|8|16 forces a variant. */
template <int DIM, int SH, int SL, class F>
int launch(vcu_ctx* ctx, const F& f, const BinGrid& g, const vcu_nested& n, int iterations, float* d_bins,
           int32_t* d_trace, uint32_t& launches) {
    if constexpr (DIM == 2 && (SH - 1) * SH <= 24) {
        auto run = [&](int G) -> int {
            switch (G) {
            case 4: return launch_g<DIM, SH, SL, 4>(ctx, f, g, n, iterations, d_bins, d_trace, launches);
            case 16: return launch_g<DIM, SH, SL, 16>(ctx, f, g, n, iterations, d_bins, d_trace, launches);
            default: return launch_g<DIM, SH, SL, 8>(ctx, f, g, n, iterations, d_bins, d_trace, launches);
            }
        };
        if (const char* env = std::getenv("VCU_NESTED_LANES")) {
            const int G = std::atoi(env);
            if (G == 4 || G == 8 || G == 16) return run(G);
        }
        if (!ctx->tune || g.nbins < 4096 || d_trace) return run(8);
        /* key: integrand functor size and arity, rules, iterations, bins (coarse) */
        const uint64_t key = ((uint64_t)sizeof(F) << 40) ^ ((uint64_t)F::DIM << 36) ^ ((uint64_t)SH << 32) ^
                             ((uint64_t)SL << 28) ^ ((uint64_t)iterations << 20) ^ (uint64_t)(63 - __builtin_clzll(g.nbins));
        for (int i = 0; i < ctx->ntuned; ++i)
            if (ctx->tuned[i].key == key) return run(ctx->tuned[i].value);
        int best = 8;
        float best_ms = 1e30f;
        for (int G : {4, 8, 16}) {
            VCU_CUDA(ctx, cudaEventRecord(ctx->ev_tune[0], ctx->stream));
            const int rc = run(G);
            if (rc) return rc;
            VCU_CUDA(ctx, cudaEventRecord(ctx->ev_tune[1], ctx->stream));
            VCU_CUDA(ctx, cudaEventSynchronize(ctx->ev_tune[1]));
            float ms = 0.0f;
            VCU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_tune[0], ctx->ev_tune[1]));
            if (ms < best_ms) {
                best_ms = ms;
                best = G;
            }
        }
        if (ctx->ntuned < 32) ctx->tuned[ctx->ntuned++] = vcu_tuned{key, best};
        return VCU_OK; /* every timed launch wrote the same bins */
    } else {
        return launch_g<DIM, SH, SL, lanes_per_bin<DIM, SH>()>(ctx, f, g, n, iterations, d_bins, d_trace, launches);
    }
}

}  // namespace nc_detail
using namespace nc_detail;

/* per-bin nested quadrature for one rule pair; region storage is limited to S^dim <= 125
 * nodes (Boole up to 3-D, Simpson up to 4-D) */
template <int SH, int SL>
int run_nested_pair(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                    float* d_bins, int32_t* d_trace, uint32_t& launches) {
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        auto by_dim = [&](auto dimc) -> int {
            constexpr int DIM = decltype(dimc)::value;
            if constexpr (ipow(SH, DIM) <= 125)
                return launch<DIM, SH, SL>(ctx, f, g, n, iterations, d_bins, d_trace, launches);
            else
                return fail(ctx, VCU_UNSUPPORTED, "per-bin nested regions are limited to 125 nodes (S^dim)");
        };
        if constexpr (F::DIM == 6) {
            /* the half-space functor takes its arity at run time */
            switch (p->dim) {
            case 2: return by_dim(std::integral_constant<int, 2>{});
            case 3: return by_dim(std::integral_constant<int, 3>{});
            default:
                return fail(ctx, VCU_UNSUPPORTED,
                            "per-bin nested quadrature of the half-space integrand is built for 2-3 dimensions");
            }
        } else if constexpr (F::DIM <= 4) {
            return by_dim(std::integral_constant<int, F::DIM>{});
        } else {
            return fail(ctx, VCU_UNSUPPORTED, "per-bin nested quadrature is built for up to 4 dimensions");
        }
    });
}

}  // namespace vcu
