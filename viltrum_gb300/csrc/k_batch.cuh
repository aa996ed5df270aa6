/*
 * k_batch.cuh -- many independent single-value integrals of uneven dimension and budget in one
 * persistent launch.
 *
 * Each item is viltrum::integrate(I, f, range) (src/integrate.h:105-113: a call with one bin of
 * resolution {1}) for
 *   MONTE_CARLO : I = monte_carlo(budget, seed) (src/monte-carlo/monte-carlo.h:39-63): the value is
 *                 volume/budget * sum of f over `budget` uniform points of the range.  The points
 *                 come from Philox4x32-10 keyed by the item's seed, counter (sample, item, 0xBA7C0000
 *                 + word block) instead of the item's std::mt19937, so the check is statistical.
 *   NESTED      : I = integrator_adaptive_iterations(nested(H,L), heuristic, budget-1)
 *                 (src/nested/integrator-adaptive-iterations.h:12-15): a max-error heap over the range
 *                 split budget-1 times with the reference's decisions (error estimates with its
 *                 rounding, libstdc++ heap order), then the sum in heap order of every region's
 *                 integral over (range n region) (src/newton-cotes/regions-integrator-sequential.h:37-58
 *                 with one bin), so results match the reference's to the last bit.
 *
 * GB300 mapping.  A grid of resident blocks loops taking the next item from a device counter;
 * the host orders the items by estimated cost, largest first, so the blocks that finish early
 * keep draining small items while the long ones run.  A block works on one item with all its
 * threads: Monte Carlo items split the samples over 512 virtual lanes (FP32 Kahan per lane, FP64
 * fixed-tree lane sum, so results do not depend on the block size); nested items evaluate a split's new nodes, the per-line error metrics and the
 * level-by-level error folds in parallel, while one thread keeps the heap.  Unlike the per-bin
 * kernel, a nested item's regions (node values, ranges, volumes: up to 65 537 regions of 729
 * nodes) and its heap live in global memory, in a slice of a pool the host lays out per item;
 * the heap's top levels stay in L1 and each heap level costs one 16-byte load of both children.
 * Each item's wall time on the device is recorded (%globaltimer) for the tail-latency report.
 */
#pragma once
#include <algorithm>
#include <utility>

#include "k_nested.cuh"

namespace vcu {
namespace batch {

using nc_detail::ipow;
using nc_detail::node_index;

constexpr int MAX_THREADS = 1024;
constexpr int MC_LANES = 1024;
constexpr int SLOT_FLOATS = 2 * VCU_MAX_DIM; /* rmin[6], rmax[6] per region slot */
constexpr uint32_t MAX_NESTED_BUDGET = (1u << 24) - 2;

struct Item {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
    uint64_t budget, seed;
    uint64_t val_off;  /* first node value of the item's region pool          */
    uint64_t slot_off; /* first region slot (ranges, volumes) of the item      */
    uint64_t heap_off; /* first heap entry (odd, so that heap + off + 1 is 16-byte aligned) */
    int32_t dim, method, index, pad;
};

/* splits a round of a nested item attempts together: the heap's top and the regions that by their
 * keys pop after it, as many as keep a round near two passes of 512 threads (2..8) */
template <int DIM, int S> __host__ __device__ constexpr int spec_width() {
    const int tasks = ipow(S, DIM) + (S - 1) * ipow(S, DIM - 1); /* one split's children */
    const int k = 1024 / tasks;
    return k < 2 ? 2 : (k > 8 ? 8 : k);
}
/* words of shared scratch one round of a DIM-dimensional item of rule S needs: line metrics and the
 * first fold level of 2K children, node coordinates of K parents, per-dimension errors, the
 * children's node values, ranges and volumes */
template <int DIM, int S> __host__ __device__ constexpr int round_words() {
    const int K = spec_width<DIM, S>(), NL = ipow(S, DIM - 1), SD = ipow(S, DIM);
    return 2 * K * DIM * NL + 2 * K * DIM * NL / S + K * DIM * S + K * (S - 1) + 2 * K * DIM + 2 * K * SD +
           2 * K * 2 * VCU_MAX_DIM + 2 * K;
}
template <int S> __host__ __device__ constexpr int max_nl() {
    int best = 1;
    for (int d = 1; d <= VCU_MAX_DIM; ++d)
        if (ipow(S, d) <= 729) best = ipow(S, d - 1);
    return best;
}
template <int S> __host__ __device__ constexpr int scratch_words() {
    int best = 0;
    for (int d = 1; d <= VCU_MAX_DIM; ++d) {
        if (ipow(S, d) > 729) break;
        const int K = 1024 / (ipow(S, d) + (S - 1) * ipow(S, d - 1));
        const int Kc = K < 2 ? 2 : (K > 8 ? 8 : K), NL = ipow(S, d - 1), SD = ipow(S, d);
        const int w = 2 * Kc * d * NL + 2 * Kc * d * NL / S + Kc * d * S + Kc * (S - 1) + 2 * Kc * d + 2 * Kc * SD +
                      2 * Kc * 2 * VCU_MAX_DIM + 2 * Kc;
        if (w > best) best = w;
    }
    return best;
}

/* the integral of a region's polynomial over [A,B] (normalised) as the reference rounds it: folds
 * from the last dimension (region.h:141-150) with subrange() in the reference's double-promoted
 * arithmetic.  Over the whole region (A = 0, B = 1 in every dimension, the usual case for a single
 * bin) the lower end of each Horner evaluation is exactly 0 and the upper end's multiplications by
 * t = 1 are exact, so only the upper end is evaluated: in FP32 (ref_integral01, the reference's float
 * certified), in double only where FP32 cannot certify it (a sum on or next to a rounding boundary
 * that is not exact, zeros, extreme magnitudes) -- the FP64 pipe runs at 1/64 of the FP32 rate. */
static __device__ __noinline__ float integral01_double3(float c0, float c1, float c2) {
    const float c[3] = {c0, c1, c2};
    return __double2float_rn(horner_int_ref<3>(c, 1.0f));
}
static __device__ __noinline__ float integral01_double5(float c0, float c1, float c2, float c3, float c4) {
    const float c[5] = {c0, c1, c2, c3, c4};
    return __double2float_rn(horner_int_ref<5>(c, 1.0f));
}
template <int S> __device__ __forceinline__ float subrange01_ref(const float* p) {
    float c[S];
    Rule<S>::coefficients(p, c);
    if constexpr (S == 3 || S == 5) {
        float v;
        if (ref_integral01<S>(c, v)) return v;
        if constexpr (S == 3) return integral01_double3(c[0], c[1], c[2]);
        else return integral01_double5(c[0], c[1], c[2], c[3], c[4]);
    } else {
        return __double2float_rn(horner_int_ref<S>(c, 1.0f));
    }
}
template <int DIM, int S>
__device__ float region_integral_ref(const float* __restrict__ V, const float* A, const float* B, bool whole) {
    constexpr int SD = ipow(S, DIM);
    constexpr int inner = SD / S;
    float buf[inner];
    for (int i = 0; i < inner; ++i) {
        float line[S];
#pragma unroll
        for (int j = 0; j < S; ++j) line[j] = V[i + j * inner];
        buf[i] = whole ? subrange01_ref<S>(line) : subrange_ref<S>(A[DIM - 1], B[DIM - 1], line);
    }
    int n = inner;
#pragma unroll
    for (int d = DIM - 2; d >= 0; --d) {
        const int m = n / S;
        for (int i = 0; i < m; ++i) {
            float line[S];
#pragma unroll
            for (int j = 0; j < S; ++j) line[j] = buf[i + j * m];
            buf[i] = whole ? subrange01_ref<S>(line) : subrange_ref<S>(A[d], B[d], line);
        }
        n = m;
    }
    return buf[0];
}

__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* ---------------------------------------------------------------- Monte Carlo item */
template <class F, int DIM>
__device__ float mc_item(const F& f, const Item& it, double* lanes) {
    const uint32_t k0 = (uint32_t)it.seed, k1 = (uint32_t)(it.seed >> 32);
    float w[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) w[d] = vsub(it.rmax[d], it.rmin[d]);
    /* MC_LANES virtual lanes, whatever the block size: lane l sums samples l, l+MC_LANES, ... with
     * Kahan compensation, then the lanes are added by a fixed tree, so the result does not depend
     * on the launch shape the autotuner picks */
    for (int l = threadIdx.x; l < MC_LANES; l += blockDim.x) {
        float sum = 0.0f, comp = 0.0f;
        for (uint64_t s = l; s < it.budget; s += MC_LANES) {
            float x[F::DIM];
#pragma unroll
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
#pragma unroll
            for (int blk = 0; blk < (DIM + 3) / 4; ++blk) {
                const U4 r = philox4x32_10(U4{(uint32_t)s, (uint32_t)(s >> 32), (uint32_t)it.index, 0xBA7C0000u + blk}, k0, k1);
                const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int d = blk * 4 + k;
                    if (d < DIM) x[d] = vadd(vmul(u01(rr[k]), w[d]), it.rmin[d]);
                }
            }
            float v[1];
            f(x, v);
            const float y = vsub(v[0], comp);
            const float t = vadd(sum, y);
            comp = vsub(vsub(t, sum), y);
            sum = t;
        }
        lanes[l] = (double)sum - (double)comp;
    }
    __syncthreads();
    for (int half = MC_LANES / 2; half > 0; half >>= 1) {
        for (int i = threadIdx.x; i < half; i += blockDim.x) lanes[i] += lanes[i + half];
        __syncthreads();
    }
    double vol = 1.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) vol *= (double)w[d];
    return (float)(lanes[0] * (vol / (double)it.budget));
}

/* ---------------------------------------------------------------- nested item */
template <class F, int DIM, int SH, int SL>
__device__ float nested_item(const F& f, const Item& it, const Cfg& cfg, float* __restrict__ vals,
                             float* __restrict__ ranges, float* __restrict__ vols, HeapEntry* __restrict__ heap,
                             HeapEntry* hs, float* sm) {
    constexpr int S = SH;
    constexpr int SD = ipow(S, DIM);
    constexpr int NL = ipow(S, DIM - 1);
    constexpr int NNEW = (S - 1) * NL;
    const int tid = threadIdx.x, nth = blockDim.x;
    constexpr int K = spec_width<DIM, S>();
    constexpr int TASKS = NNEW + S * NL; /* one split's children: new nodes, then the parent's */
    static_assert(round_words<DIM, S>() <= scratch_words<S>(), "scratch too small for a round");
    float* LN = sm;                          /* 2K*DIM*NL line metrics          */
    float* LF = LN + 2 * K * DIM * NL;       /* first fold level                */
    float* CO = LF + 2 * K * DIM * NL / S;   /* K x DIM*S node coordinates      */
    float* CN = CO + K * DIM * S;            /* K x (S-1) new coordinates       */
    float* EC = CN + K * (S - 1);            /* 2K x DIM errors                 */
    float* VC = EC + 2 * K * DIM;            /* 2K x SD children node values    */
    float* CR = VC + 2 * K * SD;             /* 2K x SLOT_FLOATS children ranges */
    float* CV = CR + 2 * K * SLOT_FLOATS;    /* 2K children volumes             */
    float* V = vals + it.val_off;
    float* R = ranges + it.slot_off * SLOT_FLOATS;
    float* VOL = vols + it.slot_off;
    /* heap: the first cfg.hcap elements in shared memory, the others in the item's global slice */
    const HeapSplit h{hs, heap + it.heap_off, cfg.hcap};
    const int iters = (int)it.budget - 1;

    /* error estimates of the nreg regions whose node values are VC[r*SD ..] and volumes CV[r] into
     * EC[r*DIM + d] (region.h:379-418) */
    auto region_errors = [&](int nreg) {
        /* line metrics LN[(r*DIM + d)*NL + J]: the line of region r along dimension d whose other
         * coordinates are J's digits; its nodes are base + i*S^d */
        static_for<DIM>([&](auto dc) {
            constexpr int d = decltype(dc)::value;
            constexpr int PD = ipow(S, d);
            for (int t = tid; t < nreg * NL; t += nth) {
                const int r = t / NL;
                const int J = t - r * NL;
                const float* RV = VC + r * SD + (J % PD + (J / PD) * (PD * S));
                float line[S], low[SL];
#pragma unroll
                for (int i = 0; i < S; ++i) line[i] = RV[i * PD];
#pragma unroll
                for (int i = 0; i < SL; ++i) low[i] = line[i * (S - 1) / (SL - 1)];
                LN[(r * DIM + d) * NL + J] =
                    metric_value(cfg.relative, cfg.min_val_f, RefRule<S>::scalar(line), RefRule<SL>::scalar(low));
            }
        });
        __syncthreads();
        /* fold dimension 0 of the remaining dimensions with the high rule, one level at a time */
        float* src = LN;
        float* dst = LF;
        static_for<DIM - 1>([&](auto lc) {
            constexpr int n = NL / ipow(S, decltype(lc)::value), m = n / S;
            for (int t = tid; t < nreg * DIM * m; t += nth) {
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
        if (tid < nreg * DIM) EC[tid] = vmul(CV[tid / DIM], src[tid]);
        __syncthreads();
    };
    /* error_heuristic_default / error_heuristic_size (error-heuristic.h:10-47) of region r with ranges
     * rs (rmin at 0, rmax at VCU_MAX_DIM) */
    auto heuristic = [&](int r, const float* rs, float& err_out, int& dim_out) {
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
        float w = vsub(rs[VCU_MAX_DIM], rs[0]);
        float max_err;
        if ((double)w < cfg.min_size || isnan(w)) max_err = 0.0f;
        else max_err = __double2float_rn(__dadd_rn((double)e[0], __dmul_rn(cfg.size_weight, (double)fabsf(w))));
        int max_dim = 0;
#pragma unroll
        for (int d = 1; d < DIM; ++d) {
            w = vsub(rs[VCU_MAX_DIM + d], rs[d]);
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

    /* ---- root region in slot 0 (region.h:74-78); slot 1 is the first scratch child */
    if (tid == 0) {
        float vol = 1.0f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            R[d] = it.rmin[d];
            R[VCU_MAX_DIM + d] = it.rmax[d];
            vol = vmul(vol, vsub(it.rmax[d], it.rmin[d]));
        }
        VOL[0] = vol;
        CV[0] = vol;
    }
    for (int t = tid; t < DIM * S; t += nth) {
        const int d = t / S, j = t % S;
        CO[t] = node_coord(node_pos<S>(j), vsub(it.rmax[d], it.rmin[d]), it.rmin[d]);
    }
    __syncthreads();
    for (int t = tid; t < SD; t += nth) {
        float x[F::DIM];
#pragma unroll
        for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
        int rem = t;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            x[d] = CO[d * S + rem % S];
            rem /= S;
        }
        float v[1];
        f(x, v);
        VC[t] = v[0];
        V[t] = v[0];
    }
    __syncthreads();
    region_errors(1);
    __shared__ int s_cand[8], s_slot[16], s_nc, s_adv, s_scratch;
    if (tid == 0) {
        float e;
        int dm;
        heuristic(0, R, e, dm);
        h.set(0, HeapEntry{e, 0 | (dm << 24)});
        s_scratch = 1;
    }

    /* Rounds: split the heap's top and the K-1 regions that by their keys pop after it, all children
     * on chip; then commit in order -- split q only if, after splits 0..q-1 went into the heap, q's
     * region is exactly the top the sequential algorithm pops (same entry) -- and copy the committed
     * children to the pool.  Slots follow the sequential scheme (first child in the slot the previous
     * split freed, second in slot k+2), so the result is the sequential one, bit for bit. */
    int k = 0;
#pragma unroll 1
    while (k < iters) {
        __syncthreads();
        if (tid == 0) {
            const int n = k + 1; /* heap size */
            int nc = (K < iters - k) ? K : iters - k;
            /* the next pops by key: a small queue of heap positions whose parents were taken */
            int qpos[2 * 8 + 2];
            float qkey[2 * 8 + 2];
            int qn = 0;
            s_cand[0] = h.get(0).pay;
            for (int c = 1; c <= 2; ++c)
                if (c < n) {
                    qpos[qn] = c;
                    qkey[qn] = h.get(c).key;
                    ++qn;
                }
            for (int c = 1; c < nc; ++c) {
                if (qn == 0) {
                    nc = c;
                    break;
                }
                int b = 0;
                for (int i = 1; i < qn; ++i)
                    if (qkey[b] < qkey[i]) b = i;
                const int pos = qpos[b];
                s_cand[c] = h.get(pos).pay;
                qpos[b] = qpos[qn - 1];
                qkey[b] = qkey[qn - 1];
                --qn;
                for (int ch = 2 * pos + 1; ch <= 2 * pos + 2; ++ch)
                    if (ch < n) {
                        qpos[qn] = ch;
                        qkey[qn] = h.get(ch).key;
                        ++qn;
                    }
            }
            s_nc = nc;
        }
        __syncthreads();
        const int nc = s_nc;
        /* node coordinates of each candidate, and of its new nodes along its split dimension */
        for (int t = tid; t < nc * (DIM * S + (S - 1)); t += nth) {
            const int q = t / (DIM * S + (S - 1)), u = t - q * (DIM * S + (S - 1));
            const int P = s_cand[q] & 0xffffff, dd = s_cand[q] >> 24;
            const float* pr = R + (size_t)P * SLOT_FLOATS;
            if (u < DIM * S) {
                const int d = u / S, j = u % S;
                CO[q * DIM * S + u] = node_coord(node_pos<S>(j), vsub(pr[VCU_MAX_DIM + d], pr[d]), pr[d]);
            } else {
                const int c = u - DIM * S;
                CN[q * (S - 1) + c] = node_coord(mid_pos<S>(c), vsub(pr[VCU_MAX_DIM + dd], pr[dd]), pr[dd]);
            }
        }
        __syncthreads();
        /* region.h:345-359 / split.h:13-49: new nodes at the odd positions, parent nodes at the even,
         * built on chip.  One instance per split dimension, so every stride and divisor is a constant. */
        auto build_children = [&](auto ddc, int q, int u) {
            constexpr int DD = decltype(ddc)::value;
            constexpr int PD = ipow(S, DD);
            const int P = s_cand[q] & 0xffffff;
            const float* VP = V + (size_t)P * SD;
            float* W0 = VC + (2 * q) * SD;
            float* W1 = W0 + SD;
            const bool fresh = u < NNEW;
            const int w = fresh ? u : u - NNEW;
            const int c = w / NL, J = w - c * NL;
            const int base = J % PD + (J / PD) * (PD * S);
            float v;
            int i;
            if (fresh) {
                float x[F::DIM];
#pragma unroll
                for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
                static_for<DIM>([&](auto ec) {
                    constexpr int e = decltype(ec)::value;
                    if constexpr (e != DD) {
                        constexpr int pe = e < DD ? ipow(S, e) : ipow(S, e - 1);
                        x[e] = CO[q * DIM * S + e * S + (J / pe) % S];
                    }
                });
                x[DD] = CN[q * (S - 1) + c];
                float fv[1];
                f(x, fv);
                v = fv[0];
                i = 2 * c + 1;
            } else {
                v = VP[base + c * PD];
                i = 2 * c;
            }
            if (i <= S - 1) W0[base + i * PD] = v;
            if (i >= S - 1) W1[base + (i - (S - 1)) * PD] = v;
        };
        for (int t = tid; t < nc * TASKS; t += nth) {
            const int q = t / TASKS, u = t - q * TASKS;
            const int dd = s_cand[q] >> 24;
            static_for<DIM>([&](auto dc) {
                if (dd == decltype(dc)::value) build_children(dc, q, u);
            });
        }
        /* the children's ranges and volumes */
        for (int q = tid; q < nc; q += nth) {
            const int P = s_cand[q] & 0xffffff, dd = s_cand[q] >> 24;
            const float* pr = R + (size_t)P * SLOT_FLOATS;
            const float pmn = pr[dd], pmx = pr[VCU_MAX_DIM + dd];
            const float half = vmul(vsub(pmx, pmn), 0.5f); /* = (max - min) / 2.0, exactly */
            const float mid = vadd(pmn, vmul(half, 1.0f));
            float* r0 = CR + (2 * q) * SLOT_FLOATS;
            float* r1 = r0 + SLOT_FLOATS;
            float vol0 = 1.0f, vol1 = 1.0f;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const float mn = pr[d], mx = pr[VCU_MAX_DIM + d];
                const float mx0 = (d == dd) ? mid : mx;
                const float mn1 = (d == dd) ? mid : mn;
                r0[d] = mn;
                r0[VCU_MAX_DIM + d] = mx0;
                r1[d] = mn1;
                r1[VCU_MAX_DIM + d] = mx;
                vol0 = vmul(vol0, vsub(mx0, mn));
                vol1 = vmul(vol1, vsub(mx, mn1));
            }
            CV[2 * q] = vol0;
            CV[2 * q + 1] = vol1;
        }
        __syncthreads();
        region_errors(2 * nc);
        if (tid == 0) {
            int adv = 0, scratch = s_scratch;
            for (int q = 0; q < nc; ++q) {
                if (q > 0 && h.get(0).pay != s_cand[q]) break;
                const int C0 = scratch, C1 = k + q + 2;
                const float* r0 = CR + (2 * q) * SLOT_FLOATS;
                const float* r1 = r0 + SLOT_FLOATS;
                float* d0r = R + (size_t)C0 * SLOT_FLOATS;
                float* d1r = R + (size_t)C1 * SLOT_FLOATS;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    d0r[d] = r0[d];
                    d0r[VCU_MAX_DIM + d] = r0[VCU_MAX_DIM + d];
                    d1r[d] = r1[d];
                    d1r[VCU_MAX_DIM + d] = r1[VCU_MAX_DIM + d];
                }
                VOL[C0] = CV[2 * q];
                VOL[C1] = CV[2 * q + 1];
                float e0, e1;
                int dm0, dm1;
                heuristic(2 * q, r0, e0, dm0);
                heuristic(2 * q + 1, r1, e1, dm1);
                const int n = k + q + 1; /* heap size before this split */
                heap_pop_entries(h, n);
                h.set(n - 1, HeapEntry{e0, C0 | (dm0 << 24)});
                heap_push_entries(h, n);
                h.set(n, HeapEntry{e1, C1 | (dm1 << 24)});
                heap_push_entries(h, n + 1);
                s_slot[2 * q] = C0;
                s_slot[2 * q + 1] = C1;
                scratch = s_cand[q] & 0xffffff; /* the split region's slot holds the next first child */
                ++adv;
            }
            s_scratch = scratch;
            s_adv = adv;
        }
        __syncthreads();
        const int adv = s_adv;
        for (int t = tid; t < adv * 2 * SD; t += nth) {
            const int r = t / SD, i = t - r * SD;
            V[(size_t)s_slot[r] * SD + i] = VC[r * SD + i];
        }
        k += adv;
    }
    __syncthreads();
    /* ---- every region's integral over (range n region), in heap order; the single bin's range has
     * dimension 0 rebuilt as min + 1*(max-min) (integrate.h:108-110, regions-integrator-sequential.h) */
    const int nreg = iters + 1;
    for (int k = tid; k < nreg; k += nth) {
        const HeapEntry e = h.get(k);
        const int s = e.pay & 0xffffff;
        const float* rs = R + (size_t)s * SLOT_FLOATS;
        float A[DIM], B[DIM];
        bool empty = false, whole = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const float blo = it.rmin[d];
            const float bhi =
                (d == 0) ? vadd(it.rmin[0], vmul(1.0f, vdiv(vsub(it.rmax[0], it.rmin[0]), 1.0f))) : it.rmax[d];
            const float rmn = rs[d], rmx = rs[VCU_MAX_DIM + d];
            const float a = smax(blo, rmn);
            const float b = smax(a, smin(bhi, rmx));
            empty = empty || (a >= b);
            A[d] = (rmn >= rmx) ? rmn : vdiv(vsub(a, rmn), vsub(rmx, rmn));
            B[d] = (rmn >= rmx) ? rmn : vdiv(vsub(b, rmn), vsub(rmx, rmn));
            whole = whole && A[d] == 0.0f && B[d] == 1.0f;
        }
        /* the contribution replaces the key; a payload of -1 marks a region outside the range */
        if (empty) h.set(k, HeapEntry{0.0f, -1});
        else h.set(k, HeapEntry{vmul(VOL[s], region_integral_ref<DIM, S>(V + (size_t)s * SD, A, B, whole)), e.pay});
    }
    __syncthreads();
    float sol = 0.0f;
    if (tid == 0) {
        for (int k = 0; k < nreg; ++k) {
            const HeapEntry e = h.get(k);
            if (e.pay != -1) sol = vadd(sol, e.key);
        }
    }
    return sol; /* valid on thread 0 */
}

template <class F, int SH, int SL>
__global__ void __launch_bounds__(MAX_THREADS)
    k_batch(const Cfg cfg, const Item* __restrict__ items, const F* __restrict__ functors, uint32_t* __restrict__ queue,
            float* __restrict__ vals, float* __restrict__ ranges, float* __restrict__ vols, HeapEntry* __restrict__ heap,
            float* __restrict__ results, uint64_t* __restrict__ item_ns, uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr size_t fbytes = (sizeof(F) + 15) & ~size_t(15);
    F& f = *reinterpret_cast<F*>(smem_raw);
    /* heap top: hcap entries from smem_raw + fbytes + 8, so that element 1 is 16-byte aligned */
    HeapEntry* hs = reinterpret_cast<HeapEntry*>(smem_raw + fbytes + 8);
    float* sm = reinterpret_cast<float*>(smem_raw + fbytes + 8 + (size_t)(cfg.hcap + 1) * sizeof(HeapEntry));
    __shared__ double lanes[MC_LANES];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int q = s_item;
        if (q >= cfg.n_items) break;
        const uint64_t t0 = globaltimer();
        const Item it = items[q];
        static_assert(sizeof(F) % 4 == 0, "functor copied as words");
        for (int i = threadIdx.x; i < (int)(sizeof(F) / 4); i += blockDim.x)
            reinterpret_cast<uint32_t*>(smem_raw)[i] = reinterpret_cast<const uint32_t*>(functors + q)[i];
        __syncthreads();
        float r = 0.0f;
        auto run = [&](auto dimc) {
            constexpr int DIM = decltype(dimc)::value;
            if (it.method == VCU_BATCH_MONTE_CARLO) {
                r = mc_item<F, DIM>(f, it, lanes);
            } else if constexpr (ipow(SH, DIM) <= 729) {
                r = nested_item<F, DIM, SH, SL>(f, it, cfg, vals, ranges, vols, heap, hs, sm);
            }
        };
        if constexpr (F::DIM == VCU_MAX_DIM) {
            /* run-time arity (the half-space family) */
            switch (it.dim) {
            case 1: run(std::integral_constant<int, 1>{}); break;
            case 2: run(std::integral_constant<int, 2>{}); break;
            case 3: run(std::integral_constant<int, 3>{}); break;
            case 4: run(std::integral_constant<int, 4>{}); break;
            case 5: run(std::integral_constant<int, 5>{}); break;
            default: run(std::integral_constant<int, 6>{}); break;
            }
        } else {
            run(std::integral_constant<int, F::DIM>{});
        }
        if (threadIdx.x == 0) {
            results[it.index] = r;
            if (isnan(r)) atomicOr(status, VCU_FLAG_NAN);
            item_ns[it.index] = globaltimer() - t0;
        }
        __syncthreads();
    }
}

/* ---------------------------------------------------------------- host side */

/* The host lays out one batch: functors built per item, items sorted by estimated cost (largest
 * first), per-item offsets into the region pool.  Returns the pool sizes. */
struct BatchLayout {
    std::vector<Item> items;
    std::vector<unsigned char> functors;
    uint64_t n_vals = 0, n_slots = 0, n_heap = 1;
    uint64_t evaluations = 0, regions = 0;
};

template <class F, int SH, int SL>
int lay_out(vcu_ctx* ctx, int kind, const vcu_batch_item* in, uint64_t n, BatchLayout& L) {
    constexpr int S = SH;
    std::vector<std::pair<double, uint64_t>> order(n);
    std::vector<F> fns(n);
    for (uint64_t i = 0; i < n; ++i) {
        const vcu_batch_item& b = in[i];
        if (b.dim < 1 || b.dim > VCU_MAX_DIM) return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": bad dimension");
        if (b.method != VCU_BATCH_MONTE_CARLO && b.method != VCU_BATCH_NESTED)
            return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": unknown method");
        if (b.budget == 0) return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": zero budget");
        for (int d = 0; d < b.dim; ++d)
            if (!(b.range_min[d] <= b.range_max[d]))
                return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": empty range");
        if (b.method == VCU_BATCH_NESTED) {
            if (b.budget > MAX_NESTED_BUDGET)
                return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": nested budget above 2^24-2 regions");
            if (ipow(S, b.dim) > 729)
                return fail(ctx, VCU_UNSUPPORTED, "batch item " + std::to_string(i) + ": nested regions are limited to 729 nodes (S^dim)");
        }
        vcu_integrand fi{kind, b.n_params, b.params};
        bool same = false;
        const int rc = with_integrand(ctx, fi, b.dim, [&](const auto& f) -> int {
            if constexpr (std::is_same_v<std::decay_t<decltype(f)>, F>) {
                fns[i] = f;
                same = true;
            }
            return VCU_OK;
        });
        if (rc) return rc;
        if (!same) return fail(ctx, VCU_INVALID_ARG, "batch item " + std::to_string(i) + ": integrand kind differs");
        const double nodes = (double)ipow(S, b.dim - 1) * (S - 1);
        const double cost = b.method == VCU_BATCH_NESTED ? (double)b.budget * (64.0 + nodes * b.dim) : (double)b.budget * b.dim;
        order[i] = {cost, i};
    }
    std::stable_sort(order.begin(), order.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    L.items.resize(n);
    L.functors.resize(n * sizeof(F));
    L.n_vals = 0;
    L.n_slots = 0;
    L.n_heap = 1;
    for (uint64_t q = 0; q < n; ++q) {
        const uint64_t i = order[q].second;
        const vcu_batch_item& b = in[i];
        Item& it = L.items[q];
        std::memset(&it, 0, sizeof(it));
        for (int d = 0; d < VCU_MAX_DIM; ++d) {
            it.rmin[d] = d < b.dim ? b.range_min[d] : 0.0f;
            it.rmax[d] = d < b.dim ? b.range_max[d] : 0.0f;
        }
        it.budget = b.budget;
        it.seed = b.seed;
        it.dim = b.dim;
        it.method = b.method;
        it.index = (int32_t)i;
        if (b.method == VCU_BATCH_NESTED) {
            const uint64_t sd = (uint64_t)ipow(S, b.dim);
            const uint64_t slots = b.budget + 1;
            it.val_off = L.n_vals;
            it.slot_off = L.n_slots;
            it.heap_off = L.n_heap;
            L.n_vals += slots * sd;
            L.n_vals = (L.n_vals + 3) & ~uint64_t(3);
            L.n_slots += slots;
            L.n_heap += (b.budget + 1) & ~uint64_t(1); /* keeps every offset odd */
            L.evaluations += sd + (b.budget - 1) * (uint64_t)(S - 1) * (uint64_t)ipow(S, b.dim - 1);
            L.regions += b.budget;
        } else {
            L.evaluations += b.budget;
        }
        std::memcpy(L.functors.data() + q * sizeof(F), &fns[i], sizeof(F));
    }
    return VCU_OK;
}

}  // namespace batch

/* one rule pair: lay out, upload, tune the block size, capture the launch in a graph */
template <int SH, int SL>
int run_batch_pair(vcu_ctx* ctx, int kind, const vcu_nested& n, const vcu_batch_item* items, uint64_t count,
                   uint32_t& launches) {
    using namespace batch;
    vcu_integrand probe{kind, items[0].n_params, items[0].params};
    return with_integrand(ctx, probe, items[0].dim, [&](const auto& f0) -> int {
        using F = std::decay_t<decltype(f0)>;
        if constexpr (F::CH != 1) {
            return fail(ctx, VCU_UNSUPPORTED, "batched integrals take scalar integrands");
        } else {
            BatchLayout L;
            int rc = lay_out<F, SH, SL>(ctx, kind, items, count, L);
            if (rc) return rc;
            /* buffers: items | functors | results | item times | queue ; pool: vals | ranges | vols | heap */
            const size_t b_items = count * sizeof(Item), b_fn = count * sizeof(F);
            const size_t o_fn = (b_items + 255) & ~size_t(255);
            const size_t o_res = (o_fn + b_fn + 255) & ~size_t(255);
            const size_t o_ns = (o_res + count * 4 + 255) & ~size_t(255);
            const size_t o_q = (o_ns + count * 8 + 255) & ~size_t(255);
            rc = ensure(ctx, ctx->batch_in, o_q + 256);
            if (rc) return rc;
            const size_t o_rng = (L.n_vals * 4 + 255) & ~size_t(255);
            const size_t o_vol = (o_rng + L.n_slots * SLOT_FLOATS * 4 + 255) & ~size_t(255);
            const size_t o_heap = (o_vol + L.n_slots * 4 + 255) & ~size_t(255);
            rc = ensure(ctx, ctx->batch_pool, o_heap + L.n_heap * sizeof(HeapEntry) + 256);
            if (rc) return rc;
            char* in = static_cast<char*>(ctx->batch_in.ptr);
            char* pool = static_cast<char*>(ctx->batch_pool.ptr);
            VCU_CUDA(ctx, cudaMemcpyAsync(in, L.items.data(), b_items, cudaMemcpyHostToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(in + o_fn, L.functors.data(), b_fn, cudaMemcpyHostToDevice, ctx->stream));

            Cfg cfg{};
            cfg.n_items = (int32_t)count;
            cfg.heuristic = n.heuristic;
            cfg.relative = n.metric == VCU_METRIC_RELATIVE;
            float mv = (float)n.min_val;
            if ((double)mv < n.min_val) mv = nextafterf(mv, INFINITY);
            cfg.min_val_f = mv;
            cfg.size_weight = n.size_weight;
            cfg.min_size = n.min_size;

            auto kern = k_batch<F, SH, SL>;
            const size_t fixed = ((sizeof(F) + 15) & ~size_t(15)) + 8 + (size_t)scratch_words<SH>() * 4;
            auto smem_for = [&](int hcap) { return fixed + (size_t)(hcap + 1) * sizeof(HeapEntry); };
            /* dynamic shared memory: what the opt-in limit leaves beside the kernel's static arrays */
            cudaFuncAttributes fa;
            VCU_CUDA(ctx, cudaFuncGetAttributes(&fa, kern));
            const size_t room = ctx->smem_optin - fa.sharedSizeBytes;
            if (smem_for(1) > room) return fail(ctx, VCU_UNSUPPORTED, "integrand too large for the batch kernel");
            VCU_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room));
            const size_t smem = smem_for(1);
            vcu_batch_state& P = ctx->batch;
            P.valid = false;
            P.kind = kind;
            P.sh = SH;
            P.sl = SL;
            P.n = count;
            P.cfg = cfg;
            P.smem = smem;
            P.kernel = reinterpret_cast<void*>(kern);
            P.evaluations = L.evaluations;
            P.regions = L.regions;
            P.vals = pool;
            P.ranges = pool + o_rng;
            P.vols = pool + o_vol;
            P.heap = pool + o_heap;
            P.items = in;
            P.functors = in + o_fn;
            P.results = reinterpret_cast<float*>(in + o_res);
            P.item_ns = reinterpret_cast<uint64_t*>(in + o_ns);
            P.queue = reinterpret_cast<uint32_t*>(in + o_q);

            /* launch shapes: (threads per block, heap elements in shared memory) */
            struct Shape {
                int threads, hcap;
            };
            static constexpr Shape shapes[] = {{256, 2047}, {512, 4095}, {512, 16383}, {1024, 16383}};
            auto launch_with = [&](int si) -> int {
                int hcap = shapes[si].hcap;
                /* the kernel's static shared memory (Monte Carlo lanes, a few words) comes on top */
                while (hcap > 1 && smem_for(hcap) > room) hcap = (hcap - 1) / 2;
                const size_t sm = smem_for(hcap);
                int per_sm = 0;
                VCU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, shapes[si].threads, sm));
                if (per_sm < 1) return fail(ctx, VCU_UNSUPPORTED, "batch kernel does not fit on an SM");
                const uint64_t cap = (uint64_t)ctx->sm_count * per_sm;
                P.threads = shapes[si].threads;
                P.smem = sm;
                P.cfg.hcap = hcap;
                P.blocks = (unsigned)(count < cap ? count : cap);
                return batch_capture(ctx, launches);
            };
            /* shape: tuned once per (integrand, rules, batch size class, total work class) */
            if (const char* env = std::getenv("VCU_BATCH_THREADS")) {
                const int t = std::atoi(env);
                for (int si = 0; si < 4; ++si)
                    if (shapes[si].threads == t) return launch_with(si);
            }
            const uint64_t key = 0xBA7C000000000000ull ^ ((uint64_t)kind << 44) ^ ((uint64_t)SH << 40) ^ ((uint64_t)SL << 36) ^
                                 ((uint64_t)(63 - __builtin_clzll(count)) << 28) ^
                                 (uint64_t)(63 - __builtin_clzll(L.evaluations | 1));
            if (!ctx->tune) return launch_with(1);
            for (int i = 0; i < ctx->ntuned; ++i)
                if (ctx->tuned[i].key == key) return launch_with(ctx->tuned[i].value);
            float best_ms = 1e30f;
            int best = 1;
            for (int si = 0; si < 4; ++si) {
                VCU_CUDA(ctx, cudaEventRecord(ctx->ev_tune[0], ctx->stream));
                rc = launch_with(si);
                if (rc) return rc;
                VCU_CUDA(ctx, cudaEventRecord(ctx->ev_tune[1], ctx->stream));
                VCU_CUDA(ctx, cudaEventSynchronize(ctx->ev_tune[1]));
                float ms = 0.0f;
                VCU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_tune[0], ctx->ev_tune[1]));
                if (ms < best_ms) {
                    best_ms = ms;
                    best = si;
                }
            }
            if (ctx->ntuned < 32) ctx->tuned[ctx->ntuned++] = vcu_tuned{key, best};
            if (best != 3) return launch_with(best);
            return VCU_OK;
        }
    });
}

}  // namespace vcu
