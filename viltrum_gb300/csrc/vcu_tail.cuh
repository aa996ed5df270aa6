/*
 * vcu_tail.cuh -- integrand wrappers of viltrum's combinators, shared by the control-variate and
 * the per-bin Fubini kernels: the Monte Carlo tail of integrator_fubini / regions_generator_fubini
 * (TailMC) and the coordinate permutation of integrator_reorder (Permuted).
 */
#pragma once
#include "vcu_internal.cuh"

namespace vcu {
namespace cv_detail {

/* ---------------------------------------------------------------- Fubini tail
 * regions_generator_fubini<N>(generator, monte_carlo(mc_samples, seed)) and the residual's
 * function_split_and_integrate_at<N>(f, monte_carlo_per_bin(rng, 1), range_rest)
 * (src/combination/regions-generator-fubini.h:7-28, fubini.h:51-63,
 * regions-integrator-parallel-variance-reduction.h:68): the regions span the first N dimensions and
 * every evaluation at x integrates the remaining ones by Monte Carlo, value = sum_k f(x, u_k) *
 * (volume(rest) / K) accumulated in float as viltrum's MonteCarlo adds into its one bin
 * (monte-carlo.h:41-63).  The reference draws u_k from one sequential std::mt19937 stream in the
 * order the nodes are visited; here u_k comes from Philox keyed by the seed with the counter (k, the
 * bits of x), so an evaluation is a deterministic function of its point and of K. */
template <class F, int N> struct TailMC {
    static constexpr int DIM = N, CH = F::CH;
    F f;
    int32_t full_dim; /* dimensions of f (runtime for the half-space family) */
    uint32_t k;       /* Monte Carlo samples per evaluation */
    uint32_t k0, k1, tag;
    float tmin[VCU_MAX_DIM], tlen[VCU_MAX_DIM];
    double vol;    /* volume(rest), its float product widened */
    double factor; /* vol / k */
    __device__ void operator()(const float* x, float* out) const {
        float acc[CH];
        for (int c = 0; c < CH; ++c) acc[c] = 0.0f;
        if constexpr (is_unbounded<F>::value) {
            /* an integrand of unbounded dimension: the rest is its own stream, one per sample
             * (the range beyond the first coordinates is [0,1) per dimension, volume 1) */
            for (uint32_t s = 0; s < k; ++s) {
                const float v = f.sample(x[0], x[1], tag ^ s);
                acc[0] = __double2float_rn(__dadd_rn((double)acc[0], __dmul_rn((double)v, factor)));
            }
            out[0] = acc[0];
            return;
        }
        float full[F::DIM];
        for (int d = 0; d < F::DIM; ++d) full[d] = 0.0f;
        for (int d = 0; d < N; ++d) full[d] = x[d];
        const uint32_t b0 = __float_as_uint(x[0]), b1 = N > 1 ? __float_as_uint(x[N > 1 ? 1 : 0]) : 0u;
        const uint32_t b2 = N > 2 ? __float_as_uint(x[N > 2 ? 2 : 0]) : 0u;
        for (uint32_t s = 0; s < k; ++s) {
            const U4 r = philox4x32_10(U4{s, b0, b1 ^ (b2 * 0x9E3779B9u), tag}, k0, k1);
            const uint32_t q[4] = {r.x, r.y, r.z, r.w};
            for (int d = N; d < full_dim; ++d) full[d] = vadd(vmul(u01(q[(d - N) & 3]), tlen[d]), tmin[d]);
            float v[CH];
            f(full, v);
            for (int c = 0; c < CH; ++c) acc[c] = __double2float_rn(__dadd_rn((double)acc[c], __dmul_rn((double)v[c], factor)));
        }
        for (int c = 0; c < CH; ++c) out[c] = acc[c];
    }
};

}  // namespace cv_detail

/* ---------------------------------------------------------------- reorder
 * IntegratorReorder (src/combination/reorder.h:15-58): the integrator integrates
 * f_reordered(x) = f(reorder(x)) over reorder(range), where reorder(v) puts v[from] at `to` for each
 * (to, from) pair and the other entries of v, in order, into the free places (reorder.h:19-45).  For
 * a vector of the integrand's dimension that is a fixed index map, computed on the host
 * (reorder_map) as src[to] = the index of v it takes, or -1 for a place left at the default. */
constexpr int VCU_REORDER_MAX_PAIRS = VCU_MAX_DIM;

/* src[0..n) of reorder() for vectors of n entries; false when the pairs would make the vector
 * longer than n (a `to` beyond the dimension) */
inline bool reorder_map(int n, const int32_t* to_from, int npairs, int* src) {
    bool tos[2 * VCU_MAX_DIM + 2] = {}, froms[VCU_MAX_DIM] = {};
    int ntos_size = n;
    for (int k = 0; k < npairs; ++k) {
        const int to = to_from[2 * k], from = to_from[2 * k + 1];
        if (to < 0 || from < 0 || to > 2 * VCU_MAX_DIM) return false;
        if (from < n) {
            if (to >= ntos_size) ntos_size = to + 1;
            froms[from] = true;
            tos[to] = true;
        }
    }
    int ntos = 0, nfroms = 0;
    for (int i = 0; i < ntos_size; ++i) ntos += tos[i];
    for (int i = 0; i < n; ++i) nfroms += froms[i];
    const int size = ntos_size > ntos + n - nfroms ? ntos_size : ntos + n - nfroms;
    if (size != n) return false;
    for (int i = 0; i < n; ++i) src[i] = -1;
    for (int k = 0; k < npairs; ++k) {
        const int to = to_from[2 * k], from = to_from[2 * k + 1];
        if (from < n && to < size) src[to] = from;
    }
    int to = 0;
    for (int from = 0; from < n; ++from) {
        if (!froms[from]) {
            while (to < size && tos[to]) ++to;
            if (to < size) src[to++] = from;
        }
    }
    return true;
}

/* f evaluated at the permuted point y[i] = x[src[i]] (0 where src[i] < 0) */
template <class F> struct Permuted {
    static constexpr int DIM = F::DIM, CH = F::CH;
    F f;
    int32_t n;                /* the problem's dimension (runtime for the half-space family) */
    int8_t src[VCU_MAX_DIM];
    __device__ void operator()(const float* x, float* out) const {
        float y[F::DIM];
        for (int i = 0; i < F::DIM; ++i) y[i] = 0.0f;
        for (int i = 0; i < n; ++i) y[i] = src[i] >= 0 ? x[src[i]] : 0.0f;
        f(y, out);
    }
};

}  // namespace vcu
