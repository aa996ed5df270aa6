/*
 * oracle.h -- C interface of the CPU oracle (test infrastructure, NOT the product).
 *
 * liboracle.so is a plain-C++ restatement of viltrum's per-bin integration path, written to
 * reproduce the reference's results bit for bit (same float/double promotions, same libstdc++
 * std::mt19937 / uniform distributions / push_heap / pop_heap).  Only tests/, bench.py's
 * cpu_baseline leg and __graft_entry__.smoke() use it, and only as the checker.
 *
 * The same symbols with an "ref_" prefix instead of "orc_" are exported by oracle/_ref/
 * libvref.so, built (where the reference sources are available) from ref_driver.cc, which
 * calls the unmodified reference headers; the goldens under tests/golden/ come from it.
 *
 * Conventions shared by every entry point:
 *   kind, params, n_params   integrand (vcu_integrands.h VCU_F_* tag + flat parameters)
 *   dim, rmin[dim], rmax[dim] integration range (viltrum::Range<float,dim>)
 *   dimbins, res[dimbins]    bin resolution; bins are written dim-0-fastest, channels
 *                            interleaved (out[bin*channels + c])
 *   return 0 on success, non-zero on a bad argument.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rule ids (Nested<H,L> pairs of src/nested/nested.h:7-34) */
enum { ORC_RULE_TRAPEZOIDAL = 2, ORC_RULE_SIMPSON = 3, ORC_RULE_BOOLE = 5 };
/* error heuristics (src/nested/error-heuristic.h) and metrics (src/nested/error-metric.h) */
enum { ORC_HEUR_DEFAULT = 0, ORC_HEUR_SIZE = 1 };
enum { ORC_METRIC_ABSOLUTE = 0, ORC_METRIC_RELATIVE = 1 };
/* control-variate weight strategies (src/control-variates/weight-strategy.h) */
enum { ORC_CV_OPTIMIZE = 0, ORC_CV_FIXED = 1 };
/* residual region choice (src/control-variates/region-russian-roulette.h): rr_uniform_region,
 * rr_integral_region, rr_error_region */
enum { ORC_RR_UNIFORM = 0, ORC_RR_INTEGRAL = 1, ORC_RR_ERROR = 2, ORC_RR_PDF = 3 };
/* residual point sampling in bin n region (src/control-variates/region-sampling.h):
 * region_sampling_uniform, region_sampling_importance, region_sampling_russian_roulette,
 * region_sampling_mis; all but uniform need a Simpson high rule */
enum { ORC_RS_UNIFORM = 0, ORC_RS_IMPORTANCE = 1, ORC_RS_RUSSIAN_ROULETTE = 2, ORC_RS_MIS = 3 };

/* residual strategy of the control-variate integrator */
typedef struct orc_cv {
    int32_t weight;     /* ORC_CV_OPTIMIZE / ORC_CV_FIXED                                */
    int32_t rr;         /* ORC_RR_*                                                      */
    double alpha;       /* cv_fixed_weight(alpha)                                        */
    float rr_factor;    /* rr_pdf_region(factor_prob): floor of the weights (0.01f)      */
    int32_t sampling;   /* ORC_RS_*                                                      */
    double mis_power;   /* region_sampling_mis(power, cutoff)                            */
    double mis_cutoff;
} orc_cv;

/* floats per residual sample in replay_out: the chosen list index and the point, then for
 * ORC_RS_RUSSIAN_ROULETTE / ORC_RS_MIS a 1/0 flag (importance branch taken) and for ORC_RS_MIS
 * the importance point its weight was computed at */
static inline int orc_replay_width(int dim, int sampling) {
    return 1 + dim + (sampling == ORC_RS_RUSSIAN_ROULETTE ? 1 : sampling == ORC_RS_MIS ? 1 + dim : 0);
}
/* Monte Carlo flavours */
enum {
    ORC_MC_PER_BIN_PARALLEL = 0, /* integrator_per_bin_parallel(monte_carlo(spp, seed))    */
    ORC_MC_PER_BIN_PARALLEL_SINGLE = 1 /* monte_carlo_per_bin_parallel(spp, seed), += into bins */
};

typedef struct orc_nested {
    int32_t rule_hi, rule_lo;
    int32_t heuristic, metric;
    double size_weight; /* error_heuristic_size: 1e-5 by default   */
    double min_size;    /* error_heuristic_size: 1e-37 by default  */
    double min_val;     /* error_metric_relative: 1e-37 by default */
} orc_nested;

int orc_channels(int32_t kind);
/* f at npts points (row-major npts x dim) -> out[npts*channels] */
int orc_eval(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* x,
             int64_t npts, float* out);

/* Per-bin Monte Carlo.  points_out (nullable) receives every sample point in the order the
 * reference draws them: bin-major (dim-0-fastest bins), then sample, then coordinate.      */
int orc_per_bin_monte_carlo(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                            const float* rmin, const float* rmax, int32_t dimbins,
                            const uint64_t* res, uint64_t spp, uint64_t seed, int32_t flavour,
                            float* out, float* points_out);

/* integrator_per_bin_parallel(integrator_adaptive_iterations(nested(H,L), heuristic, iters)).
 * trace (nullable) receives, per bin, iterations x (split dimension, popped error bits).   */
int orc_per_bin_adaptive_nested(int32_t kind, const float* params, int32_t n_params,
                                int32_t dim, const float* rmin, const float* rmax,
                                int32_t dimbins, const uint64_t* res, const orc_nested* nested,
                                uint64_t iterations, float* out, int32_t* trace);

/* integrator_region_based(regions_generator_adaptive_heap(nested, heuristic, iters),
 *   regions_integrator_parallel_variance_reduction(rr, weight, sampling, std::mt19937(seed), spp))
 *   -- crespo2021 when nested = (simpson, trapezoidal, size, relative), rr = ORC_RR_UNIFORM and
 *   sampling = ORC_RS_UNIFORM.  rr: rr_uniform_region(), rr_integral_region(), rr_error_region(),
 *   rr_pdf_region(rr_factor); sampling: region_sampling_uniform(), region_sampling_importance(),
 *   region_sampling_russian_roulette(), region_sampling_mis(power, cutoff); NormDefault throughout.
 * approx_out (nullable): per-bin control-variate integral (the "approximation").
 * regions_out (nullable): (iters+1) x (2*dim) float ranges in heap order.
 * replay_out (nullable): per bin, spp x orc_replay_width(dim, sampling) floats.               */
int orc_control_variates(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                         const float* rmin, const float* rmax, int32_t dimbins,
                         const uint64_t* res, const orc_nested* nested, uint64_t iterations,
                         uint64_t spp, uint64_t seed, const orc_cv* cv, float* out, float* approx_out,
                         float* regions_out, float* replay_out);

/* Same per-bin adaptive nested arithmetic over a contiguous slice of bins [bin_begin, bin_end),
 * on nthreads host threads (bins are independent: integrator-per-bin-parallel.h:28-34).  Used to
 * time the CPU path on all host cores and to check full-size images; trace (optional, indexed by
 * the absolute bin like orc_per_bin_adaptive_nested's) receives the split traces of the slice. */
int orc_per_bin_adaptive_nested_threads(int32_t kind, const float* params, int32_t n_params,
                                        int32_t dim, const float* rmin, const float* rmax,
                                        int32_t dimbins, const uint64_t* res,
                                        const orc_nested* nested, uint64_t iterations,
                                        uint64_t bin_begin, uint64_t bin_end, int32_t nthreads,
                                        float* out, int32_t* trace);

/* integrate(integrator_adaptive_iterations(nested(H,L), heuristic, iters), bins, f, range) with the
 * integrator used directly (not per bin): one max-error heap over the whole range, then every region,
 * in heap order, added into the bins it overlaps (src/newton-cotes/regions-integrator-sequential.h:
 * 37-58: bins(pos) += double(factor) * integral_subrange).  out holds the initial bins (it is
 * accumulated into, as the reference does).                                                 */
int orc_adaptive_global(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* rmin,
                        const float* rmax, int32_t dimbins, const uint64_t* res, const orc_nested* nested,
                        uint64_t iterations, float* out);

/* integrate(integrator_adaptive_tolerance(nested(H,L), heuristic, tolerance), bins, f, range)
 * (src/nested/integrator-adaptive-tolerance.h:9-56): depth-first, regions whose error is below the
 * tolerance are added into the bins (accumulating into out), others split.  Returns the number of
 * leaf regions, -1 if more than max_regions regions would be built, -2 on a bad argument.      */
int64_t orc_adaptive_tolerance(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                               const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                               const orc_nested* nested, float tolerance, uint64_t max_regions, float* out);

/* One single-value viltrum::integrate(I, f, range) (src/integrate.h:105-113):
 *   method 0: I = monte_carlo(budget, seed)  (std::mt19937(seed), float accumulation,
 *             src/monte-carlo/monte-carlo.h:39-63, 89-95)
 *   method 1: I = integrator_adaptive_iterations(nested(H,L), heuristic, budget - 1)
 * -> *out.  This is the shape of each item of a batch of independent integrals.           */
int orc_integrate_single(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                         const float* rmin, const float* rmax, int32_t method, uint64_t budget,
                         uint64_t seed, const orc_nested* nested, float* out);


/* Control-variate weight accumulator (cv_optimize_weight, src/control-variates/weight-strategy.h:40-110)
 * fed the n pairs (f[i], g[i]) in order, f the function sample and g the approximation's ->
 * out[0] = variance of g, out[1] = covariance of (f, g) (both online, shifted by the first pair,
 * divided by n-1), out[2] = alpha, out[3] = integral(approximation). */
int orc_cv_optimize_moments(const float* f, const float* g, uint64_t n, float approximation, double* out);

/* A one-dimensional Simpson region over [0,1] whose three nodes hold nodes[3]
 * (src/newton-cotes/region.h, rules.h:102-248):
 *   pdf_1d    -> *out = pdf_subrange(t, [t0,t1])  (region.h:324-342)
 *   sample_1d -> *out = sample_subrange(s, [t0,t1]) for a uniform s in [0,1)  (region.h:243-268) */
int orc_simpson_pdf_1d(const float* nodes, float t, float t0, float t1, float* out);
int orc_simpson_sample_1d(const float* nodes, float s, float t0, float t1, float* out);

#ifdef __cplusplus
}
#endif
