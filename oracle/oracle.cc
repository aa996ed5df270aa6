/*
 * oracle.cc -- CPU restatement of viltrum's per-bin integration path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker the CUDA library is compared against (and the
 * timed CPU baseline).  It is never linked into, loaded by or called from the product.
 *
 * It restates the reference's algorithms with the reference's arithmetic, so that its results
 * are bit-identical to the reference headers (pinned by tests/test_oracle_golden.py against
 * fixtures produced by oracle/_ref, which runs the unmodified reference):
 *   - rules: expressions of src/newton-cotes/rules.h:9-319 (float coefficients, double literal
 *     promotions in operator() and subrange()), Nested<H,L> of src/nested/nested.h:7-34;
 *   - regions: fill at i/(S-1) in double mapped to Float (src/newton-cotes/region.h:39-47,
 *     src/multiarray/fill.h:45-72), split from the parent's mapping (region.h:345-359,
 *     src/multiarray/split.h:13-49), error(dim, metric) and max_error_dimension
 *     (region.h:387-418), integral_subrange folding from the last dimension (region.h:141-169),
 *     approximation_at folding from the first (region.h:86-112);
 *   - heuristics and metrics: src/nested/error-heuristic.h:10-47, src/nested/error-metric.h;
 *   - adaptive heap: std::push_heap / std::pop_heap exactly as
 *     src/nested/regions-generator-adaptive-heap.h:18-45;
 *   - per-bin wrappers: src/integrator-per-bin-parallel.h:17-35 (including the copy-reseed
 *     chain of src/monte-carlo/monte-carlo.h:32-33), monte-carlo.h:39-63,
 *     src/monte-carlo/monte-carlo-per-bin-parallel.h:40-71,
 *     src/newton-cotes/regions-integrator-sequential.h:37-58, pixels_in_region region.h:454-463;
 *   - control variates: src/control-variates/regions-integrator-parallel-variance-reduction.h:32-109,
 *     weight-strategy.h:7-110, region-russian-roulette.h:9-108, region-sampling.h:9-20.
 * Random numbers come from libstdc++ (std::mt19937, uniform_real_distribution<float>,
 * uniform_int_distribution<size_t>, discrete_distribution<size_t>) exactly as the reference
 * draws them.
 */
#include "oracle_impl.h"

using namespace orc;

extern "C" int orc_channels(int32_t kind) {
    return kind == vcu::VCU_F_MOVING_SCENE3 ? 3 : 1;
}

extern "C" int orc_eval(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* x, int64_t npts,
                        float* out) {
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        using T = decltype(t);
        constexpr int DIM = decltype(D)::value;
        for (int64_t i = 0; i < npts; ++i) {
            std::array<float, DIM> xi;
            for (int d = 0; d < DIM; ++d) xi[d] = x[i * DIM + d];
            float o[3];
            f(xi.data(), o);
            for (int c = 0; c < VT<T>::CH; ++c) out[i * VT<T>::CH + c] = o[c];
        }
        return 0;
    });
}

static bool valid_problem(int32_t dim, int32_t dimbins, const uint64_t* res) {
    if (dim < 1 || dim > 6 || dimbins < 1 || dimbins > dim || dimbins > 4) return false;
    for (int i = 0; i < dimbins; ++i)
        if (res[i] == 0) return false;
    return true;
}

extern "C" int orc_per_bin_monte_carlo(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                       const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                       uint64_t spp, uint64_t seed, int32_t flavour, float* out, float* points_out) {
    if (!valid_problem(dim, dimbins, res) || spp == 0) return 1;
    Problem p{dim, dimbins, rmin, rmax, res};
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        per_bin_mc<decltype(D)::value, decltype(t)>(f, p, spp, seed, flavour, out, points_out);
        return 0;
    });
}

template <class Body> static int with_metric(const orc_nested& nc, Body&& body) {
    if (nc.metric == ORC_METRIC_RELATIVE) return body(MetricRel{nc.min_val});
    return body(MetricAbs{});
}

extern "C" int orc_per_bin_adaptive_nested(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                           const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                           const orc_nested* nested, uint64_t iterations, float* out, int32_t* trace) {
    if (!valid_problem(dim, dimbins, res) || !nested) return 1;
    Problem p{dim, dimbins, rmin, rmax, res};
    const uint64_t nb = p.nbins();
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                per_bin_nested_range<decltype(h), decltype(l), decltype(D)::value, decltype(t)>(
                    f, p, *nested, m, iterations, 0, nb, out, trace);
                return 0;
            });
        });
    });
}

extern "C" int orc_per_bin_adaptive_nested_threads(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                                   const float* rmin, const float* rmax, int32_t dimbins,
                                                   const uint64_t* res, const orc_nested* nested, uint64_t iterations,
                                                   uint64_t bin_begin, uint64_t bin_end, int32_t nthreads, float* out,
                                                   int32_t* trace) {
    if (!valid_problem(dim, dimbins, res) || !nested || bin_end < bin_begin || nthreads < 1) return 1;
    Problem p{dim, dimbins, rmin, rmax, res};
    if (bin_end > p.nbins()) return 1;
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                std::vector<std::thread> pool;
                const uint64_t n = bin_end - bin_begin;
                for (int k = 0; k < nthreads; ++k) {
                    const uint64_t a = bin_begin + n * k / nthreads, b = bin_begin + n * (k + 1) / nthreads;
                    pool.emplace_back([&, a, b] {
                        per_bin_nested_range<decltype(h), decltype(l), decltype(D)::value, decltype(t)>(
                            f, p, *nested, m, iterations, a, b, out, trace);
                    });
                }
                for (auto& th : pool) th.join();
                return 0;
            });
        });
    });
}

extern "C" int orc_control_variates(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                    const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                    const orc_nested* nested, uint64_t iterations, uint64_t spp, uint64_t seed,
                                    const orc_cv* cv, float* out, float* approx_out, float* regions_out,
                                    float* replay_out) {
    if (!valid_problem(dim, dimbins, res) || !nested || !cv) return 1;
    if (cv->rr < ORC_RR_UNIFORM || cv->rr > ORC_RR_PDF) return 1;
    if (cv->sampling < ORC_RS_UNIFORM || cv->sampling > ORC_RS_MIS) return 1;
    /* the pdf machinery exists for Simpson only (src/newton-cotes/rules.h:102-248) */
    if ((cv->rr == ORC_RR_PDF || cv->sampling != ORC_RS_UNIFORM) && nested->rule_hi != ORC_RULE_SIMPSON) return 2;
    Problem p{dim, dimbins, rmin, rmax, res};
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                control_variates<decltype(h), decltype(l), decltype(D)::value, decltype(t)>(
                    f, p, *nested, m, iterations, spp, seed, *cv, out, approx_out, regions_out, replay_out);
                return 0;
            });
        });
    });
}

extern "C" int orc_integrate_single(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* rmin,
                                    const float* rmax, int32_t method, uint64_t budget, uint64_t seed,
                                    const orc_nested* nested, float* out) {
    if (dim < 1 || dim > 6 || budget == 0 || !out || (method != 0 && method != 1)) return 1;
    if (method == 1 && !nested) return 1;
    if (orc_channels(kind) != 1) return 2;
    Problem p{dim, 1, rmin, rmax, nullptr};
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        (void)t;
        constexpr int DIM = decltype(D)::value;
        const auto range = make_range<DIM>(p);
        if (method == 0) {
            *out = single_mc<DIM>(f, range, budget, seed);
            return 0;
        }
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                *out = single_nested<decltype(h), decltype(l), DIM>(f, range, *nested, m, budget - 1);
                return 0;
            });
        });
    });
}

extern "C" int orc_adaptive_global(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* rmin,
                                   const float* rmax, int32_t dimbins, const uint64_t* res, const orc_nested* nested,
                                   uint64_t iterations, float* out) {
    if (!valid_problem(dim, dimbins, res) || !nested || !out) return 1;
    Problem p{dim, dimbins, rmin, rmax, res};
    return with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                adaptive_global<decltype(h), decltype(l), decltype(D)::value, decltype(t)>(f, p, *nested, m, iterations,
                                                                                              out);
                return 0;
            });
        });
    });
}

extern "C" int64_t orc_adaptive_tolerance(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                          const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                          const orc_nested* nested, float tolerance, uint64_t max_regions,
                                          float* out) {
    if (!valid_problem(dim, dimbins, res) || !nested || !out) return -2;
    Problem p{dim, dimbins, rmin, rmax, res};
    int64_t leaves = -2;
    const int rc = with_integrand(kind, params, n_params, dim, [&](const auto& f, auto D, auto t) -> int {
        return with_rules(*nested, [&](auto h, auto l) -> int {
            return with_metric(*nested, [&](auto m) -> int {
                leaves = adaptive_tolerance<decltype(h), decltype(l), decltype(D)::value, decltype(t)>(
                    f, p, *nested, m, tolerance, max_regions, out);
                return 0;
            });
        });
    });
    return rc ? -2 : leaves;
}

/* ------------------------------------------------------------------ accumulator and 1-D pdf probes */
extern "C" int orc_cv_optimize_moments(const float* f, const float* g, uint64_t n, float approximation,
                                       double* out) {
    if ((n && (!f || !g)) || !out) return 1;
    CvOptimize<float> acc(0.0f);
    for (uint64_t i = 0; i < n; ++i) acc.push(f[i], g[i]);
    out[0] = acc.variance();
    out[1] = acc.covariance();
    out[2] = acc.alpha();
    out[3] = acc.integral(approximation);
    return 0;
}

/* a 1-D region over [0,1] has volume 1 and maps positions unchanged, so its pdf and sampler are
 * the Simpson line's own */
extern "C" int orc_simpson_pdf_1d(const float* nodes, float t, float t0, float t1, float* out) {
    if (!nodes || !out) return 1;
    const auto ps = SimpsonPdf::points(nodes);
    *out = SimpsonPdf::at(t, ps) / SimpsonPdf::integral(t0, t1, ps);
    return 0;
}

extern "C" int orc_simpson_sample_1d(const float* nodes, float s, float t0, float t1, float* out) {
    if (!nodes || !out) return 1;
    *out = SimpsonPdf::sample(s, t0, t1, nodes);
    return 0;
}
