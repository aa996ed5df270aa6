/*
 * viltrum_cuda.hpp -- drop-in CUDA integrators for viltrum's integrate() (header-only host C++).
 *
 * Each type below satisfies viltrum's Integrator concept (src/integrate.h:72-79):
 *
 *     template<class Bins, size_t DIMBINS, class F, class R, class Logger>
 *     void integrate(Bins& bins, const std::array<size_t,DIMBINS>& resolution, const F& f,
 *                    const R& range, Logger& logger) const;
 *
 * so it can be passed wherever a CPU per-bin integrator was:
 *
 *     #include "viltrum.h"
 *     #include "viltrum_cuda.hpp"
 *     std::vector<std::vector<float>> image(512, std::vector<float>(512));
 *     auto scene = viltrum::cuda::builtin_integrand::scene2(params);
 *     viltrum::integrate(viltrum::cuda::per_bin_adaptive_nested(viltrum::cuda::boole_simpson(), 15),
 *                        image, scene, viltrum::range_primary<2>());
 *
 * The integrand must be a viltrum::cuda::builtin_integrand (a built-in functor of the CUDA
 * library, selected by tag: functor code cannot cross the C ABI).  It is also callable on the host
 * with std::array<float,DIM> (the same functor, bit-identical to the device), which is what
 * viltrum's integrate() checks its result type against.
 *
 * Results are written back through the caller's bins(pos) accessor in viltrum's
 * multidimensional_range order (dim 0 fastest) with the semantics of the integrator replaced:
 * per_bin_monte_carlo and per_bin_adaptive_nested ASSIGN, like integrator_per_bin_parallel
 * (src/integrator-per-bin-parallel.h:33); per_bin_monte_carlo_accumulate ADDS, like
 * monte_carlo_per_bin_parallel (src/monte-carlo/monte-carlo-per-bin-parallel.h:70).
 * Failures throw viltrum::cuda::error with the library's message; there is no CPU fallback.
 * The context (one CUDA stream and the library's device buffers) is per host thread.
 */
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "vcu_integrands.h"
#include "viltrum_cuda.h"

namespace viltrum {
namespace cuda {

#ifndef VILTRUM_CUDA_ERROR_DEFINED
#define VILTRUM_CUDA_ERROR_DEFINED
class error : public std::runtime_error {
public:
    int code;
    error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
#endif

/* RAII owner of a vcu_ctx */
class context {
    vcu_ctx* ctx_ = nullptr;

public:
    explicit context(int device = 0, void* stream = nullptr) {
        vcu_opts o{device, 0, stream};
        const int rc = vcu_create(&ctx_, &o);
        if (rc != VCU_OK) throw error(rc, "vcu_create failed (status " + std::to_string(rc) + ")");
    }
    context(const context&) = delete;
    context& operator=(const context&) = delete;
    ~context() { vcu_destroy(ctx_); }
    vcu_ctx* get() const { return ctx_; }
    void check(int rc) const {
        if (rc == VCU_OK) return;
        char buf[512];
        vcu_last_error(ctx_, buf, sizeof(buf));
        throw error(rc, buf);
    }
};

inline context& thread_context() {
    thread_local context ctx(0);
    return ctx;
}

/* A built-in integrand: tag + flat parameters (include/vcu_integrands.h). */
class builtin_integrand {
public:
    int32_t kind = 0;
    std::vector<float> params;

    builtin_integrand() = default;
    builtin_integrand(int32_t k, std::vector<float> p) : kind(k), params(std::move(p)) {}
    static builtin_integrand poly2() { return {vcu::VCU_F_POLY2, {}}; }
    static builtin_integrand sin1() { return {vcu::VCU_F_SIN1, {}}; }
    static builtin_integrand sphere3() { return {vcu::VCU_F_SPHERE3, {}}; }
    static builtin_integrand wave2() { return {vcu::VCU_F_WAVE2, {}}; }
    static builtin_integrand scene2(std::vector<float> p) { return {vcu::VCU_F_SCENE2, std::move(p)}; }
    static builtin_integrand moving_scene3(std::vector<float> p) { return {vcu::VCU_F_MOVING_SCENE3, std::move(p)}; }
    static builtin_integrand halfspace(std::vector<float> p) { return {vcu::VCU_F_HALFSPACE, std::move(p)}; }
    /* the random walk over scene2: unbounded dimension (integrate it over the first two coordinates,
     * e.g. viltrum::range_infinite(0, 0, 1, 1); it draws the rest itself) */
    static builtin_integrand walk2(std::vector<float> p) { return {vcu::VCU_F_WALK2, std::move(p)}; }
    static builtin_integrand occluded_scene5(std::vector<float> p) {
        return {vcu::VCU_F_OCCLUDED_SCENE5, std::move(p)};
    }
    int channels() const { return vcu_channels(kind); }

    /* host evaluation of the same functor (first channel); only std::array arguments, so
     * viltrum's detail::adapt passes this object through unchanged (src/integrate.h:11-16) */
    template <std::size_t DIM> float operator()(const std::array<float, DIM>& x) const {
        float out[3] = {0, 0, 0};
        float xx[vcu::kMaxHalfspaceDim > 5 ? 6 : 6] = {0, 0, 0, 0, 0, 0};
        for (std::size_t i = 0; i < DIM && i < 6; ++i) xx[i] = x[i];
        eval(xx, out);
        return out[0];
    }
    void eval(const float* x, float* out) const {
        switch (kind) {
        case vcu::VCU_F_POLY2: vcu::Poly2{}(x, out); break;
        case vcu::VCU_F_SIN1: vcu::Sin1{}(x, out); break;
        case vcu::VCU_F_SPHERE3: vcu::Sphere3{}(x, out); break;
        case vcu::VCU_F_WAVE2: vcu::Wave2{}(x, out); break;
        case vcu::VCU_F_SCENE2: { vcu::Scene2 f{}; if (!f.build(params.data(), (int)params.size())) f(x, out); break; }
        case vcu::VCU_F_MOVING_SCENE3: {
            vcu::MovingScene3 f{};
            if (!f.build(params.data(), (int)params.size())) f(x, out);
            break;
        }
        case vcu::VCU_F_HALFSPACE: { vcu::Halfspace f{}; if (!f.build(params.data(), (int)params.size())) f(x, out); break; }
        default: throw error(VCU_INVALID_ARG, "host evaluation not available for this integrand");
        }
    }
};

namespace detail {

template <class R> constexpr std::size_t range_dim() { return R::size; }

template <std::size_t DIMBINS, class R>
vcu_problem make_problem(const builtin_integrand& f, const std::array<std::size_t, DIMBINS>& res, const R& range) {
    static_assert(DIMBINS >= 1 && DIMBINS <= VCU_MAX_DIMBINS, "1..4 binned dimensions");
    constexpr std::size_t DIM = range_dim<R>();
    static_assert(DIM >= DIMBINS && DIM <= VCU_MAX_DIM, "range dimension must be DIMBINS..6");
    vcu_problem p{};
    p.f.kind = f.kind;
    p.f.n_params = (int32_t)f.params.size();
    p.f.params = f.params.empty() ? nullptr : f.params.data();
    p.dim = (int32_t)DIM;
    p.dimbins = (int32_t)DIMBINS;
    for (std::size_t d = 0; d < DIM; ++d) {
        p.range_min[d] = (float)range.min(d);
        p.range_max[d] = (float)range.max(d);
    }
    for (std::size_t d = 0; d < DIMBINS; ++d) p.resolution[d] = res[d];
    p.mem = VCU_MEM_HOST;
    return p;
}

/* write channel values into whatever bins(pos) returns: a float&/double& or an indexable value */
template <class T> void store(T& dst, const float* v, int ch, bool accumulate) {
    if constexpr (std::is_arithmetic_v<T>) {
        if (accumulate) dst += v[0];
        else dst = v[0];
    } else {
        for (int c = 0; c < ch; ++c) {
            if (accumulate) dst[c] += v[c];
            else dst[c] = v[c];
        }
    }
}

template <class Bins, std::size_t DIMBINS>
void write_back(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const std::vector<float>& out, int ch,
                bool accumulate) {
    std::array<std::size_t, DIMBINS> pos{};
    const std::size_t n = out.size() / ch;
    for (std::size_t lin = 0; lin < n; ++lin) {
        store(bins(pos), &out[lin * ch], ch, accumulate);
        for (std::size_t d = 0; d < DIMBINS; ++d) {
            if (++pos[d] < res[d]) break;
            pos[d] = 0;
        }
    }
}

/* the caller's bins(pos) values in viltrum's linear order (the start of an accumulating call) */
template <class T> void load(const T& src, float* v, int ch) {
    if constexpr (std::is_arithmetic_v<T>) {
        v[0] = (float)src;
    } else {
        for (int c = 0; c < ch; ++c) v[c] = (float)src[c];
    }
}
template <class Bins, std::size_t DIMBINS>
void read_in(Bins& bins, const std::array<std::size_t, DIMBINS>& res, std::vector<float>& out, int ch) {
    std::array<std::size_t, DIMBINS> pos{};
    const std::size_t n = out.size() / ch;
    for (std::size_t lin = 0; lin < n; ++lin) {
        load(bins(pos), &out[lin * ch], ch);
        for (std::size_t d = 0; d < DIMBINS; ++d) {
            if (++pos[d] < res[d]) break;
            pos[d] = 0;
        }
    }
}

template <class F> const builtin_integrand& as_builtin(const F& f) {
    static_assert(std::is_same_v<std::decay_t<F>, builtin_integrand>,
                  "CUDA integrators take a viltrum::cuda::builtin_integrand (integrand code cannot cross the C ABI)");
    return f;
}

template <std::size_t DIMBINS> std::size_t bin_count(const std::array<std::size_t, DIMBINS>& res) {
    std::size_t n = 1;
    for (auto r : res) n *= r;
    return n;
}

}  // namespace detail

/* ---------------------------------------------------------------- per-bin Monte Carlo */
/* drop-in for integrator_per_bin_parallel(monte_carlo(samples, seed)) (assigns), or with
 * accumulate=true for monte_carlo_per_bin_parallel(samples, seed) (adds into the bins) */
class per_bin_monte_carlo {
    unsigned long samples_;
    std::uint64_t seed_;
    bool accumulate_;

public:
    per_bin_monte_carlo(unsigned long samples, std::uint64_t seed, bool accumulate = false)
        : samples_(samples), seed_(seed), accumulate_(accumulate) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        const int ch = fi.channels();
        std::vector<float> out(detail::bin_count(res) * (std::size_t)ch);
        vcu_stats st{};
        if (accumulate_) {
            /* monte_carlo_per_bin_parallel's own factor, added on the device to the current values */
            detail::read_in(bins, res, out, ch);
            ctx.check(vcu_per_bin_monte_carlo_accumulate(ctx.get(), &p, samples_, seed_, nullptr, out.data(), &st));
        } else {
            ctx.check(vcu_per_bin_monte_carlo(ctx.get(), &p, samples_, seed_, out.data(), &st));
        }
        detail::write_back(bins, res, out, ch, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

inline per_bin_monte_carlo per_bin_monte_carlo_accumulate(unsigned long samples, std::uint64_t seed) {
    return per_bin_monte_carlo(samples, seed, true);
}

/* ---------------------------------------------------------------- per-bin adaptive nested */
struct nested_rule {
    vcu_nested n;
};
inline nested_rule boole_simpson(int heuristic = VCU_HEUR_DEFAULT, int metric = VCU_METRIC_ABSOLUTE) {
    return {{VCU_RULE_BOOLE, VCU_RULE_SIMPSON, heuristic, metric, 1e-5, 1e-37, 1e-37}};
}
inline nested_rule boole_trapezoidal(int heuristic = VCU_HEUR_DEFAULT, int metric = VCU_METRIC_ABSOLUTE) {
    return {{VCU_RULE_BOOLE, VCU_RULE_TRAPEZOIDAL, heuristic, metric, 1e-5, 1e-37, 1e-37}};
}
inline nested_rule simpson_trapezoidal(int heuristic = VCU_HEUR_DEFAULT, int metric = VCU_METRIC_ABSOLUTE) {
    return {{VCU_RULE_SIMPSON, VCU_RULE_TRAPEZOIDAL, heuristic, metric, 1e-5, 1e-37, 1e-37}};
}

/* drop-in for integrator_per_bin_parallel(integrator_adaptive_iterations(nested(H,L), heuristic,
 * iterations)) (assigns) */
class per_bin_adaptive_nested {
    nested_rule rule_;
    unsigned long iterations_;

public:
    per_bin_adaptive_nested(nested_rule r, unsigned long iterations) : rule_(r), iterations_(iterations) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        const int ch = fi.channels();
        std::vector<float> out(detail::bin_count(res) * (std::size_t)ch);
        vcu_stats st{};
        ctx.check(vcu_per_bin_adaptive_nested(ctx.get(), &p, &rule_.n, iterations_, out.data(), nullptr, &st));
        detail::write_back(bins, res, out, ch, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* drop-in for integrator_adaptive_iterations(nested(H,L), heuristic, iterations) used directly, and
 * integrator_adaptive_iterations_parallel: one heap over the whole range, every region added into
 * the bins it overlaps -- ACCUMULATES, like regions_integrator_sequential
 * (src/newton-cotes/regions-integrator-sequential.h:37-58) */
class adaptive_iterations {
    nested_rule rule_;
    unsigned long iterations_;

public:
    adaptive_iterations(nested_rule r, unsigned long iterations) : rule_(r), iterations_(iterations) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        const int ch = fi.channels();
        std::vector<float> out(detail::bin_count(res) * (std::size_t)ch);
        detail::read_in(bins, res, out, ch);
        vcu_stats st{};
        ctx.check(vcu_adaptive_iterations_global(ctx.get(), &p, &rule_.n, iterations_, out.data(), &st));
        detail::write_back(bins, res, out, ch, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* drop-in for integrator_adaptive_tolerance(nested(H,L), heuristic, tolerance)
 * (src/nested/integrator-adaptive-tolerance.h:9-56): ACCUMULATES, leaves in depth-first order */
class adaptive_tolerance {
    nested_rule rule_;
    float tolerance_;
    std::uint64_t max_regions_;

public:
    adaptive_tolerance(nested_rule r, float tolerance = 1e-3f, std::uint64_t max_regions = 0)
        : rule_(r), tolerance_(tolerance), max_regions_(max_regions) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        const int ch = fi.channels();
        std::vector<float> out(detail::bin_count(res) * (std::size_t)ch);
        detail::read_in(bins, res, out, ch);
        vcu_stats st{};
        ctx.check(vcu_adaptive_tolerance(ctx.get(), &p, &rule_.n, tolerance_, max_regions_, out.data(), nullptr, &st));
        detail::write_back(bins, res, out, ch, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* ---------------------------------------------------------------- control variates */
/* drop-in for integrator_region_based(regions_generator_adaptive_heap(nested(H,L), heuristic,
 * iterations), regions_integrator_parallel_variance_reduction(rr_uniform_region(), weight,
 * region_sampling_uniform(), std::mt19937(seed), samples)) -- integrator_crespo2021(iterations,
 * samples, seed) with crespo2021() (src/control-variates/integrator-crespo2021.h:7-22); assigns.
 * weight: cv_optimize_weight() (VCU_CV_OPTIMIZE) or cv_fixed_weight(alpha) (VCU_CV_FIXED). */
class control_variates {
    nested_rule rule_;
    unsigned long iterations_, samples_;
    std::uint64_t seed_;
    int weight_;
    double alpha_;
    int rr_, sampling_;
    float rr_factor_;
    double mis_power_, mis_cutoff_;
    int fubini_dims_ = 0;
    unsigned tail_samples_ = 0;

public:
    /* rr: VCU_RR_UNIFORM (rr_uniform_region), VCU_RR_INTEGRAL (rr_integral_region), VCU_RR_ERROR
     * (rr_error_region) or VCU_RR_PDF (rr_pdf_region(rr_factor)), region-russian-roulette.h:9-149;
     * sampling: VCU_RS_UNIFORM (region_sampling_uniform), VCU_RS_IMPORTANCE, VCU_RS_RUSSIAN_ROULETTE or
     * VCU_RS_MIS (region_sampling_mis(mis_power, mis_cutoff)), region-sampling.h:9-135 */
    control_variates(nested_rule r, unsigned long iterations, unsigned long samples, std::uint64_t seed,
                     int weight = VCU_CV_OPTIMIZE, double alpha = 1.0, int rr = VCU_RR_UNIFORM,
                     int sampling = VCU_RS_UNIFORM, float rr_factor = 0.01f, double mis_power = 1.0,
                     double mis_cutoff = 0.0)
        : rule_(r), iterations_(iterations), samples_(samples), seed_(seed), weight_(weight), alpha_(alpha),
          rr_(rr), sampling_(sampling), rr_factor_(rr_factor), mis_power_(mis_power), mis_cutoff_(mis_cutoff) {}

    /* regions over the first `dims` (2) dimensions only, the others integrated by `tail_samples` Monte
     * Carlo samples in every evaluation: regions_generator_fubini<2>(..., monte_carlo(tail_samples, ...))
     * (src/combination/regions-generator-fubini.h:7-28) */
    control_variates& fubini(int dims, unsigned tail_samples) {
        fubini_dims_ = dims;
        tail_samples_ = tail_samples;
        return *this;
    }

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        const int ch = fi.channels();
        std::vector<float> out(detail::bin_count(res) * (std::size_t)ch);
        vcu_cv cv{};
        cv.samples_per_bin = samples_;
        cv.seed = seed_;
        cv.weight = weight_;
        cv.alpha = alpha_;
        cv.rr = rr_;
        cv.sampling = sampling_;
        cv.rr_factor = rr_factor_;
        cv.mis_power = mis_power_;
        cv.mis_cutoff = mis_cutoff_;
        cv.fubini_dims = fubini_dims_;
        cv.tail_samples = tail_samples_;
        vcu_stats st{};
        ctx.check(vcu_control_variates(ctx.get(), &p, &rule_.n, iterations_, &cv, nullptr, out.data(), nullptr,
                                       nullptr, &st));
        detail::write_back(bins, res, out, ch, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* nested(simpson, trapezoidal) with error_heuristic_size(error_metric_relative()), as
 * integrator_crespo2021 builds it */
inline nested_rule crespo2021_rule() { return simpson_trapezoidal(VCU_HEUR_SIZE, VCU_METRIC_RELATIVE); }
inline control_variates crespo2021(unsigned long iterations, unsigned long samples, std::uint64_t seed = 0) {
    return control_variates(crespo2021_rule(), iterations, samples, seed);
}
/* integrator_crespo2021_infinite<2>(iterations, mc_samples, spp, seed) over a finite range
 * (src/control-variates/integrator-crespo2021.h:24-44) */
inline control_variates crespo2021_infinite(unsigned long iterations, unsigned mc_samples, unsigned long samples,
                                            std::uint64_t seed = 0) {
    return control_variates(crespo2021_rule(), iterations, samples, seed).fubini(2, mc_samples);
}

/* ---------------------------------------------------------------- learned control variate */
/* No reference counterpart: per bin, a frequency-encoded 4x64 MLP g trained online on the
 * integrand's own samples (early stopping on a held-out set every check_every steps), the
 * piecewise-quadratic interpolant h of g on each bin's grid of Simpson nodes as the control variate
 * (its integral is exact: the estimate is unbiased), and only f - h sampled; with fallback, a pilot
 * per bin picks the lower-variance of this and plain Monte Carlo (vcu_learned_control_variates);
 * assigns. */
class learned_control_variates {
    vcu_learned opt_;

public:
    explicit learned_control_variates(unsigned long samples, std::uint64_t seed = 0, unsigned train_steps = 1000,
                                      unsigned batch = 32768, float learning_rate = 3e-3f, int cells = 2,
                                      int cells_unbinned = 4, bool fallback = true, unsigned check_every = 0)
        : opt_{} {
        opt_.samples_per_bin = samples;
        opt_.seed = seed;
        opt_.train_steps = train_steps;
        opt_.batch = batch;
        opt_.learning_rate = learning_rate;
        opt_.check_every = check_every;
        opt_.fallback = fallback ? 1 : 0;
        opt_.cells = cells;
        opt_.cells_unbinned = cells_unbinned;
    }

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        const builtin_integrand& fi = detail::as_builtin(f);
        context& ctx = thread_context();
        logger.log_progress(std::size_t(0), std::size_t(1));
        vcu_problem p = detail::make_problem(fi, res, range);
        std::vector<float> out(detail::bin_count(res));
        vcu_stats st{};
        ctx.check(vcu_learned_control_variates(ctx.get(), &p, &opt_, out.data(), nullptr, nullptr, &st));
        detail::write_back(bins, res, out, 1, false);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* ---------------------------------------------------------------- independent integrals */
/* Many single-value viltrum::integrate(I, f, range) calls at once (vcu_integrate_batch): item i
 * uses monte_carlo(budget, seed) (method VCU_BATCH_MONTE_CARLO) or
 * integrator_adaptive_iterations(nested, budget - 1) (VCU_BATCH_NESTED) over its own range with its
 * own parameters of one integrand family.  Returns the values in item order. */
struct batch_item {
    int dim = 0;
    int method = VCU_BATCH_NESTED;
    std::uint64_t budget = 1, seed = 0;
    std::array<float, VCU_MAX_DIM> range_min{}, range_max{};
    std::vector<float> params;
};

inline std::vector<float> integrate_batch(int32_t kind, const std::vector<batch_item>& items,
                                          nested_rule rule = simpson_trapezoidal(),
                                          std::vector<float>* item_ms = nullptr) {
    context& ctx = thread_context();
    std::vector<vcu_batch_item> c(items.size());
    for (std::size_t i = 0; i < items.size(); ++i) {
        vcu_batch_item& b = c[i];
        b = vcu_batch_item{};
        b.dim = items[i].dim;
        b.method = items[i].method;
        b.budget = items[i].budget;
        b.seed = items[i].seed;
        for (int d = 0; d < VCU_MAX_DIM; ++d) {
            b.range_min[d] = items[i].range_min[d];
            b.range_max[d] = items[i].range_max[d];
        }
        b.n_params = (int32_t)items[i].params.size();
        b.params = items[i].params.empty() ? nullptr : items[i].params.data();
    }
    std::vector<float> out(items.size());
    vcu_batch_report rep{};
    if (item_ms) {
        item_ms->assign(items.size(), 0.0f);
        rep.item_ms = item_ms->data();
    }
    ctx.check(vcu_integrate_batch(ctx.get(), kind, &rule.n, c.data(), c.size(), out.data(), VCU_MEM_HOST, &rep,
                                  nullptr));
    return out;
}

}  // namespace cuda
}  // namespace viltrum
