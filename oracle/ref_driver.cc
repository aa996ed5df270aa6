/*
 * ref_driver.cc -- runs the UNMODIFIED viltrum reference headers on the built-in integrands.
 *
 * Test infrastructure only.  Compiled by oracle/Makefile (target `ref`) against the reference
 * sources where they lie (-I <reference root>) into oracle/_ref/libvref.so, which exports the
 * oracle.h entry points with a "ref_" prefix.  tests/golden/make_golden.py calls it to produce
 * the golden fixtures that pin the CPU restatement (oracle.cc) to the reference.
 *
 * Only the configurations the fixtures use are instantiated (the reference composes integrators
 * as compile-time types); anything else returns 9.
 */
#include "viltrum.h"

#include <array>
#include <cstring>
#include <vector>

#include "../include/vcu_integrands.h"
#include "oracle.h"
#include "vrgb.h"

namespace {

template <class T> struct VT;
template <> struct VT<float> {
    static constexpr int CH = 1;
    static float from(const float* o) { return o[0]; }
    static void to(const float& v, float* o) { o[0] = v; }
};
template <> struct VT<vrgb> {
    static constexpr int CH = 3;
    static vrgb from(const float* o) { return vrgb(o[0], o[1], o[2]); }
    static void to(const vrgb& v, float* o) { o[0] = v.c[0]; o[1] = v.c[1]; o[2] = v.c[2]; }
};

/* integrand as viltrum sees it: std::array<float,DIM> -> value; records points if asked */
struct Recorder {
    float* next = nullptr;
};
template <class Fun, std::size_t DIM, class T> struct RefF {
    const Fun* f;
    Recorder* rec;
    T operator()(const std::array<float, DIM>& x) const {
        if (rec && rec->next)
            for (std::size_t i = 0; i < DIM; ++i) *rec->next++ = x[i];
        float o[3];
        (*f)(x.data(), o);
        return VT<T>::from(o);
    }
};

template <std::size_t DIM> viltrum::Range<float, DIM> mk_range(const float* a, const float* b) {
    std::array<float, DIM> x, y;
    for (std::size_t i = 0; i < DIM; ++i) {
        x[i] = a[i];
        y[i] = b[i];
    }
    return viltrum::Range<float, DIM>(x, y);
}

template <std::size_t DB> std::array<std::size_t, DB> mk_res(const uint64_t* r) {
    std::array<std::size_t, DB> a;
    for (std::size_t i = 0; i < DB; ++i) a[i] = r[i];
    return a;
}

template <std::size_t DB, class T> struct BinStore {
    std::array<std::size_t, DB> res;
    std::vector<T> v;
    std::size_t lin(const std::array<std::size_t, DB>& p) const {
        std::size_t l = 0, m = 1;
        for (std::size_t i = 0; i < DB; ++i) {
            l += p[i] * m;
            m *= res[i];
        }
        return l;
    }
};

/* logger that captures the region list handed to Logger::log by IntegratorRegionBased
 * (src/newton-cotes/integrator-region-based.h:13-22) */
struct RegionLogger {
    float* regions_out = nullptr;
    Recorder* arm = nullptr; /* recording starts once the regions are built */
    float* arm_at = nullptr;
    std::string n;
    RegionLogger() = default;
    std::string name() const { return n; }
    void set_name(const std::string& s) { n = s; }
    template <typename Number> void log_progress(const Number&, const Number& = Number(1)) {}
    template <typename Data> void log(const Data& data) {
        if (arm) arm->next = arm_at;
        if (!regions_out) return;
        std::size_t k = 0;
        for (const auto& r : data) {
            constexpr std::size_t D = std::decay_t<decltype(r.range())>::size;
            for (std::size_t d = 0; d < D; ++d) {
                regions_out[k * 2 * D + d] = r.range().min(d);
                regions_out[k * 2 * D + D + d] = r.range().max(d);
            }
            ++k;
        }
    }
};

template <class Fun, std::size_t DIM, std::size_t DB, class T>
int run_mc(const Fun& fun, const float* rmin, const float* rmax, const uint64_t* res, uint64_t spp, uint64_t seed,
           int flavour, float* out, float* points) {
    Recorder rec{points};
    RefF<Fun, DIM, T> f{&fun, &rec};
    auto range = mk_range<DIM>(rmin, rmax);
    BinStore<DB, T> bs{mk_res<DB>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.resize(nb);
    for (std::size_t i = 0; i < nb; ++i) bs.v[i] = VT<T>::from(out + i * VT<T>::CH);
    auto bins = [&bs](const std::array<std::size_t, DB>& p) -> T& { return bs.v[bs.lin(p)]; };
    if (flavour == ORC_MC_PER_BIN_PARALLEL)
        viltrum::integrate(viltrum::integrator_per_bin_parallel(viltrum::monte_carlo(spp, seed)), bins, bs.res, f, range);
    else
        viltrum::integrate(viltrum::monte_carlo_per_bin_parallel(spp, seed), bins, bs.res, f, range);
    for (std::size_t i = 0; i < nb; ++i) VT<T>::to(bs.v[i], out + i * VT<T>::CH);
    return 0;
}

template <class Fun, std::size_t DIM, std::size_t DB, class T, class Rule, class Heur>
int run_nested(const Fun& fun, const float* rmin, const float* rmax, const uint64_t* res, const Rule& rule,
               const Heur& heur, uint64_t iters, float* out) {
    RefF<Fun, DIM, T> f{&fun, nullptr};
    auto range = mk_range<DIM>(rmin, rmax);
    BinStore<DB, T> bs{mk_res<DB>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.assign(nb, T(0.0));
    auto bins = [&bs](const std::array<std::size_t, DB>& p) -> T& { return bs.v[bs.lin(p)]; };
    viltrum::integrate(viltrum::integrator_per_bin_parallel(viltrum::integrator_adaptive_iterations(rule, heur, iters)),
                       bins, bs.res, f, range);
    for (std::size_t i = 0; i < nb; ++i) VT<T>::to(bs.v[i], out + i * VT<T>::CH);
    return 0;
}

/* integrator_adaptive_iterations used directly: one heap over the whole range, regions added into
 * the caller's bins (which start from `out`) */
template <class Fun, std::size_t DIM, std::size_t DB, class T, class Rule, class Heur>
int run_global(const Fun& fun, const float* rmin, const float* rmax, const uint64_t* res, const Rule& rule,
               const Heur& heur, uint64_t iters, float* out) {
    RefF<Fun, DIM, T> f{&fun, nullptr};
    auto range = mk_range<DIM>(rmin, rmax);
    BinStore<DB, T> bs{mk_res<DB>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.resize(nb);
    for (std::size_t i = 0; i < nb; ++i) bs.v[i] = VT<T>::from(out + i * VT<T>::CH);
    auto bins = [&bs](const std::array<std::size_t, DB>& p) -> T& { return bs.v[bs.lin(p)]; };
    viltrum::integrate(viltrum::integrator_adaptive_iterations(rule, heur, iters), bins, bs.res, f, range);
    for (std::size_t i = 0; i < nb; ++i) VT<T>::to(bs.v[i], out + i * VT<T>::CH);
    return 0;
}

template <class Fun, std::size_t DIM, std::size_t DB, class T, class Rule, class Heur>
int run_tolerance(const Fun& fun, const float* rmin, const float* rmax, const uint64_t* res, const Rule& rule,
                  const Heur& heur, float tol, float* out) {
    RefF<Fun, DIM, T> f{&fun, nullptr};
    auto range = mk_range<DIM>(rmin, rmax);
    BinStore<DB, T> bs{mk_res<DB>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.resize(nb);
    for (std::size_t i = 0; i < nb; ++i) bs.v[i] = VT<T>::from(out + i * VT<T>::CH);
    auto bins = [&bs](const std::array<std::size_t, DB>& p) -> T& { return bs.v[bs.lin(p)]; };
    viltrum::integrate(viltrum::integrator_adaptive_tolerance(rule, heur, tol), bins, bs.res, f, range);
    for (std::size_t i = 0; i < nb; ++i) VT<T>::to(bs.v[i], out + i * VT<T>::CH);
    return 0;
}

template <class Fun, std::size_t DIM, std::size_t DB, class T, class Rule, class Heur, class RR, class CV, class RS>
int run_cv(const Fun& fun, const float* rmin, const float* rmax, const uint64_t* res, const Rule& rule,
           const Heur& heur, uint64_t iters, uint64_t spp, uint64_t seed, RR rr, CV cv, RS rs, float* out,
           float* regions_out, float* points) {
    Recorder rec{nullptr};
    RefF<Fun, DIM, T> f{&fun, &rec};
    auto range = mk_range<DIM>(rmin, rmax);
    BinStore<DB, T> bs{mk_res<DB>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.assign(nb, T(0.0));
    auto bins = [&bs](const std::array<std::size_t, DB>& p) -> T& { return bs.v[bs.lin(p)]; };
    auto integrator = viltrum::integrator_region_based(
        viltrum::regions_generator_adaptive_heap(rule, heur, iters),
        viltrum::regions_integrator_parallel_variance_reduction(std::move(rr), std::move(cv), std::move(rs),
                                                                std::mt19937(seed),
                                                                spp));
    RegionLogger logger;
    logger.regions_out = regions_out;
    if (points) {
        logger.arm = &rec;
        logger.arm_at = points;
    }
    viltrum::integrate(integrator, bins, bs.res, f, range, logger);
    for (std::size_t i = 0; i < nb; ++i) VT<T>::to(bs.v[i], out + i * VT<T>::CH);
    return 0;
}

}  // namespace

extern "C" int ref_per_bin_monte_carlo(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                       const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                       uint64_t spp, uint64_t seed, int32_t flavour, float* out, float* points_out) {
    if (kind == vcu::VCU_F_WAVE2 && dim == 2 && dimbins == 1) {
        vcu::Wave2 f{};
        return run_mc<vcu::Wave2, 2, 1, float>(f, rmin, rmax, res, spp, seed, flavour, out, points_out);
    }
    if (kind == vcu::VCU_F_POLY2 && dim == 2 && dimbins == 2) {
        vcu::Poly2 f{};
        return run_mc<vcu::Poly2, 2, 2, float>(f, rmin, rmax, res, spp, seed, flavour, out, points_out);
    }
    if (kind == vcu::VCU_F_SIN1 && dim == 1 && dimbins == 1) {
        vcu::Sin1 f{};
        return run_mc<vcu::Sin1, 1, 1, float>(f, rmin, rmax, res, spp, seed, flavour, out, points_out);
    }
    if (kind == vcu::VCU_F_SPHERE3 && dim == 3 && dimbins == 1) {
        vcu::Sphere3 f{};
        return run_mc<vcu::Sphere3, 3, 1, float>(f, rmin, rmax, res, spp, seed, flavour, out, points_out);
    }
    if (kind == vcu::VCU_F_MOVING_SCENE3 && dim == 3 && dimbins == 2) {
        auto* f = new vcu::MovingScene3;
        int r = f->build(params, n_params) ? 3
                                           : run_mc<vcu::MovingScene3, 3, 2, vrgb>(*f, rmin, rmax, res, spp, seed,
                                                                                   flavour, out, points_out);
        delete f;
        return r;
    }
    return 9;
}

extern "C" int ref_per_bin_adaptive_nested(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                           const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                           const orc_nested* nc, uint64_t iterations, float* out, int32_t* trace) {
    (void)trace;
    using namespace viltrum;
    const bool bs_da = nc->rule_hi == ORC_RULE_BOOLE && nc->rule_lo == ORC_RULE_SIMPSON &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    const bool bs_dr = nc->rule_hi == ORC_RULE_BOOLE && nc->rule_lo == ORC_RULE_SIMPSON &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_RELATIVE;
    const bool st_sr = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_SIZE && nc->metric == ORC_METRIC_RELATIVE;
    const bool bt_da = nc->rule_hi == ORC_RULE_BOOLE && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    const bool st_da = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    auto hda = error_heuristic_default(error_metric_absolute());
    auto hdr = error_heuristic_default(error_metric_relative(nc->min_val));
    auto hsr = error_heuristic_size(error_metric_relative(nc->min_val), nc->size_weight, nc->min_size);
    if (kind == vcu::VCU_F_SCENE2 && dim == 2 && dimbins == 2) {
        auto* f = new vcu::Scene2;
        int r = 9;
        if (f->build(params, n_params)) r = 3;
        else if (bs_da) r = run_nested<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(boole, simpson), hda, iterations, out);
        else if (bs_dr) r = run_nested<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(boole, simpson), hdr, iterations, out);
        else if (st_sr) r = run_nested<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hsr, iterations, out);
        delete f;
        return r;
    }
    if (kind == vcu::VCU_F_POLY2 && dim == 2 && dimbins == 1 && bs_da) {
        vcu::Poly2 f{};
        return run_nested<vcu::Poly2, 2, 1, float>(f, rmin, rmax, res, nested(boole, simpson), hda, iterations, out);
    }
    if (kind == vcu::VCU_F_WAVE2 && dim == 2 && dimbins == 1 && bs_da) {
        vcu::Wave2 f{};
        return run_nested<vcu::Wave2, 2, 1, float>(f, rmin, rmax, res, nested(boole, simpson), hda, iterations, out);
    }
    if (kind == vcu::VCU_F_WAVE2 && dim == 2 && dimbins == 2 && bt_da) {
        vcu::Wave2 f{};
        return run_nested<vcu::Wave2, 2, 2, float>(f, rmin, rmax, res, nested(boole, trapezoidal), hda, iterations, out);
    }
    if (kind == vcu::VCU_F_HALFSPACE && dim == 3 && dimbins == 1 && st_da) {
        vcu::Halfspace f{};
        if (f.build(params, n_params) || f.dim != 3) return 3;
        return run_nested<vcu::Halfspace, 3, 1, float>(f, rmin, rmax, res, nested(simpson, trapezoidal),
                                                        error_heuristic_default(error_metric_absolute()), iterations, out);
    }
    if (kind == vcu::VCU_F_MOVING_SCENE3 && dim == 3 && dimbins == 2 && st_sr) {
        auto* f = new vcu::MovingScene3;
        int r = f->build(params, n_params)
                    ? 3
                    : run_nested<vcu::MovingScene3, 3, 2, vrgb>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hsr,
                                                                 iterations, out);
        delete f;
        return r;
    }
    return 9;
}

/* the residual strategy, as the reference's own objects: the region choice (rr_uniform_region,
 * rr_integral_region, rr_error_region, rr_pdf_region) and the point sampler (region_sampling_uniform,
 * region_sampling_importance, region_sampling_russian_roulette, region_sampling_mis).  The point
 * samplers other than uniform are built with the uniform or the pdf region choice only. */
template <class Fn> int with_rr(const orc_cv& cv, Fn&& fn) {
    using namespace viltrum;
    const float fp = cv.rr_factor;
    switch (cv.sampling) {
    case ORC_RS_UNIFORM:
        switch (cv.rr) {
        case ORC_RR_UNIFORM: return fn(rr_uniform_region(), region_sampling_uniform());
        case ORC_RR_INTEGRAL: return fn(rr_integral_region(), region_sampling_uniform());
        case ORC_RR_ERROR: return fn(rr_error_region(), region_sampling_uniform());
        case ORC_RR_PDF: return fn(rr_pdf_region(fp), region_sampling_uniform());
        default: return 1;
        }
    case ORC_RS_IMPORTANCE:
        if (cv.rr == ORC_RR_UNIFORM) return fn(rr_uniform_region(), region_sampling_importance());
        if (cv.rr == ORC_RR_PDF) return fn(rr_pdf_region(fp), region_sampling_importance());
        return 9;
    case ORC_RS_RUSSIAN_ROULETTE:
        if (cv.rr == ORC_RR_UNIFORM) return fn(rr_uniform_region(), region_sampling_russian_roulette());
        if (cv.rr == ORC_RR_PDF) return fn(rr_pdf_region(fp), region_sampling_russian_roulette());
        return 9;
    case ORC_RS_MIS:
        if (cv.rr == ORC_RR_UNIFORM) return fn(rr_uniform_region(), region_sampling_mis(cv.mis_power, cv.mis_cutoff));
        if (cv.rr == ORC_RR_PDF) return fn(rr_pdf_region(fp), region_sampling_mis(cv.mis_power, cv.mis_cutoff));
        return 9;
    default: return 1;
    }
}

extern "C" int ref_control_variates(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                    const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                    const orc_nested* nc, uint64_t iterations, uint64_t spp, uint64_t seed,
                                    const orc_cv* cv, float* out, float* approx_out, float* regions_out,
                                    float* replay_out) {
    (void)approx_out;
    using namespace viltrum;
    const bool st_sr = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_SIZE && nc->metric == ORC_METRIC_RELATIVE;
    if (!st_sr) return 9;
    auto hsr = error_heuristic_size(error_metric_relative(nc->min_val), nc->size_weight, nc->min_size);
    /* replay_out receives the recorded sample points only (spp x dim per bin); the chosen
     * region indices are internal to the reference */
    return with_rr(*cv, [&](auto rrs, auto rs) -> int {
        if (kind == vcu::VCU_F_MOVING_SCENE3 && dim == 3 && dimbins == 2 && cv->weight == ORC_CV_OPTIMIZE) {
            auto* f = new vcu::MovingScene3;
            int r = f->build(params, n_params)
                        ? 3
                        : run_cv<vcu::MovingScene3, 3, 2, vrgb>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hsr,
                                                                 iterations, spp, seed, rrs, cv_optimize_weight(), rs,
                                                                 out, regions_out, replay_out);
            delete f;
            return r;
        }
        if (kind == vcu::VCU_F_SCENE2 && dim == 2 && dimbins == 2) {
            auto* f = new vcu::Scene2;
            int r = 3;
            if (!f->build(params, n_params)) {
                if (cv->weight == ORC_CV_OPTIMIZE)
                    r = run_cv<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hsr,
                                                          iterations, spp, seed, rrs, cv_optimize_weight(), rs, out,
                                                          regions_out, replay_out);
                else
                    r = run_cv<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hsr,
                                                          iterations, spp, seed, rrs, cv_fixed_weight(cv->alpha), rs,
                                                          out, regions_out, replay_out);
            }
            delete f;
            return r;
        }
        if (kind == vcu::VCU_F_POLY2 && dim == 2 && dimbins == 1 && cv->weight == ORC_CV_OPTIMIZE) {
            vcu::Poly2 f{};
            return run_cv<vcu::Poly2, 2, 1, float>(f, rmin, rmax, res, nested(simpson, trapezoidal), hsr, iterations,
                                                    spp, seed, rrs, cv_optimize_weight(), rs, out, regions_out,
                                                    replay_out);
        }
        return 9;
    });
}

/* the walk over the scene as the reference takes an integrand of unbounded dimension: a callable
 * on its random sequence (src/monte-carlo/random-sequence-*.h), read in order */
struct RefWalk {
    const vcu::Walk2* w;
    template <class Seq> float operator()(const Seq& seq) const {
        auto it = seq.begin();
        const float x = *it;
        ++it;
        const float y = *it;
        ++it;
        return w->walk(x, y, [&]() {
            const float v = *it;
            ++it;
            return v;
        });
    }
};

/* over range_infinite(rmin, rmax) (two listed dimensions, the rest [0,1]): per-bin Monte Carlo
 * (method 0: integrator_per_bin_parallel(monte_carlo(spp, seed))) or crespo2021_infinite<2>
 * (method 1, iterations, mc_samples) into res[0] x res[1] bins */
extern "C" int ref_walk(const float* params, int32_t n_params, const float* rmin, const float* rmax,
                        const uint64_t* res, int32_t method, uint64_t spp, uint64_t seed, uint64_t iterations,
                        uint64_t mc_samples, float* out) {
    auto* fn = new vcu::Walk2;
    if (fn->build(params, n_params)) {
        delete fn;
        return 3;
    }
    RefWalk f{fn};
    const auto range = viltrum::range_infinite(rmin[0], rmin[1], rmax[0], rmax[1]);
    BinStore<2, float> bs{mk_res<2>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.assign(nb, 0.0f);
    auto bins = [&bs](const std::array<std::size_t, 2>& q) -> float& { return bs.v[bs.lin(q)]; };
    if (method == 0)
        viltrum::integrate(viltrum::integrator_per_bin_parallel(viltrum::monte_carlo(spp, seed)), bins, bs.res, f,
                           range);
    else
        viltrum::integrate(viltrum::integrator_crespo2021_infinite<2>(iterations, mc_samples, spp, seed), bins, bs.res,
                           f, range);
    for (std::size_t i = 0; i < nb; ++i) out[i] = bs.v[i];
    delete fn;
    return 0;
}

/* integrator_crespo2021_infinite<2>(iterations, mc_samples, spp, seed) over the finite range of the
 * moving-disk scene: regions over (x, y), time integrated by Monte Carlo in every evaluation
 * (src/control-variates/integrator-crespo2021.h:24-44) */
extern "C" int ref_crespo2021_infinite(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                       const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                       uint64_t iterations, uint64_t mc_samples, uint64_t spp, uint64_t seed,
                                       float* out) {
    if (kind != vcu::VCU_F_MOVING_SCENE3 || dim != 3 || dimbins != 2) return 9;
    auto* fn = new vcu::MovingScene3;
    if (fn->build(params, n_params)) {
        delete fn;
        return 3;
    }
    RefF<vcu::MovingScene3, 3, vrgb> f{fn, nullptr};
    auto range = mk_range<3>(rmin, rmax);
    BinStore<2, vrgb> bs{mk_res<2>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.assign(nb, vrgb(0.0));
    auto bins = [&bs](const std::array<std::size_t, 2>& q) -> vrgb& { return bs.v[bs.lin(q)]; };
    viltrum::integrate(viltrum::integrator_crespo2021_infinite<2>(iterations, mc_samples, spp, seed), bins, bs.res, f,
                       range);
    for (std::size_t i = 0; i < nb; ++i) VT<vrgb>::to(bs.v[i], out + i * 3);
    delete fn;
    return 0;
}

/* integrator_fubini<2>(integrator_per_bin_parallel(first), monte_carlo(mc_samples, seed + 1)) over the
 * moving-disk scene (RGB), first = monte_carlo(spp, seed) (method 0) or
 * integrator_adaptive_iterations(nested(simpson, trapezoidal), iterations) (method 1); with
 * swap_xt the problem is reordered first, integrator_fubini({0, 2}, ...) (fubini.h:111-115): the
 * bins span dimensions 0 and 2 and dimension 1 is the Monte Carlo tail */
extern "C" int ref_per_bin_fubini(const float* params, int32_t n_params, const float* rmin, const float* rmax,
                                  const uint64_t* res, int32_t method, uint64_t spp, uint64_t iterations,
                                  uint64_t mc_samples, uint64_t seed, int32_t swap_xt, float* out) {
    auto* fn = new vcu::MovingScene3;
    if (fn->build(params, n_params)) {
        delete fn;
        return 3;
    }
    using namespace viltrum;
    RefF<vcu::MovingScene3, 3, vrgb> f{fn, nullptr};
    auto range = mk_range<3>(rmin, rmax);
    BinStore<2, vrgb> bs{mk_res<2>(res), {}};
    std::size_t nb = 1;
    for (auto r : bs.res) nb *= r;
    bs.v.assign(nb, vrgb(0.0));
    auto bins = [&bs](const std::array<std::size_t, 2>& q) -> vrgb& { return bs.v[bs.lin(q)]; };
    auto rest = monte_carlo((unsigned long)mc_samples, (std::size_t)(seed + 1));
    auto go = [&](const auto& first) {
        /* integrator_fubini's return type takes the argument types as deduced: pass rvalues */
        auto a = first;
        auto b = rest;
        if (swap_xt)
            integrate(integrator_fubini(std::tuple<std::size_t, std::size_t>{0, 2}, std::move(a), std::move(b)), bins,
                      bs.res, f, range);
        else
            integrate(integrator_fubini<2>(std::move(a), std::move(b)), bins, bs.res, f, range);
    };
    if (method == 0)
        go(integrator_per_bin_parallel(monte_carlo((unsigned long)spp, (std::size_t)seed)));
    else
        go(integrator_per_bin_parallel(integrator_adaptive_iterations(nested(simpson, trapezoidal), (std::size_t)iterations)));
    for (std::size_t i = 0; i < nb; ++i) VT<vrgb>::to(bs.v[i], out + i * 3);
    delete fn;
    return 0;
}

/* single-value integrate(I, f, range) of the half-space family: the items of a batch of
 * independent integrals (monte_carlo(budget, seed), or adaptive nested(simpson, trapezoidal) with
 * budget regions and the default heuristic / absolute metric) */
template <std::size_t DIM>
static int ref_single_halfspace(const vcu::Halfspace& f, const float* rmin, const float* rmax, int32_t method,
                                uint64_t budget, uint64_t seed, float* out) {
    using namespace viltrum;
    RefF<vcu::Halfspace, DIM, float> F{&f, nullptr};
    const auto range = mk_range<DIM>(rmin, rmax);
    if (method == 0) {
        *out = integrate(monte_carlo((unsigned long)budget, (std::size_t)seed), F, range);
    } else {
        *out = integrate(integrator_adaptive_iterations(nested(simpson, trapezoidal), (std::size_t)(budget - 1)), F, range);
    }
    return 0;
}

extern "C" int ref_integrate_single(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* rmin,
                                    const float* rmax, int32_t method, uint64_t budget, uint64_t seed,
                                    const orc_nested* nc, float* out) {
    if (kind != vcu::VCU_F_HALFSPACE || budget == 0 || (method != 0 && method != 1)) return 9;
    if (method == 1 && !(nc && nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                         nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE))
        return 9;
    vcu::Halfspace f{};
    if (f.build(params, n_params) || f.dim != dim) return 3;
    switch (dim) {
    case 2: return ref_single_halfspace<2>(f, rmin, rmax, method, budget, seed, out);
    case 3: return ref_single_halfspace<3>(f, rmin, rmax, method, budget, seed, out);
    case 4: return ref_single_halfspace<4>(f, rmin, rmax, method, budget, seed, out);
    case 5: return ref_single_halfspace<5>(f, rmin, rmax, method, budget, seed, out);
    case 6: return ref_single_halfspace<6>(f, rmin, rmax, method, budget, seed, out);
    default: return 9;
    }
}

extern "C" int ref_adaptive_global(int32_t kind, const float* params, int32_t n_params, int32_t dim, const float* rmin,
                                   const float* rmax, int32_t dimbins, const uint64_t* res, const orc_nested* nc,
                                   uint64_t iterations, float* out) {
    using namespace viltrum;
    const bool st_da = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    const bool bs_da = nc->rule_hi == ORC_RULE_BOOLE && nc->rule_lo == ORC_RULE_SIMPSON &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    const bool st_sr = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_SIZE && nc->metric == ORC_METRIC_RELATIVE;
    auto hda = error_heuristic_default(error_metric_absolute());
    auto hsr = error_heuristic_size(error_metric_relative(nc->min_val), nc->size_weight, nc->min_size);
    if (kind == vcu::VCU_F_SCENE2 && dim == 2 && dimbins == 2 && st_da) {
        auto* f = new vcu::Scene2;
        const int r = f->build(params, n_params)
                          ? 3
                          : run_global<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(simpson, trapezoidal), hda,
                                                                 iterations, out);
        delete f;
        return r;
    }
    if (kind == vcu::VCU_F_MOVING_SCENE3 && dim == 3 && dimbins == 2 && bs_da) {
        auto* f = new vcu::MovingScene3;
        const int r = f->build(params, n_params)
                          ? 3
                          : run_global<vcu::MovingScene3, 3, 2, vrgb>(*f, rmin, rmax, res, nested(boole, simpson), hda,
                                                                      iterations, out);
        delete f;
        return r;
    }
    if (kind == vcu::VCU_F_HALFSPACE && dim == 3 && dimbins == 1 && st_sr) {
        vcu::Halfspace f{};
        if (f.build(params, n_params) || f.dim != 3) return 3;
        return run_global<vcu::Halfspace, 3, 1, float>(f, rmin, rmax, res, nested(simpson, trapezoidal), hsr, iterations,
                                                       out);
    }
    return 9;
}

extern "C" int64_t ref_adaptive_tolerance(int32_t kind, const float* params, int32_t n_params, int32_t dim,
                                          const float* rmin, const float* rmax, int32_t dimbins, const uint64_t* res,
                                          const orc_nested* nc, float tolerance, uint64_t max_regions, float* out) {
    (void)max_regions;
    using namespace viltrum;
    const bool st_da = nc->rule_hi == ORC_RULE_SIMPSON && nc->rule_lo == ORC_RULE_TRAPEZOIDAL &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    const bool bs_da = nc->rule_hi == ORC_RULE_BOOLE && nc->rule_lo == ORC_RULE_SIMPSON &&
                       nc->heuristic == ORC_HEUR_DEFAULT && nc->metric == ORC_METRIC_ABSOLUTE;
    auto hda = error_heuristic_default(error_metric_absolute());
    if (kind == vcu::VCU_F_SCENE2 && dim == 2 && dimbins == 2 && bs_da) {
        auto* f = new vcu::Scene2;
        const int r = f->build(params, n_params)
                          ? 3
                          : run_tolerance<vcu::Scene2, 2, 2, float>(*f, rmin, rmax, res, nested(boole, simpson), hda,
                                                                    tolerance, out);
        delete f;
        return r ? -2 : 0;
    }
    if (kind == vcu::VCU_F_MOVING_SCENE3 && dim == 3 && dimbins == 2 && st_da) {
        auto* f = new vcu::MovingScene3;
        const int r = f->build(params, n_params)
                          ? 3
                          : run_tolerance<vcu::MovingScene3, 3, 2, vrgb>(*f, rmin, rmax, res, nested(simpson, trapezoidal),
                                                                         hda, tolerance, out);
        delete f;
        return r ? -2 : 0;
    }
    return -9;
}

/* the weight accumulator and the 1-D Simpson pdf / sampler of the reference itself */
extern "C" int ref_cv_optimize_moments(const float* f, const float* g, uint64_t n, float approximation,
                                       double* out) {
    if ((n && (!f || !g)) || !out) return 1;
    auto acc = viltrum::cv_optimize_weight().accumulator<float>();
    for (uint64_t i = 0; i < n; ++i) acc.push(f[i], g[i]);
    out[0] = acc.variance();
    out[1] = acc.covariance();
    out[2] = acc.alpha();
    out[3] = acc.integral(approximation);
    return 0;
}

namespace {
/* a region over [0,1] whose nodes 0, 0.5, 1 read the given values */
auto node_region(const float* nodes) {
    const float n0 = nodes[0], n1 = nodes[1], n2 = nodes[2];
    auto f = [n0, n1, n2](const std::array<float, 1>& x) { return (x[0] == 0.0f) ? n0 : ((x[0] == 1.0f) ? n2 : n1); };
    return viltrum::region(f, viltrum::simpson, viltrum::range(0.0f, 1.0f));
}
}  // namespace

extern "C" int ref_simpson_pdf_1d(const float* nodes, float t, float t0, float t1, float* out) {
    if (!nodes || !out) return 1;
    *out = node_region(nodes).pdf_subrange(std::array<float, 1>{t}, viltrum::range(t0, t1));
    return 0;
}

extern "C" int ref_simpson_sample_1d(const float* nodes, float s, float t0, float t1, float* out) {
    if (!nodes || !out) return 1;
    *out = node_region(nodes).sample_subrange(std::array<float, 1>{s}, viltrum::range(t0, t1))[0];
    return 0;
}
