/*
 * The C++ drop-in integrators of include/viltrum_cuda.hpp used the way viltrum code uses its own.
 *
 * With -DWITH_VILTRUM (and the reference's sources on the include path) every integrator goes
 * through viltrum::integrate(integrator, bins, f, range) exactly where a CPU integrator would
 * (src/integrate.h:72-97): this is compiled, not run, on machines that have the reference.
 * Without it, a minimal range type and bins accessor call integrate() directly; the program runs
 * on the GPU and prints the results (one value per line) for the test to compare with the C ABI.
 */
#include <array>
#include <cstdio>
#include <vector>
#ifdef WITH_VILTRUM
#include "viltrum.h"
#endif
#include "viltrum_cuda.hpp"

namespace vc = viltrum::cuda;

#ifndef WITH_VILTRUM
template <std::size_t DIM> struct box {
    static constexpr std::size_t size = DIM;
    std::array<float, DIM> lo, hi;
    float min(std::size_t i) const { return lo[i]; }
    float max(std::size_t i) const { return hi[i]; }
};
struct quiet {
    void log_progress(std::size_t, std::size_t) {}
};
#endif

static std::vector<float> scene_params() {
    /* two Gaussian bumps and one disk: [ng, nd, (cx, cy, sigma, a) x ng, (cx, cy, r, v) x nd] */
    return {2, 1, 0.3f, 0.4f, 0.05f, 0.8f, 0.7f, 0.6f, 0.1f, 0.5f, 0.5f, 0.5f, 0.2f, 0.25f};
}

int main() {
    const auto scene = vc::builtin_integrand::scene2(scene_params());
    const auto wave = vc::builtin_integrand::wave2();
    std::vector<std::vector<float>> image(16, std::vector<float>(16, 0.0f));
    std::vector<float> row(64, 0.0f), cv_bins(64, 0.0f), learned(16, 0.0f), global(32, 0.5f), cv_err(64, 0.0f);
    /* rr_error_region with cv_fixed_weight(0.5) */
    const auto cv_error = vc::control_variates(vc::crespo2021_rule(), 255, 16, 4, VCU_CV_FIXED, 0.5, VCU_RR_ERROR);
#ifdef WITH_VILTRUM
    viltrum::integrate(vc::per_bin_adaptive_nested(vc::boole_simpson(), 15), image, scene, viltrum::range_primary<2>());
    viltrum::integrate(vc::per_bin_monte_carlo(256, 7), row, wave, viltrum::range_primary<2>());
    viltrum::integrate(vc::per_bin_monte_carlo_accumulate(256, 9), row, wave, viltrum::range_primary<2>());
    viltrum::integrate(vc::crespo2021(255, 16, 3), cv_bins, scene, viltrum::range_primary<2>());
    viltrum::integrate(vc::learned_control_variates(16, 5, 50), learned, wave, viltrum::range_primary<2>());
    viltrum::integrate(vc::adaptive_iterations(vc::simpson_trapezoidal(), 127), global, scene, viltrum::range_primary<2>());
    viltrum::integrate(vc::adaptive_tolerance(vc::boole_simpson(), 1e-6f), global, scene, viltrum::range_primary<2>());
    viltrum::integrate(cv_error, cv_err, scene, viltrum::range_primary<2>());
#else
    quiet log;
    const box<2> unit{{0.0f, 0.0f}, {1.0f, 1.0f}};
    auto img = [&](const std::array<std::size_t, 2>& p) -> float& { return image[p[1]][p[0]]; };
    auto r1 = [&](const std::array<std::size_t, 1>& p) -> float& { return row[p[0]]; };
    auto c1 = [&](const std::array<std::size_t, 1>& p) -> float& { return cv_bins[p[0]]; };
    auto l1 = [&](const std::array<std::size_t, 1>& p) -> float& { return learned[p[0]]; };
    vc::per_bin_adaptive_nested(vc::boole_simpson(), 15).integrate(img, std::array<std::size_t, 2>{16, 16}, scene, unit, log);
    vc::per_bin_monte_carlo(256, 7).integrate(r1, std::array<std::size_t, 1>{64}, wave, unit, log);
    vc::per_bin_monte_carlo_accumulate(256, 9).integrate(r1, std::array<std::size_t, 1>{64}, wave, unit, log);
    vc::crespo2021(255, 16, 3).integrate(c1, std::array<std::size_t, 1>{64}, scene, unit, log);
    vc::learned_control_variates(16, 5, 50).integrate(l1, std::array<std::size_t, 1>{16}, wave, unit, log);
    auto g1 = [&](const std::array<std::size_t, 1>& p) -> float& { return global[p[0]]; };
    vc::adaptive_iterations(vc::simpson_trapezoidal(), 127).integrate(g1, std::array<std::size_t, 1>{32}, scene, unit, log);
    vc::adaptive_tolerance(vc::boole_simpson(), 1e-6f).integrate(g1, std::array<std::size_t, 1>{32}, scene, unit, log);
    auto e1 = [&](const std::array<std::size_t, 1>& p) -> float& { return cv_err[p[0]]; };
    cv_error.integrate(e1, std::array<std::size_t, 1>{64}, scene, unit, log);
#endif
    /* independent integrals: two half-space items, one nested and one Monte Carlo */
    std::vector<vc::batch_item> items(2);
    for (int i = 0; i < 2; ++i) {
        items[i].dim = 2;
        items[i].method = i == 0 ? VCU_BATCH_NESTED : VCU_BATCH_MONTE_CARLO;
        items[i].budget = i == 0 ? 100 : 4096;
        items[i].seed = 11;
        items[i].range_max = {1, 1, 0, 0, 0, 0};
        items[i].params = {2, 1.5f, 0.5f, 0, 0, 0, 0, 3.0f, 7.0f, 0, 0, 0, 0, 0.6f, 0.8f, 0, 0, 0, 0, 0.9f};
    }
    const std::vector<float> batch = vc::integrate_batch(vcu::VCU_F_HALFSPACE, items);
    for (auto& r : image)
        for (float v : r) std::printf("%.9g\n", v);
    for (float v : row) std::printf("%.9g\n", v);
    for (float v : cv_bins) std::printf("%.9g\n", v);
    for (float v : learned) std::printf("%.9g\n", v);
    for (float v : global) std::printf("%.9g\n", v);
    for (float v : batch) std::printf("%.9g\n", v);
    for (float v : cv_err) std::printf("%.9g\n", v);
    return 0;
}
