/*
 * A caller's own integrand functors through include/viltrum_cuda_device.cuh.
 *
 * Standalone form (the GPU test, tests/test_gpu_user_functor.py): runs the device integrators on
 * three user functors and prints their bins next to the oracle's (oracle/oracle_impl.h run on the
 * host over the very same functors), plus a per-bin Monte Carlo image of the first functor.
 * WITH_VILTRUM form (the CPU test, compile only): the same integrators passed to the reference's
 * own viltrum::integrate with the same functors -- the std::array form and, through
 * viltrum::cuda::device::arity, a functor of separate float arguments.
 *
 * The functors use correctly rounded operations (vcu_integrands.h's vadd/vmul/vsub/vexp/vsin),
 * so they return the same bits on the host and on the device.
 */
#include <array>
#include <cstdio>
#include <vector>

#ifdef WITH_VILTRUM
/* the parts of viltrum the integrate() call needs (nvcc's front end rejects a combination header of
 * viltrum.h, src/combination/sequence_from_iterators.h:14, that g++ accepts) */
#include "src/integrate.h"
#include "src/range.h"
#endif
#include "viltrum_cuda_device.cuh"
#ifndef WITH_VILTRUM
#include "../../oracle/oracle_impl.h"
#endif

namespace vd = viltrum::cuda::device;

/* sin(8x) e^-y + x^2 + y^2 (the library's built-in "wave", written as a user would) */
struct UserWave {
    __host__ __device__ float operator()(const std::array<float, 2>& x) const {
        float t = vcu::vmul(vcu::vsin(vcu::vmul(8.0f, x[0])), vcu::vexp(-x[1]));
        t = vcu::vadd(t, vcu::vmul(x[0], x[0]));
        return vcu::vadd(t, vcu::vmul(x[1], x[1]));
    }
};

/* a Gaussian shell in 3-D, taking three separate coordinates (passed through vd::arity<3>) */
struct Shell {
    float cx, cy, cz, r0, k;
    __host__ __device__ float operator()(float x, float y, float z) const {
        const float dx = vcu::vsub(x, cx), dy = vcu::vsub(y, cy), dz = vcu::vsub(z, cz);
        const float r2 = vcu::vadd(vcu::vadd(vcu::vmul(dx, dx), vcu::vmul(dy, dy)), vcu::vmul(dz, dz));
        const float d = vcu::vsub(r2, vcu::vmul(r0, r0));
        return vcu::vexp(vcu::vmul(-k, vcu::vmul(d, d)));
    }
};

/* three channels: a colour ramp times a step */
struct Ramp {
    float edge;
    __host__ __device__ std::array<float, 3> operator()(const std::array<float, 2>& x) const {
        const float s = vcu::vadd(x[0], x[1]) > edge ? 1.0f : 0.25f;
        return {vcu::vmul(s, x[0]), vcu::vmul(s, x[1]), vcu::vmul(s, vcu::vmul(x[0], x[1]))};
    }
};

#ifdef WITH_VILTRUM
int main() {
    std::vector<std::vector<float>> image(16, std::vector<float>(32));
    viltrum::integrate(vd::per_bin_adaptive_nested<5, 3>(15), image, UserWave{}, viltrum::range_primary<2>());
    viltrum::integrate(vd::per_bin_monte_carlo(256, 7), image, UserWave{}, viltrum::range_primary<2>());
    std::vector<std::vector<float>> slab(8, std::vector<float>(8));
    viltrum::integrate(vd::per_bin_adaptive_nested<3, 2>(8, VCU_HEUR_SIZE, VCU_METRIC_RELATIVE), slab,
                       vd::arity<3>(Shell{0.5f, 0.5f, 0.5f, 0.3f, 40.0f}), viltrum::range_primary<3>());
    std::vector<std::vector<std::array<float, 3>>> rgb(16, std::vector<std::array<float, 3>>(16));
    viltrum::integrate(vd::per_bin_adaptive_nested<5, 2>(7), rgb, Ramp{0.9f}, viltrum::range_primary<2>());
    return 0;
}
#else
template <int DIM> struct box {
    static constexpr std::size_t size = DIM;
    std::array<float, DIM> lo, hi;
    float min(std::size_t d) const { return lo[d]; }
    float max(std::size_t d) const { return hi[d]; }
};
struct quiet {
    void log_progress(std::size_t, std::size_t) const {}
};

template <int DIM, class F, class T, class H, class L, class M>
std::vector<float> oracle_nested(const F& f, const std::array<float, DIM>& lo, const std::array<float, DIM>& hi,
                                 std::vector<uint64_t> res, int heuristic, int metric, uint64_t iters) {
    using U = vd::detail::user_fn<F, DIM>;
    const U u{f};
    orc::Problem p{DIM, (int)res.size(), lo.data(), hi.data(), res.data()};
    orc_nested nc{H::S, L::S, heuristic, metric, 1e-5, 1e-37, 1e-37};
    std::vector<float> out(p.nbins() * U::CH);
    M m{};
    if constexpr (std::is_same_v<M, orc::MetricRel>) m.min_val = nc.min_val;
    orc::per_bin_nested_range<H, L, DIM, T>(u, p, nc, m, iters, 0, p.nbins(), out.data(), nullptr);
    return out;
}

static void print(const char* name, const std::vector<float>& v) {
    std::printf("%s %zu", name, v.size());
    for (float x : v) std::printf(" %.9g", x);
    std::printf("\n");
}

int main() {
    quiet log;
    /* 1. the wave, nested(boole, simpson), 15 splits, 32x16 bins */
    {
        std::vector<float> gpu(32 * 16);
        auto b = [&](const std::array<std::size_t, 2>& q) -> float& { return gpu[q[1] * 32 + q[0]]; };
        const box<2> unit{{0.0f, 0.0f}, {1.0f, 1.0f}};
        vd::per_bin_adaptive_nested<5, 3>(15).integrate(b, std::array<std::size_t, 2>{32, 16}, UserWave{}, unit, log);
        print("wave_gpu", gpu);
        print("wave_oracle", oracle_nested<2, UserWave, float, orc::Boole, orc::Simpson, orc::MetricAbs>(
                                 UserWave{}, {0.0f, 0.0f}, {1.0f, 1.0f}, {32, 16}, 0, 0, 15));
    }
    /* 2. the shell through arity<3>: nested(simpson, trapezoidal), size heuristic, relative metric,
     *    8 splits, 12x8 bins over the first two dimensions of [-0.1,1.1]x[0,1]x[0,1] */
    {
        const auto shell = vd::arity<3>(Shell{0.5f, 0.45f, 0.5f, 0.3f, 40.0f});
        std::vector<float> gpu(12 * 8);
        auto b = [&](const std::array<std::size_t, 2>& q) -> float& { return gpu[q[1] * 12 + q[0]]; };
        const box<3> r{{-0.1f, 0.0f, 0.0f}, {1.1f, 1.0f, 1.0f}};
        vd::per_bin_adaptive_nested<3, 2>(8, VCU_HEUR_SIZE, VCU_METRIC_RELATIVE)
            .integrate(b, std::array<std::size_t, 2>{12, 8}, shell, r, log);
        print("shell_gpu", gpu);
        print("shell_oracle", oracle_nested<3, decltype(shell), float, orc::Simpson, orc::Trapezoidal, orc::MetricRel>(
                                  shell, {-0.1f, 0.0f, 0.0f}, {1.1f, 1.0f, 1.0f}, {12, 8}, 1, 1, 8));
    }
    /* 3. three channels: nested(boole, trapezoidal), 7 splits, 16x16 bins */
    {
        std::vector<std::array<float, 3>> px(16 * 16);
        auto b = [&](const std::array<std::size_t, 2>& q) -> std::array<float, 3>& { return px[q[1] * 16 + q[0]]; };
        const box<2> unit{{0.0f, 0.0f}, {1.0f, 1.0f}};
        vd::per_bin_adaptive_nested<5, 2>(7).integrate(b, std::array<std::size_t, 2>{16, 16}, Ramp{0.9f}, unit, log);
        std::vector<float> gpu;
        for (const auto& c : px) gpu.insert(gpu.end(), c.begin(), c.end());
        print("ramp_gpu", gpu);
        print("ramp_oracle", oracle_nested<2, Ramp, vrgb, orc::Boole, orc::Trapezoidal, orc::MetricAbs>(
                                 Ramp{0.9f}, {0.0f, 0.0f}, {1.0f, 1.0f}, {16, 16}, 0, 0, 7));
    }
    /* 4. per-bin Monte Carlo of the wave: 64 bins x 256 samples, seed 7 */
    {
        std::vector<float> gpu(64);
        auto b = [&](const std::array<std::size_t, 1>& q) -> float& { return gpu[q[0]]; };
        const box<2> unit{{0.0f, 0.0f}, {1.0f, 1.0f}};
        vd::per_bin_monte_carlo(256, 7).integrate(b, std::array<std::size_t, 1>{64}, UserWave{}, unit, log);
        print("wave_mc_gpu", gpu);
    }
    return 0;
}
#endif
