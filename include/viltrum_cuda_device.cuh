/*
 * viltrum_cuda_device.cuh -- CUDA per-bin integrators for a caller's OWN integrand functor
 * (header-only; compiled by nvcc in the caller's .cu translation unit).
 *
 * The C ABI of libviltrum_cuda.so (viltrum_cuda.h) selects built-in integrands by tag, because a
 * functor's code cannot cross a C ABI.  This header is the other route: it instantiates the
 * library's kernel templates -- the per-bin adaptive nested quadrature kernel
 * (viltrum_gb300/csrc/k_nested.cuh) and the per-bin Monte Carlo kernel (k_mc.cuh) -- for the
 * caller's functor inside the caller's own binary, so a viltrum user keeps their integrand and
 * swaps only the integrator:
 *
 *     #include "viltrum.h"
 *     #include "viltrum_cuda_device.cuh"
 *     struct Ring {   // trivially copyable, callable on host and device
 *         float r;
 *         __host__ __device__ float operator()(const std::array<float, 2>& x) const { ... }
 *     };
 *     viltrum::integrate(viltrum::cuda::device::per_bin_adaptive_nested<5, 3>(15), image, Ring{0.3f},
 *                        viltrum::range_primary<2>());
 *
 * Each type satisfies viltrum's Integrator concept (src/integrate.h:72-79) and replaces
 *   per_bin_adaptive_nested<SH, SL>  : integrator_per_bin_parallel(integrator_adaptive_iterations(
 *                                      nested(rule SH, rule SL), heuristic, iterations))
 *                                      (src/integrator-per-bin-parallel.h:17-35,
 *                                      src/nested/integrator-adaptive-iterations.h:12-30); ASSIGNS;
 *   per_bin_monte_carlo              : integrator_per_bin_parallel(monte_carlo(samples, seed))
 *                                      (src/monte-carlo/monte-carlo.h:39-63), Philox draws; ASSIGNS.
 * Rules by node count: 5 = boole, 3 = simpson, 2 = trapezoidal (pairs 5/3, 5/2, 3/2).
 *
 * Requirements on the functor F (compile with nvcc -std=c++17 --expt-relaxed-constexpr):
 *   - trivially copyable: it is passed to the kernel by value as a __grid_constant__ parameter;
 *   - callable on the device as f(std::array<float, DIM>) -- the form viltrum's detail::adapt
 *     passes through unchanged (src/integrate.h:13-16).  A functor taking DIM separate floats
 *     (the arities detail::adapt wraps in a host lambda, integrate.h:18-65) is passed as
 *     viltrum::cuda::device::arity<DIM>(f);
 *   - returning float or double (one channel) or an indexable value of 2..4 channels
 *     (std::array<float, 3>, ...).
 * The results follow the reference's algorithm exactly; they are bit-identical to the CPU path
 * wherever f returns the same bits on the host and on the device (correctly rounded operations,
 * no contraction into fused multiply-adds -- e.g. the __f*_rn intrinsics on the device and
 * -ffp-contract=off on the host, or vcu_integrands.h's vadd/vmul/vexp/vsin).
 * Failures throw viltrum::cuda::error; there is no CPU fallback.  Calls run on `stream` (default:
 * the legacy default stream) of the current device and return after the bins are written.
 */
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../viltrum_gb300/csrc/k_mc.cuh"
#include "../viltrum_gb300/csrc/k_nested.cuh"

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

namespace device {

/* f(x0, ..., x_{DIM-1}) presented as f(std::array<float, DIM>), callable on host and device */
template <int DIM, class F> struct arity_fn {
    F f;
    template <std::size_t... I>
    __host__ __device__ auto call(const std::array<float, DIM>& x, std::index_sequence<I...>) const {
        return f(x[I]...);
    }
    __host__ __device__ auto operator()(const std::array<float, DIM>& x) const {
        return call(x, std::make_index_sequence<DIM>{});
    }
};
template <int DIM, class F> arity_fn<DIM, F> arity(const F& f) { return arity_fn<DIM, F>{f}; }

namespace detail {

template <class V, class = void> struct channels_of {
    static constexpr int value = 1;
};
template <class V> struct channels_of<V, std::enable_if_t<!std::is_arithmetic_v<V>>> {
    static constexpr int value = (int)std::tuple_size<V>::value;
};

/* the caller's functor in the kernels' interface: DIM and CH members, operator()(const float*, float*) */
template <class F, int D> struct user_fn {
    using V = std::decay_t<decltype(std::declval<const F&>()(std::array<float, D>{}))>;
    static constexpr int DIM = D;
    static constexpr int CH = channels_of<V>::value;
    static_assert(CH >= 1 && CH <= 4, "integrand values have 1 to 4 channels");
    F f;
    __host__ __device__ void operator()(const float* x, float* out) const {
        std::array<float, D> a{};
        for (int i = 0; i < D; ++i) a[i] = x[i];
        const V v = f(a);
        if constexpr (std::is_arithmetic_v<V>) {
            out[0] = (float)v;
        } else {
            for (int c = 0; c < CH; ++c) out[c] = (float)v[c];
        }
    }
};

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw error(VCU_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
inline void check_status(int rc, const vcu_ctx& ctx) {
    if (rc != VCU_OK) throw error(rc, ctx.last_error.empty() ? std::string("status ") + std::to_string(rc)
                                                             : ctx.last_error);
}

/* one call's device state: the launch context the kernels read (device limits, stream, status
 * word) and the bins, released when the call ends */
struct call_state {
    vcu_ctx ctx;
    float* bins = nullptr;
    call_state(void* stream, std::size_t bin_floats) {
        check(cudaGetDevice(&ctx.device), "cudaGetDevice");
        int v = 0;
        check(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx.device), "cudaDeviceGetAttribute");
        ctx.sm_count = v;
        check(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.device),
              "cudaDeviceGetAttribute");
        ctx.smem_optin = (std::size_t)v;
        ctx.tune = 0;
        ctx.stream = static_cast<cudaStream_t>(stream);
        check(cudaMalloc(&ctx.d_status, 256), "cudaMalloc");
        check(cudaMemsetAsync(ctx.d_status, 0, 4, ctx.stream), "cudaMemsetAsync");
        check(cudaMalloc(&bins, bin_floats * 4 + 16), "cudaMalloc");
    }
    call_state(const call_state&) = delete;
    call_state& operator=(const call_state&) = delete;
    ~call_state() {
        if (bins) cudaFree(bins);
        if (ctx.d_status) cudaFree(ctx.d_status);
    }
    /* copy the bins back; VCU_NAN_DETECTED if a kernel saw a NaN */
    void finish(std::vector<float>& out) {
        uint32_t flags = 0;
        check(cudaMemcpyAsync(out.data(), bins, out.size() * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
        check(cudaMemcpyAsync(&flags, ctx.d_status, 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(ctx.stream), "cudaStreamSynchronize");
        if (flags & VCU_FLAG_NAN) throw error(VCU_NAN_DETECTED, "the integrand produced NaN in a bin");
    }
};

template <class R> constexpr int range_dim() { return (int)R::size; }

template <std::size_t DIMBINS, class R>
vcu_problem make_problem(const std::array<std::size_t, DIMBINS>& res, const R& range) {
    constexpr int DIM = range_dim<R>();
    static_assert(DIMBINS >= 1 && DIMBINS <= VCU_MAX_DIMBINS, "1..4 binned dimensions");
    static_assert(DIM >= (int)DIMBINS && DIM <= VCU_MAX_DIM, "range dimension must be DIMBINS..6");
    vcu_problem p{};
    p.dim = DIM;
    p.dimbins = (int32_t)DIMBINS;
    for (int d = 0; d < DIM; ++d) {
        p.range_min[d] = (float)range.min(d);
        p.range_max[d] = (float)range.max(d);
    }
    for (std::size_t d = 0; d < DIMBINS; ++d) p.resolution[d] = res[d];
    p.mem = VCU_MEM_DEVICE;
    return p;
}

/* bins(pos) = value, in viltrum's multidimensional_range order (dim 0 fastest) */
template <class T> void store(T& dst, const float* v, int ch) {
    if constexpr (std::is_arithmetic_v<T>) {
        dst = v[0];
    } else {
        for (int c = 0; c < ch; ++c) dst[c] = v[c];
    }
}
template <class Bins, std::size_t DIMBINS>
void write_back(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const std::vector<float>& out, int ch) {
    std::array<std::size_t, DIMBINS> pos{};
    const std::size_t n = out.size() / ch;
    for (std::size_t lin = 0; lin < n; ++lin) {
        store(bins(pos), &out[lin * ch], ch);
        for (std::size_t d = 0; d < DIMBINS; ++d) {
            if (++pos[d] < res[d]) break;
            pos[d] = 0;
        }
    }
}

}  // namespace detail

/* integrator_per_bin_parallel(integrator_adaptive_iterations(nested(SH, SL), heuristic, iterations))
 * for a caller's functor.  heuristic: VCU_HEUR_DEFAULT or VCU_HEUR_SIZE (size_weight, min_size);
 * metric: VCU_METRIC_ABSOLUTE or VCU_METRIC_RELATIVE (min_val).  Regions up to 125 nodes (Boole to
 * 3-D, Simpson to 4-D), at most 62 splits per bin. */
template <int SH = 5, int SL = 3> class per_bin_adaptive_nested {
    static_assert((SH == 5 && (SL == 3 || SL == 2)) || (SH == 3 && SL == 2),
                  "rule pairs: boole/simpson, boole/trapezoidal, simpson/trapezoidal");
    unsigned long iterations_;
    vcu_nested nested_;
    void* stream_;

public:
    explicit per_bin_adaptive_nested(unsigned long iterations, int heuristic = VCU_HEUR_DEFAULT,
                                     int metric = VCU_METRIC_ABSOLUTE, double size_weight = 1e-5,
                                     double min_size = 1e-37, double min_val = 1e-37, void* stream = nullptr)
        : iterations_(iterations), nested_{SH, SL, heuristic, metric, size_weight, min_size, min_val}, stream_(stream) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        constexpr int DIM = detail::range_dim<R>();
        static_assert(std::is_trivially_copyable_v<F>, "the integrand functor must be trivially copyable");
        static_assert(vcu::ipow(SH, DIM) <= 125, "per-bin nested regions are limited to 125 nodes (S^DIM)");
        using U = detail::user_fn<F, DIM>;
        if (iterations_ > 62) throw error(VCU_UNSUPPORTED, "per-bin region budget is limited to 62 splits");
        logger.log_progress(std::size_t(0), std::size_t(1));
        const vcu_problem p = detail::make_problem(res, range);
        vcu::BinGrid g;
        std::size_t nbins = 1;
        for (auto r : res) nbins *= r;
        detail::call_state s(stream_, nbins * U::CH);
        detail::check_status(vcu::make_grid(&s.ctx, &p, g), s.ctx);
        detail::check_status(vcu::check_per_bin_nested(&s.ctx, nested_), s.ctx);
        uint32_t launches = 0;
        detail::check_status(vcu::nc_detail::launch<DIM, SH, SL>(&s.ctx, U{f}, g, nested_, (int)iterations_, s.bins,
                                                                 nullptr, launches),
                             s.ctx);
        std::vector<float> out(nbins * U::CH);
        s.finish(out);
        detail::write_back(bins, res, out, U::CH);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

/* integrator_per_bin_parallel(monte_carlo(samples, seed)) for a caller's functor: sample j of bin b
 * draws Philox4x32-10 with key = seed and counter (j, b, block), like vcu_per_bin_monte_carlo */
class per_bin_monte_carlo {
    unsigned long samples_;
    std::uint64_t seed_;
    void* stream_;

public:
    per_bin_monte_carlo(unsigned long samples, std::uint64_t seed, void* stream = nullptr)
        : samples_(samples), seed_(seed), stream_(stream) {}

    template <class Bins, std::size_t DIMBINS, class F, class R, class Logger>
    void integrate(Bins& bins, const std::array<std::size_t, DIMBINS>& res, const F& f, const R& range,
                   Logger& logger) const {
        constexpr int DIM = detail::range_dim<R>();
        static_assert(std::is_trivially_copyable_v<F>, "the integrand functor must be trivially copyable");
        using U = detail::user_fn<F, DIM>;
        if (samples_ == 0 || samples_ > 0xffffffffull) throw error(VCU_INVALID_ARG, "samples per bin must be 1..2^32-1");
        logger.log_progress(std::size_t(0), std::size_t(1));
        const vcu_problem p = detail::make_problem(res, range);
        vcu::BinGrid g;
        std::size_t nbins = 1;
        for (auto r : res) nbins *= r;
        detail::call_state s(stream_, nbins * U::CH);
        detail::check_status(vcu::make_grid(&s.ctx, &p, g), s.ctx);
        using namespace vcu::mc_detail;
        const unsigned blocks = (unsigned)((g.nbins + MC_WARPS - 1) / MC_WARPS);
        k_per_bin_mc<U, DIM, false, false><<<blocks, MC_WARPS * 32, 0, s.ctx.stream>>>(
            U{f}, g, (uint64_t)samples_, (uint32_t)seed_, (uint32_t)(seed_ >> 32), nullptr, s.bins, s.ctx.d_status,
            1.0f);
        detail::check(cudaGetLastError(), "k_per_bin_mc launch");
        std::vector<float> out(nbins * U::CH);
        s.finish(out);
        detail::write_back(bins, res, out, U::CH);
        logger.log_progress(std::size_t(1), std::size_t(1));
    }
};

}  // namespace device
}  // namespace cuda
}  // namespace viltrum
