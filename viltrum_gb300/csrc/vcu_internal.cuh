/*
 * vcu_internal.cuh -- runtime shared by the translation units of libviltrum_cuda.so:
 * the context (stream, grow-only device buffers, status word, timing events), error plumbing,
 * the Philox4x32-10 counter generator and the integrand dispatcher.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/vcu_integrands.h"
#include "../../include/viltrum_cuda.h"

/* status bits written by kernels into the context's status word */
#define VCU_FLAG_NAN 1u
#define VCU_FLAG_TIMEOUT 2u
#define VCU_FLAG_OVERFLOW 4u

struct vcu_buffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

/* autotuner cache entry: launch configuration chosen for one kernel configuration */
struct vcu_tuned {
    uint64_t key;
    int32_t value;
};

namespace vcu {
namespace batch {
/* configuration of the batched-integral kernel shared by all its items */
struct Cfg {
    int32_t n_items;
    int32_t heuristic, relative;
    float min_val_f;
    double size_weight, min_size;
    int32_t hcap; /* heap elements kept in shared memory (odd) */
    int32_t pad;
};
}  // namespace batch
}  // namespace vcu

/* device state of the batch last uploaded on a context: the kernel, its launch shape, the
 * captured graph (queue reset + persistent launch) and the buffers it reads and writes */
struct vcu_batch_state {
    bool valid = false;
    int kind = 0, sh = 0, sl = 0;
    uint64_t n = 0;
    vcu::batch::Cfg cfg{};
    void* kernel = nullptr;
    size_t smem = 0;
    unsigned blocks = 0;
    int threads = 0;
    uint64_t evaluations = 0, regions = 0;
    char *items = nullptr, *functors = nullptr, *vals = nullptr, *ranges = nullptr, *vols = nullptr, *heap = nullptr;
    float* results = nullptr;
    uint64_t* item_ns = nullptr;
    uint32_t* queue = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct vcu_ctx {
    int device = 0;
    int tune = 1;                 /* time launch-configuration candidates on first use */
    vcu_tuned tuned[32] = {};     /* fixed-size autotuner cache (no allocation)         */
    int ntuned = 0;
    cudaEvent_t ev_tune[2] = {nullptr, nullptr};
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaStream_t copy_stream = nullptr; /* device-to-host copies that overlap the main stream's work */
    cudaEvent_t ev_snap = nullptr;      /* orders them after the main stream's snapshot */
    uint32_t* d_status = nullptr; /* one word of device status flags */
    vcu_buffer out, aux, in, scratch;
    vcu_buffer batch_in, batch_pool; /* owned by the batched-integral path only */
    vcu_batch_state batch;
    size_t held = 0;              /* bytes held by the grow-only buffers                 */
    uint64_t mem_limit = 0;       /* vcu_set_device_memory_limit (0: none)               */
    std::string last_error;
};

namespace vcu {

inline int fail(vcu_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}
inline int cuda_fail(vcu_ctx* ctx, cudaError_t e, const char* where) {
    return fail(ctx, VCU_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}
#define VCU_CUDA(ctx, call)                                      \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return vcu::cuda_fail(ctx, e_, #call); \
    } while (0)

/* grow-only device buffer owned by the context; a growth that would take the context's buffers
 * past its memory limit fails with VCU_OOM before anything is freed or allocated */
inline int ensure(vcu_ctx* ctx, vcu_buffer& b, size_t bytes) {
    if (b.bytes >= bytes) return VCU_OK;
    if (ctx && ctx->mem_limit && ctx->held - b.bytes + bytes > ctx->mem_limit)
        return fail(ctx, VCU_OOM, std::string("device allocation of ") + std::to_string(bytes) +
                                      " bytes would exceed the context's memory limit of " +
                                      std::to_string(ctx->mem_limit) + " bytes");
    if (b.ptr) cudaFree(b.ptr);
    if (ctx) ctx->held -= b.bytes;
    b.ptr = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes < 256 ? 256 : bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return fail(ctx, VCU_OOM, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed");
    }
    b.bytes = bytes;
    if (ctx) ctx->held += bytes;
    return VCU_OK;
}

/* Problem geometry shared by the per-bin kernels (plain data, passed by value). */
struct BinGrid {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
    float drange[VCU_MAX_DIMBINS]; /* (max-min)/float(res), float arithmetic */
    uint32_t res[VCU_MAX_DIMBINS];
    int32_t dim, dimbins;
    uint64_t nbins;
    float factor; /* prod(res) as float (exact below 2^24) */
};

/* the bin grid of a problem, with viltrum's float arithmetic for the bin widths */
inline int make_grid(vcu_ctx* ctx, const vcu_problem* p, BinGrid& g) {
    if (!p) return fail(ctx, VCU_INVALID_ARG, "null problem");
    if (p->dim < 1 || p->dim > VCU_MAX_DIM) return fail(ctx, VCU_INVALID_ARG, "dim must be 1..6");
    if (p->dimbins < 1 || p->dimbins > VCU_MAX_DIMBINS || p->dimbins > p->dim)
        return fail(ctx, VCU_INVALID_ARG, "dimbins must be 1..min(dim,4)");
    if (p->mem != VCU_MEM_HOST && p->mem != VCU_MEM_DEVICE) return fail(ctx, VCU_INVALID_ARG, "mem must be host or device");
    std::memset(&g, 0, sizeof(g));
    g.dim = p->dim;
    g.dimbins = p->dimbins;
    for (int d = 0; d < p->dim; ++d) {
        if (!std::isfinite(p->range_min[d]) || !std::isfinite(p->range_max[d]))
            return fail(ctx, VCU_INVALID_ARG, "range bounds must be finite");
        g.rmin[d] = p->range_min[d];
        g.rmax[d] = p->range_max[d];
    }
    uint64_t nb = 1;
    double prod = 1.0;
    for (int d = 0; d < p->dimbins; ++d) {
        const uint64_t r = p->resolution[d];
        if (r == 0 || r > 0xffffffffull) return fail(ctx, VCU_INVALID_ARG, "resolution must be 1..2^32-1");
        if (nb > (1ull << 40) / r) return fail(ctx, VCU_INVALID_ARG, "too many bins");
        nb *= r;
        prod *= (double)r;
        g.res[d] = (uint32_t)r;
        /* (range.max(i) - range.min(i)) / Float(res[i]) in float (integrator-per-bin-parallel.h:22) */
        volatile float w = p->range_max[d] - p->range_min[d];
        g.drange[d] = w / (float)r;
    }
    g.nbins = nb;
    g.factor = (float)prod;
    return VCU_OK;
}
/* VCU_INVALID_ARG unless heuristic, metric and rule pair are ones the per-bin nested kernels
 * instantiate (boole/simpson, boole/trapezoidal, simpson/trapezoidal) */
inline int check_per_bin_nested(vcu_ctx* ctx, const vcu_nested& n) {
    if (n.heuristic != VCU_HEUR_DEFAULT && n.heuristic != VCU_HEUR_SIZE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error heuristic");
    if (n.metric != VCU_METRIC_ABSOLUTE && n.metric != VCU_METRIC_RELATIVE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error metric");
    const bool pair = (n.rule_hi == VCU_RULE_BOOLE && n.rule_lo == VCU_RULE_SIMPSON) ||
                      (n.rule_hi == VCU_RULE_BOOLE && n.rule_lo == VCU_RULE_TRAPEZOIDAL) ||
                      (n.rule_hi == VCU_RULE_SIMPSON && n.rule_lo == VCU_RULE_TRAPEZOIDAL);
    if (!pair)
        return fail(ctx, VCU_INVALID_ARG,
                    "unsupported nested rule pair (boole/simpson, boole/trapezoidal, simpson/trapezoidal)");
    return VCU_OK;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the multiply-xor bijection
 * with the published multipliers and Weyl key increments. */
struct U4 {
    uint32_t x, y, z, w;
};
__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
/* top 24 bits -> float in [0,1), exact */
__device__ __forceinline__ float u01(uint32_t r) { return (float)(r >> 8) * 5.9604644775390625e-08f; }

/* fn(integral_constant<int, 0>), ..., fn(integral_constant<int, N-1>): loops whose index must be a
 * compile-time constant (strides, divisors) */
template <class Fn, int... I>
__device__ __forceinline__ void static_for_impl(Fn& fn, std::integer_sequence<int, I...>) {
    (fn(std::integral_constant<int, I>{}), ...);
}
template <int N, class Fn> __device__ __forceinline__ void static_for(Fn fn) {
    static_for_impl(fn, std::make_integer_sequence<int, N>{});
}

/* integrands that evaluate two points at once (two independent dependency chains per lane) */
template <class F, class = void> struct has_pair : std::false_type {};
template <class F>
struct has_pair<F, std::void_t<decltype(std::declval<const F&>().pair((const float*)nullptr, (const float*)nullptr,
                                                                        (float*)nullptr, (float*)nullptr))>>
    : std::true_type {};

/* integrands of unbounded dimension (a kUnbounded member): their first DIM coordinates come from
 * the integrator, the rest from a stream the functor draws itself */
template <class F, class = void> struct is_unbounded : std::false_type {};
template <class F> struct is_unbounded<F, std::void_t<decltype(F::kUnbounded)>> : std::bool_constant<F::kUnbounded> {};

/* integrands that evaluate N points at once (multi<N>: N independent dependency chains per lane) */
template <class F, class = void> struct has_multi : std::false_type {};
template <class F>
struct has_multi<F, std::void_t<decltype(std::declval<const F&>().template multi<2>(
                        (const float(*)[F::DIM]) nullptr, (float(*)[F::CH]) nullptr))>> : std::true_type {};

/* integrands that can list the terms that may be non-zero in a box (cull) and evaluate only those
 * (multi_cull<N>), bit for bit what multi<N> returns at any point of the box */
template <class F, class = void> struct has_cull : std::false_type {};
template <class F>
struct has_cull<F, std::void_t<typename F::Cull,
                               decltype(std::declval<const F&>().cull((const float*)nullptr, (const float*)nullptr))>>
    : std::true_type {};

/* integrands whose cull decision splits into independent per-term tests (cull_prepare: the box
 * the tests read; cull_keep(t): term t of the mask's kCullWords 32-bit words; cull_from_words),
 * so that the lanes of a group can share the terms */
template <class F, class = void> struct has_cull_terms : std::false_type {};
template <class F>
struct has_cull_terms<F, std::void_t<decltype(F::kCullWords), decltype(F::kCullBox),
                                     decltype(std::declval<const F&>().cull_keep(0, (const float*)nullptr)),
                                     decltype(F::cull_from_words((const uint32_t*)nullptr))>> : std::true_type {};

/* integrands that list the terms that can be non-zero over a box of their coordinates (cull_box,
 * lo/hi of F::DIM entries) and evaluate with only those -- two points (pair_culled) or one
 * (eval_culled) -- bit for bit what pair() / operator() return at points of the box: the per-bin
 * Monte Carlo, learned residual and control-variate residual kernels cull once per warp (one bin) */
template <class F, class = void> struct has_cull_box : std::false_type {};
template <class F>
struct has_cull_box<F, std::void_t<typename F::CullBox,
                                   decltype(std::declval<const F&>().cull_box((const float*)nullptr,
                                                                                (const float*)nullptr))>>
    : std::true_type {};
template <class F, class = void> struct has_pair_cull : std::false_type {};
template <class F>
struct has_pair_cull<F, std::void_t<decltype(std::declval<const F&>().pair_culled(
                            std::declval<const typename F::CullBox&>(), (const float*)nullptr, (const float*)nullptr,
                            (float*)nullptr, (float*)nullptr))>> : std::true_type {};
template <class F, class = void> struct has_eval_cull : std::false_type {};
template <class F>
struct has_eval_cull<F, std::void_t<decltype(std::declval<const F&>().eval_culled(
                            std::declval<const typename F::CullBox&>(), (const float*)nullptr, (float*)nullptr))>>
    : std::true_type {};

template <class F, bool = has_cull_box<F>::value> struct cull_box_of { using type = int; };
template <class F> struct cull_box_of<F, true> { using type = typename F::CullBox; };

/* Calls v(functor, channels) with the built-in functor selected by kind.  The functor object is
 * built on the host (vcu_integrands.h build()); its size decides the kernel parameter size. */
template <class V> int with_integrand(vcu_ctx* ctx, const vcu_integrand& f, int dim, V&& v) {
    switch (f.kind) {
    case VCU_F_POLY2: {
        if (dim != 2) break;
        Poly2 fn{};
        return v(fn);
    }
    case VCU_F_SIN1: {
        if (dim != 1) break;
        Sin1 fn{};
        return v(fn);
    }
    case VCU_F_SPHERE3: {
        if (dim != 3) break;
        Sphere3 fn{};
        return v(fn);
    }
    case VCU_F_WAVE2: {
        if (dim != 2) break;
        Wave2 fn{};
        return v(fn);
    }
    case VCU_F_SCENE2: {
        if (dim != 2) break;
        Scene2 fn{};
        if (fn.build(f.params, f.n_params)) return fail(ctx, VCU_INVALID_ARG, "bad scene parameters");
        return v(fn);
    }
    case VCU_F_MOVING_SCENE3: {
        if (dim != 3) break;
        MovingScene3 fn{};
        if (fn.build(f.params, f.n_params)) return fail(ctx, VCU_INVALID_ARG, "bad moving-scene parameters");
        return v(fn);
    }
    case VCU_F_HALFSPACE: {
        Halfspace fn{};
        if (fn.build(f.params, f.n_params)) return fail(ctx, VCU_INVALID_ARG, "bad half-space parameters");
        if (fn.dim != dim) break;
        return v(fn);
    }
    case VCU_F_WALK2: {
        if (dim != 2) break;
        static thread_local Walk2 fn;
        if (fn.build(f.params, f.n_params)) return fail(ctx, VCU_INVALID_ARG, "bad walk parameters");
        return v(fn);
    }
    case VCU_F_OCCLUDED_SCENE5: {
        if (dim != 5) break;
        /* ~5 KB: keep it off the host stack of deep call chains */
        static thread_local OccludedScene5 fn;
        if (fn.build(f.params, f.n_params)) return fail(ctx, VCU_INVALID_ARG, "bad occluded-scene parameters");
        return v(fn);
    }
    default:
        return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind " + std::to_string(f.kind));
    }
    return fail(ctx, VCU_INVALID_ARG,
                "integrand kind " + std::to_string(f.kind) + " does not take dimension " + std::to_string(dim));
}

/* timing + status helpers around a call */
struct CallScope {
    vcu_ctx* ctx;
    vcu_stats* stats;
    uint32_t launches = 0;
    int begin();
    int end(uint64_t evaluations, uint64_t regions);
};

}  // namespace vcu

/* entry points implemented by the method translation units */
namespace vcu {
int run_mc(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, uint64_t spp, uint64_t seed, const float* points,
           float* d_bins, bool accumulate, uint32_t& launches);
int run_nested_bs(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                  float* d_bins, int32_t* d_trace, uint32_t& launches);
int run_nested_bt(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                  float* d_bins, int32_t* d_trace, uint32_t& launches);
int run_nested_st(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                  float* d_bins, int32_t* d_trace, uint32_t& launches);
int run_eval(vcu_ctx* ctx, const vcu_integrand& f, int dim, const float* d_x, int64_t npts, float* d_out,
             uint32_t& launches);
int run_learned(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_learned& opt, float* d_bins,
                float* d_integral, vcu_learned_report* report, uint32_t& launches);
/* pilot samples per bin of the learned control variate's per-bin choice */
inline uint64_t learned_pilot(uint64_t spp, uint32_t pilot) {
    if (pilot) return pilot;
    const uint64_t p = spp / 8;
    return p < 8 ? 8 : (p > 256 ? 256 : p);
}
int run_mlp_eval(vcu_ctx* ctx, int dim, const float* theta, const float* u, const float* y, int64_t npts, float* out,
                 float* grad, uint32_t& launches);
int run_batch_st(vcu_ctx* ctx, int kind, const vcu_nested& n, const vcu_batch_item* items, uint64_t count,
                 uint32_t& launches);
int run_batch_bs(vcu_ctx* ctx, int kind, const vcu_nested& n, const vcu_batch_item* items, uint64_t count,
                 uint32_t& launches);
int run_batch_bt(vcu_ctx* ctx, int kind, const vcu_nested& n, const vcu_batch_item* items, uint64_t count,
                 uint32_t& launches);
/* (re)capture the batch's queue reset + launch as a graph and launch it; launch it again */
int batch_capture(vcu_ctx* ctx, uint32_t& launches);
int batch_launch(vcu_ctx* ctx, uint32_t& launches);
int run_tol_st(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, float tol,
               uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches);
int run_tol_bs(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, float tol,
               uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches);
int run_tol_bt(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, float tol,
               uint64_t max_regions, float* d_bins, uint64_t& nregions, uint64_t& nleaves, uint32_t& launches);
int run_cv_st(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
              const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
              uint32_t& launches);
int run_cv_fubini(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
                  const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
                  uint32_t& launches);
int run_cv_bs(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
              const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
              uint32_t& launches);
int run_cv_bt(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_nested& n, int iterations,
              const vcu_cv& cv, const float* d_replay, float* d_bins, float* d_approx, float* d_regions,
              uint32_t& launches);
}  // namespace vcu
