/*
 * viltrum_cuda.h -- C ABI of libviltrum_cuda.so, the GB300 (sm_103a) per-bin integration path of
 * viltrum.
 *
 * In viltrum every integrator is a value type whose
 *     template<class Bins, size_t DIMBINS, class F, class Float, size_t DIM, class Logger>
 *     void integrate(Bins& bins, const std::array<size_t,DIMBINS>& resolution, const F& f,
 *                    const Range<Float,DIM>& range, Logger& logger) const;
 * is called by viltrum::integrate (src/integrate.h:72-79).  Each entry point below replaces one
 * such call for one family of per-bin integrators; the header-side integrator types of
 * viltrum_cuda.hpp (and the Python package viltrum_gb300) turn the bins/resolution/functor/range
 * arguments into a vcu_problem, call the entry point, and write the result back through the
 * caller's bins(pos) accessor with the assign/accumulate semantics of the integrator replaced.
 *
 * Conventions
 *   - Bins are returned as floats, dim-0-fastest (the order of viltrum's
 *     multidimensional_range, src/multidimensional-range.h:33-40), channels interleaved:
 *     bins[linear_bin * channels + c].  Bin values use viltrum's normalisation,
 *     (prod of the resolution) x integral over the bin (src/integrator-per-bin.h:26).
 *   - Pointers are host pointers when vcu_problem::mem is VCU_MEM_HOST (the library copies
 *     through its own device buffers) and device pointers when it is VCU_MEM_DEVICE.
 *   - Every call returns a vcu_status; no exception crosses the ABI.  vcu_last_error() gives the
 *     message of the last failure on a context.
 *   - A context owns one CUDA stream and its device buffers; calls on one context must not
 *     overlap (one context per host thread).  All calls are synchronous with respect to the
 *     host: they return after the results are written.
 *   - Integrands are the built-in functors of vcu_integrands.h selected by tag (a functor's
 *     code cannot cross a C ABI); the parameters are copied into the kernel launch.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VCU_ABI_VERSION 2
#define VCU_MAX_DIM 6     /* viltrum's VILTRUM_MAX_DIMENSIONS_REGION (src/newton-cotes/region.h:16-18) */
#define VCU_MAX_DIMBINS 4

typedef enum vcu_status {
    VCU_OK = 0,
    VCU_INVALID_ARG = 1,
    VCU_OOM = 2,
    VCU_QUEUE_OVERFLOW = 3,
    VCU_DEVICE_TIMEOUT = 4, /* a bounded device-side wait expired                    */
    VCU_NAN_DETECTED = 5,   /* the integrand produced NaN in at least one bin        */
    VCU_CUDA_ERROR = 6,
    VCU_NO_DEVICE = 7,
    VCU_UNSUPPORTED = 8     /* valid request outside what this build instantiates    */
} vcu_status;

enum { VCU_MEM_HOST = 0, VCU_MEM_DEVICE = 1 };
/* Newton-Cotes rules by node count (src/newton-cotes/rules.h): trapezoidal, simpson, boole */
enum { VCU_RULE_TRAPEZOIDAL = 2, VCU_RULE_SIMPSON = 3, VCU_RULE_BOOLE = 5 };
/* error heuristics (src/nested/error-heuristic.h) and metrics (src/nested/error-metric.h) */
enum { VCU_HEUR_DEFAULT = 0, VCU_HEUR_SIZE = 1 };
enum { VCU_METRIC_ABSOLUTE = 0, VCU_METRIC_RELATIVE = 1 };
/* control-variate weights (src/control-variates/weight-strategy.h) */
enum { VCU_CV_OPTIMIZE = 0, VCU_CV_FIXED = 1 };
/* residual region choice (src/control-variates/region-russian-roulette.h): rr_uniform_region,
 * rr_integral_region, rr_error_region (NormDefault) */
enum { VCU_RR_UNIFORM = 0, VCU_RR_INTEGRAL = 1, VCU_RR_ERROR = 2, VCU_RR_PDF = 3 };
/* residual point sampling in bin n region (src/control-variates/region-sampling.h):
 * region_sampling_uniform, region_sampling_importance, region_sampling_russian_roulette,
 * region_sampling_mis (NormDefault) */
enum { VCU_RS_UNIFORM = 0, VCU_RS_IMPORTANCE = 1, VCU_RS_RUSSIAN_ROULETTE = 2, VCU_RS_MIS = 3 };

typedef struct vcu_ctx vcu_ctx;

typedef struct vcu_opts {
    int32_t device;   /* CUDA device ordinal                                        */
    int32_t flags;    /* reserved, 0                                               */
    void* stream;     /* cudaStream_t to run on, or NULL for a stream of the context */
} vcu_opts;

typedef struct vcu_integrand {
    int32_t kind;          /* VCU_F_* of vcu_integrands.h          */
    int32_t n_params;      /* number of floats in params            */
    const float* params;   /* host pointer, may be NULL if n_params==0 */
} vcu_integrand;

typedef struct vcu_problem {
    vcu_integrand f;
    int32_t dim;                         /* dimension of the integration range      */
    int32_t dimbins;                     /* leading dimensions that are binned      */
    float range_min[VCU_MAX_DIM];
    float range_max[VCU_MAX_DIM];
    uint64_t resolution[VCU_MAX_DIMBINS];
    int32_t mem;                         /* VCU_MEM_HOST or VCU_MEM_DEVICE          */
    int32_t reserved;
} vcu_problem;

typedef struct vcu_nested {
    int32_t rule_hi, rule_lo;  /* Nested<H,L> (src/nested/nested.h:7-34)                     */
    int32_t heuristic, metric; /* VCU_HEUR_*, VCU_METRIC_*                                   */
    double size_weight;        /* error_heuristic_size weight, 1e-5 (error-heuristic.h:129) */
    double min_size;           /* error_heuristic_size minimum size, 1e-37                  */
    double min_val;            /* error_metric_relative minimum value, 1e-37 (error-metric.h:79) */
} vcu_nested;

typedef struct vcu_stats {
    double device_ms;          /* device time of the call's kernels (CUDA events)     */
    uint64_t evaluations;      /* integrand evaluations performed                      */
    uint64_t regions;          /* regions built (adaptive methods)                     */
    uint32_t kernel_launches;  /* kernels of this library launched by the call         */
    uint32_t flags;            /* device status bits (1: NaN seen, 2: timeout, 4: overflow) */
} vcu_stats;

/* ------------------------------------------------------------------ context */
int vcu_abi_version(void);
int vcu_create(vcu_ctx** ctx, const vcu_opts* opts);
int vcu_destroy(vcu_ctx* ctx);
int vcu_last_error(const vcu_ctx* ctx, char* buf, size_t len);
/* No reference counterpart (viltrum allocates with std::vector and has no budget).  A context grows
 * its device buffers on demand and keeps them; with a limit set, a call whose buffers would take
 * the context past `bytes` in total returns VCU_OOM (before freeing or allocating anything) and
 * the context stays usable.  0 removes the limit.  vcu_device_memory_held() returns the bytes the
 * context's buffers hold now. */
int vcu_set_device_memory_limit(vcu_ctx* ctx, uint64_t bytes);
uint64_t vcu_device_memory_held(const vcu_ctx* ctx);
/* value channels of a built-in integrand (1 or 3), or a negative vcu_status */
int vcu_channels(int32_t kind);

/* Device evaluation of a built-in integrand at npts points (row-major npts x dim); out receives
 * npts x channels floats.  Pointers follow mem.  No reference counterpart: it exposes the
 * device functor so callers can check it against a host evaluation of the same functor. */
int vcu_eval(vcu_ctx* ctx, const vcu_integrand* f, int32_t dim, const float* x, int64_t npts,
             float* out, int32_t mem);

/* ------------------------------------------------------------------ per-bin Monte Carlo
 * Replaces integrator_per_bin_parallel(monte_carlo(samples, seed))
 * (src/integrator-per-bin-parallel.h:17-35 with src/monte-carlo/monte-carlo.h:39-63) and
 * monte_carlo_per_bin_parallel(samples, seed) (src/monte-carlo/monte-carlo-per-bin-parallel.h:40-71).
 * Sample j of bin b draws its coordinates from Philox4x32-10 with key = seed and counter
 * (j, b_lo, b_hi, block), in place of the reference's per-bin std::mt19937 copies.
 * bins receives the per-bin estimate (prod(res) x volume(bin)/samples x sum f).            */
int vcu_per_bin_monte_carlo(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin,
                            uint64_t seed, float* bins, vcu_stats* stats);

/* Same estimator over caller-supplied sample points (bin-major, then sample, then coordinate:
 * nbins x samples x dim floats), e.g. the points the reference drew for the same call. */
int vcu_per_bin_monte_carlo_replay(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin,
                                   const float* points, float* bins, vcu_stats* stats);

/* Replaces monte_carlo_per_bin_parallel(samples, seed)
 * (src/monte-carlo/monte-carlo-per-bin-parallel.h:40-71) with its own arithmetic: bins ACCUMULATE,
 * bins[b] += volume(range)/samples x sum f over the bin's samples (the factor of :45, the += of
 * :69; the reference rounds to float after every sample, this adds the compensated sum once).
 * bins is read and written (follows mem).  points (nullable, same layout as the replay call's)
 * replaces the Philox draws, e.g. by the points the reference drew. */
int vcu_per_bin_monte_carlo_accumulate(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin,
                                       uint64_t seed, const float* points, float* bins, vcu_stats* stats);

/* ------------------------------------------------------------------ per-bin adaptive nested NC
 * Replaces integrator_per_bin_parallel(integrator_adaptive_iterations(nested(H,L), heuristic,
 * iterations)) (src/nested/integrator-adaptive-iterations.h:12-30,
 * src/nested/regions-generator-adaptive-heap.h:18-45,
 * src/newton-cotes/regions-integrator-sequential.h:37-58): per bin, a max-error heap of
 * regions is split `iterations` times and the iterations+1 regions are integrated into the bin.
 * trace (nullable, follows mem) receives per bin and iteration (split dimension, float bits of
 * the popped region's error): nbins x iterations x 2 int32.                                 */
int vcu_per_bin_adaptive_nested(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested,
                                uint64_t iterations, float* bins, int32_t* trace,
                                vcu_stats* stats);

/* ------------------------------------------------------------------ control variates
 * Replaces integrator_region_based(regions_generator_adaptive_heap(nested(H,L), heuristic, iterations),
 * regions_integrator_parallel_variance_reduction(rr, cv_optimize_weight() or cv_fixed_weight(alpha),
 * region_sampling_uniform(), std::mt19937(seed), samples)) with rr one of rr_uniform_region(),
 * rr_integral_region(), rr_error_region() (region-russian-roulette.h:9-108)
 * (src/control-variates/regions-integrator-parallel-variance-reduction.h:32-109,
 * src/control-variates/integrator-crespo2021.h:7-22 for nested(simpson,trapezoidal) with
 * error_heuristic_size(error_metric_relative(), 1e-5)): one max-error heap of regions over the whole
 * range (iterations splits), per-bin lists of the regions overlapping each bin, the polynomial
 * integral over bin n region as control variate, and `samples` residual samples per bin
 * (region chosen uniformly, or with probability proportional to |integral over bin n region|, to
 * |region error| x its share of volume in the bin, or to the integral of the region's pdf over bin
 * n region, floored at 1% (rr_factor) of the mean weight; point uniform in bin n region or drawn
 * from the pdf of the region's polynomial -- Simpson high rule only).  The result is ASSIGNED to the
 * bins.  With fubini_dims = 2 (nested(simpson, trapezoidal), integrands of 3+ dimensions, at most 2
 * binned): integrator_crespo2021_infinite<2> / integrator_adaptive_fubini_variance_reduction_parallel<2>
 * (integrator-crespo2021.h:24-44, integrator-adaptive-fubini-variance-reduction.h:28-41): the regions
 * span dimensions 0-1 and every evaluation integrates the others by Monte Carlo (tail_samples Philox
 * points for the region nodes, one for a residual sample); replay records and region ranges then
 * have 2 coordinates.
 * Residual sample j of bin b draws from Philox4x32-10 unless `replay` is given: nbins x samples x
 * vcu_cv_replay_width(dim, sampling) floats (index of the chosen region in the bin's list, then the
 * point, ...), e.g. the reference's own draws.  approximation (nullable) receives the
 * control-variate integral per bin, regions (nullable) the (iterations+1) x (min[dim], max[dim])
 * region ranges in heap order.  All
 * pointers follow p->mem. */
typedef struct vcu_cv {
    uint64_t samples_per_bin; /* residual samples per bin (spp)                         */
    uint64_t seed;            /* Philox key                                             */
    int32_t weight;           /* VCU_CV_OPTIMIZE or VCU_CV_FIXED                        */
    int32_t reserved;         /* 0                                                      */
    double alpha;             /* cv_fixed_weight's alpha                                */
    int32_t rr;               /* VCU_RR_UNIFORM, _INTEGRAL, _ERROR or _PDF              */
    int32_t sampling;         /* VCU_RS_UNIFORM, _IMPORTANCE, _RUSSIAN_ROULETTE or _MIS */
    float rr_factor;          /* VCU_RR_PDF: rr_pdf_region's factor_prob (0.01f there) */
    int32_t reserved2;        /* 0                                                      */
    double mis_power;         /* VCU_RS_MIS: region_sampling_mis(power, cutoff)        */
    double mis_cutoff;
    int32_t fubini_dims;      /* 0, or 2: regions over the first 2 dimensions only     */
    uint32_t tail_samples;    /* fubini_dims 2: Monte Carlo samples per evaluation     */
    float* variance;          /* nullable (follows mem): per bin, the estimated variance of the
                                 bin's estimate, Var(norm f - alpha norm g) / samples from the
                                 residual's sample moments (infinite below 2 samples)  */
} vcu_cv;

/* floats per residual sample in vcu_control_variates' replay records: the chosen list index and
 * the point; then, for VCU_RS_RUSSIAN_ROULETTE and VCU_RS_MIS, 1 when the point came from the
 * region's pdf (0 when uniform); then, for VCU_RS_MIS, the pdf point its weight was computed at */
int vcu_cv_replay_width(int32_t dim, int32_t sampling);

int vcu_control_variates(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested,
                         uint64_t iterations, const vcu_cv* cv, const float* replay, float* bins,
                         float* approximation, float* regions, vcu_stats* stats);

/* ------------------------------------------------------------------ Fubini over per-bin integrators
 * Replaces integrate(integrator_fubini<2>(first, monte_carlo(tail_samples, tail_seed)), bins, f, range)
 * and integrator_fubini({d0, d1}, first, rest) (src/combination/fubini.h:75-125) for a per-bin
 * first integrator: first = integrator_per_bin_parallel(monte_carlo(samples_per_bin, seed))
 * (method VCU_FUBINI_MONTE_CARLO) or integrator_per_bin_parallel(integrator_adaptive_iterations(
 * nested, iterations)) (VCU_FUBINI_NESTED: nested(simpson, trapezoidal) or nested(boole, simpson)).
 * The first integrator works over the first 2 dimensions (the bins take at most those), and every
 * evaluation at x integrates the remaining ones by Monte Carlo:  sum_k f(x, u_k) volume(rest) / K
 * accumulated in float (fubini.h:51-63, monte-carlo.h:41-63), with u_k from Philox keyed by
 * tail_seed and the bits of x (the reference draws them from one sequential std::mt19937, so the
 * agreement is statistical).  With n_order > 0 the problem is first reordered as integrator_reorder
 * does (src/combination/reorder.h:15-58): the integrator sees f(reorder(x)) over reorder(range),
 * where reorder puts coordinate `from` at place `to` for each (to, from) pair of `order` and the
 * others, in order, into the free places -- integrator_fubini({d0, d1}, ...) is the pairs (0, d0),
 * (1, d1).  Integrands of 3 or more dimensions (or of unbounded dimension, without reordering).
 * Bins are ASSIGNED. */
enum { VCU_FUBINI_MONTE_CARLO = 0, VCU_FUBINI_NESTED = 1 };

typedef struct vcu_fubini {
    int32_t dims;             /* dimensions integrated by the per-bin integrator: 2              */
    uint32_t tail_samples;    /* Monte Carlo samples of the remaining dimensions per evaluation  */
    uint64_t tail_seed;
    int32_t method;           /* VCU_FUBINI_MONTE_CARLO or VCU_FUBINI_NESTED                     */
    int32_t n_order;          /* (to, from) pairs in order[] (0: no reordering)                  */
    int32_t order[2 * VCU_MAX_DIM];
    uint64_t samples_per_bin; /* VCU_FUBINI_MONTE_CARLO                                          */
    uint64_t seed;
    vcu_nested nested;        /* VCU_FUBINI_NESTED                                               */
    uint64_t iterations;
} vcu_fubini;

int vcu_per_bin_fubini(vcu_ctx* ctx, const vcu_problem* p, const vcu_fubini* fubini, float* bins, vcu_stats* stats);

/* ------------------------------------------------------------------ learned control variate
 * No reference counterpart: per-bin integration (the integrator_per_bin_parallel contract,
 * src/integrator-per-bin-parallel.h:17-35, values ASSIGNED) with a small MLP control variate --
 * frequency encoding (6 bands), 4 hidden layers of 64, BF16 weights on the tensor cores, FP32
 * accumulation -- trained online (Adam, mean squared error) on `batch` fresh Philox samples of the
 * integrand per step, for at most `train_steps` steps, by the library's own forward/backward
 * kernels; with `check_every` > 0 the mean squared error on a fixed held-out set is measured every
 * `check_every` steps: after two checks without a 0.5 % improvement the learning rate drops to 0.3
 * of itself, and the third such plateau ends training.
 * The control variate of a bin is h, the piecewise-quadratic interpolant of the trained network g
 * on a grid of Simpson nodes -- `cells` cells per binned dimension inside the bin (0: h is constant
 * there, g's value at the bin centre) and `cells_unbinned` cells per unbinned dimension over the
 * range -- i.e. nested quadrature's own polynomial: the integral of h over the bin is exactly the
 * composite Simpson sum of the node values, so the estimate  integral(h) + mean(f - h)  over
 * `samples_per_bin` Philox points is unbiased.  With `fallback` set, `pilot` separate samples per
 * bin (0: samples/8 clamped to 8..256; not reused in the estimate) give the bin's weight
 * alpha = cov(f, h) / var(h), clamped to [0, 1.5], fixed before the residual samples: the estimate
 * is then  alpha integral(h) + mean(f - alpha h)  (still unbiased; alpha 0 is plain Monte Carlo of
 * the residual samples), and, when poly_bins/poly_variance are given (vcu_control_variates' bins
 * and vcu_cv::variance for the same problem), the polynomial control variate's estimate replaces
 * the bin's when its variance is the lower one.  At most 4913 grid nodes per bin.  Scalar
 * integrands of dimension 2, 3 or 5. */
typedef struct vcu_learned {
    uint64_t samples_per_bin;
    uint64_t seed;
    uint32_t train_steps;     /* at most this many Adam steps                                  */
    uint32_t batch;           /* training samples per step (rounded up to whole blocks)        */
    float learning_rate;
    uint32_t check_every;     /* held-out check period for early stopping (0: all steps)       */
    int32_t fallback;         /* 1: per-bin weight and choice of estimator from the pilot       */
    int32_t cells;            /* Simpson cells per binned dimension in a bin (0: constant)     */
    float* theta_out;         /* nullable host buffer: receives the trained fp32 parameters
                                 (vcu_mlp_eval layout), e.g. to checkpoint the network        */
    int32_t cells_unbinned;   /* Simpson cells per unbinned dimension over the range (>= 1)    */
    uint32_t pilot;           /* pilot samples per bin for the fallback choice (0: automatic)  */
    const float* poly_bins;   /* nullable (follows mem): the polynomial CV's bins              */
    const float* poly_variance; /* nullable (follows mem): their variances; both or neither    */
} vcu_learned;

typedef struct vcu_learned_report {
    double train_ms, integral_ms, residual_ms;
    double heldout_mse;       /* held-out mean squared error of the network at the end         */
    uint32_t fallback_bins;   /* bins whose weight is 0: the plain Monte Carlo estimate        */
    uint32_t polynomial_bins; /* bins that took the polynomial control variate's estimate      */
    uint32_t train_steps_run; /* Adam steps taken (early stopping)                             */
    uint32_t nodes_per_bin;   /* grid nodes of the interpolant per bin                         */
} vcu_learned_report;

/* network_integral (nullable, follows p->mem): per bin, the mean of h over the bin */
int vcu_learned_control_variates(vcu_ctx* ctx, const vcu_problem* p, const vcu_learned* opt, float* bins,
                                 float* network_integral, vcu_learned_report* report, vcu_stats* stats);

/* The network alone, for checking the kernels: outputs g(u) at npts points u in [0,1]^dim (host
 * arrays, row-major) for the fp32 parameter vector theta (layout: W0[FIN][64], b0, W1[64][64], b1,
 * W2, b2, W3, b3, w4[64], b4 with FIN = 16*ceil(13*dim/16)).  Without grad the outputs come from the
 * tcgen05 forward kernel the learned control variate evaluates its grid with; with y and grad
 * given, outputs and the gradient of mean((g - y)^2) come from the training kernel.  dim 2, 3 or 5. */
int vcu_mlp_eval(vcu_ctx* ctx, int32_t dim, const float* theta, const float* u, const float* y, int64_t npts,
                 float* out, float* grad);

/* ------------------------------------------------------------------ global adaptive nested NC
 * Replaces integrate(integrator_adaptive_iterations(nested(H,L), heuristic, iterations), bins, f,
 * range) with the integrator used directly rather than per bin
 * (src/nested/integrator-adaptive-iterations.h:12-15): one max-error heap over the whole range is
 * split `iterations` times (src/nested/regions-generator-adaptive-heap.h:18-45), then every region,
 * in heap order, is added into each bin it overlaps (src/newton-cotes/regions-integrator-sequential.h:
 * 37-58): bins ACCUMULATE (bins[b] += prod(res) * integral over bin n region).  Also the result of
 * integrator_adaptive_iterations_parallel (regions-integrator-parallel-regions.h) on one host thread.
 * Regions up to S^dim = 243 nodes, iterations < 2^23. */
int vcu_adaptive_iterations_global(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested,
                                   uint64_t iterations, float* bins, vcu_stats* stats);

/* ------------------------------------------------------------------ tolerance-driven adaptive NC
 * Replaces integrate(integrator_adaptive_tolerance(nested(H,L), heuristic, tolerance), bins, f, range)
 * (src/nested/integrator-adaptive-tolerance.h:9-56): a region whose heuristic error is below
 * `tolerance` is added into the bins it overlaps, any other is split and both halves visited, depth
 * first; bins ACCUMULATE, in the reference's depth-first order.  The tree is built breadth first on
 * the device; `max_regions` bounds the regions built (0: as many as 4 GiB of region storage holds,
 * at most 2^24-2) and VCU_QUEUE_OVERFLOW reports a tolerance that needs more.  leaves (nullable)
 * receives the number of leaf regions.  Regions up to S^dim = 243 nodes. */
int vcu_adaptive_tolerance(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested, float tolerance,
                           uint64_t max_regions, float* bins, uint64_t* leaves, vcu_stats* stats);

/* ------------------------------------------------------------------ batched independent integrals
 * Many calls of the reference's single-value form, viltrum::integrate(I, f, range)
 * (src/integrate.h:105-113), each with its own dimension, range, integrand parameters, method and
 * budget, run in one persistent launch captured in a CUDA graph.  Per item:
 *   VCU_BATCH_MONTE_CARLO : I = monte_carlo(budget, seed) (src/monte-carlo/monte-carlo.h:39-63,
 *                           89-95); Philox4x32-10 points keyed by (seed, sample, item position)
 *                           replace the item's std::mt19937, so agreement is statistical;
 *   VCU_BATCH_NESTED      : I = integrator_adaptive_iterations(nested(H,L), heuristic, budget - 1)
 *                           (src/nested/integrator-adaptive-iterations.h:12-25): budget regions;
 *                           the same value as the reference's.
 * All items share the integrand family `kind` (each item has its own parameters) and, for the
 * nested items, the rule pair / heuristic / metric of `nested` (NULL: simpson over trapezoidal,
 * default heuristic, absolute metric).  Scalar integrands only.  Nested items are limited to
 * S^dim <= 729 nodes per region (Simpson to 6-D, Boole to 4-D) and 2^24-2 regions. */
enum { VCU_BATCH_MONTE_CARLO = 0, VCU_BATCH_NESTED = 1 };

typedef struct vcu_batch_item {
    int32_t dim;        /* 1..6 */
    int32_t method;     /* VCU_BATCH_MONTE_CARLO or VCU_BATCH_NESTED */
    uint64_t budget;    /* samples (Monte Carlo) or regions (nested), >= 1 */
    uint64_t seed;      /* Monte Carlo stream */
    float range_min[VCU_MAX_DIM];
    float range_max[VCU_MAX_DIM];
    int32_t n_params;   /* this item's integrand parameters (host array) */
    int32_t reserved;
    const float* params;
} vcu_batch_item;

typedef struct vcu_batch_report {
    float* item_ms;       /* nullable host array [n_items]: each item's time on the device */
    int32_t threads;      /* block size the autotuner chose */
    uint32_t blocks;      /* resident blocks of the persistent launch */
    uint64_t nested_regions;
} vcu_batch_report;

/* results[n_items] (host or device per results_mem): item i's integral, in item order.
 * report and stats are nullable. */
int vcu_integrate_batch(vcu_ctx* ctx, int32_t kind, const vcu_nested* nested, const vcu_batch_item* items,
                        uint64_t n_items, float* results, int32_t results_mem, vcu_batch_report* report,
                        vcu_stats* stats);
/* Runs the batch last passed to vcu_integrate_batch on this context again from the copies already in
 * device memory (no host->device traffic): for repeated evaluation of a fixed batch. */
int vcu_integrate_batch_resident(vcu_ctx* ctx, float* results, int32_t results_mem, vcu_batch_report* report,
                                 vcu_stats* stats);

/* ------------------------------------------------------------------ allocation-free variant
 * No counterpart in the reference.  For host programs that must not allocate device memory -- a
 * plugin inside a process whose GPU memory belongs to another allocator, a real-time frame loop
 * that cannot take the device-wide synchronisation of cudaMalloc/cudaFree, or a service with a fixed memory budget -- this runs the same per-bin
 * adaptive nested quadrature as vcu_per_bin_adaptive_nested without a context and without any
 * cudaMalloc/cudaFree or allocating library call.  Its device scratch is a fixed array compiled
 * into the library (the status word plus a staging area of VCU_STATIC_MAX_BIN_VALUES floats for
 * host-memory bins, about 4 MiB), held by every GPU that loads the library until the process exits.
 *   - p->mem == VCU_MEM_HOST: bins is a host buffer, staged through the array; at most
 *     VCU_STATIC_MAX_BIN_VALUES bins x channels, larger requests return VCU_UNSUPPORTED.
 *     p->mem == VCU_MEM_DEVICE: bins is the caller's device buffer (no size limit).
 *   - Runs on the current device and on `stream` (a cudaStream_t, NULL = legacy default stream),
 *     and returns after the results are written.  Returns VCU_NAN_DETECTED if a bin is NaN.
 *   - The array's device address is looked up (cudaGetSymbolAddress) with the device current;
 *     the first call on a device does this set-up, so make it before any stream capture.  Calls
 *     on a stream that is not capturing look the address up again, so a cudaDeviceReset in the
 *     host process (which can move the array) is picked up by the next such call.
 *   - All calls share the array: calls that overlap on the GPU race and must be serialised.
 *   - No trace, no stats, no message: only the status code. */
#define VCU_STATIC_MAX_BIN_VALUES (1u << 20)
int vcu_per_bin_adaptive_nested_static(const vcu_problem* p, const vcu_nested* nested,
                                       uint64_t iterations, float* bins, void* stream);

#ifdef __cplusplus
}
#endif
