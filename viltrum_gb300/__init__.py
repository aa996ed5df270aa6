"""viltrum_gb300 -- viltrum's per-bin integration path on GB300 (sm_103a).

The names mirror viltrum's C++ API so a per-bin integration reads the same:

    import viltrum_gb300 as v
    bins = np.zeros(1024, np.float32)
    v.integrate(v.integrator_per_bin_parallel(v.monte_carlo(1024, seed=1)), bins,
                v.Integrand.wave2(), v.range_primary(2))

integrate(integrator, bins, f, range[, logger]) mirrors src/integrate.h:72-79/132-176 (bins is a
numpy array of shape `resolution` [+ (channels,)], indexed bins[pos0, pos1, ...] like viltrum's
bins(pos) accessor), and integrate(integrator, f, range) mirrors the single-value form
(src/integrate.h:105-113).  Each integrator keeps the write semantics of the reference one it
replaces: per-bin wrappers assign (src/integrator-per-bin-parallel.h:33), monte_carlo_per_bin_parallel
accumulates (src/monte-carlo/monte-carlo-per-bin-parallel.h:70).

Every integrator runs on the GPU through libviltrum_cuda.so; there is no CPU fallback, and a
combination the CUDA library does not implement raises NotImplementedError.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import scenes
from ._lib import (MEM_DEVICE, MEM_HOST, RR_ERROR, RR_INTEGRAL, RR_PDF, RR_UNIFORM, RS_IMPORTANCE, RS_MIS,
                   RS_RUSSIAN_ROULETTE, RS_UNIFORM, Context, Nested, VcuError, default_context, load)

__all__ = [
    "Context", "VcuError", "Integrand", "Range", "integrate", "range_", "range_all", "range_primary", "range_infinite",
    "trapezoidal", "simpson", "boole", "nested", "error_metric_absolute", "error_metric_relative",
    "error_heuristic_default", "error_heuristic_size", "monte_carlo", "monte_carlo_per_bin_parallel",
    "integrator_per_bin_parallel", "integrator_adaptive_iterations", "integrator_adaptive_iterations_parallel",
    "integrator_adaptive_tolerance",
    "scenes", "load",
    "rr_uniform_region", "rr_integral_region", "rr_error_region", "rr_pdf_region", "region_sampling_uniform",
    "region_sampling_importance", "region_sampling_russian_roulette", "region_sampling_mis", "cv_optimize_weight",
    "cv_fixed_weight", "regions_generator_adaptive_heap", "regions_integrator_parallel_variance_reduction",
    "integrator_region_based", "integrator_adaptive_variance_reduction_parallel", "integrator_crespo2021",
    "regions_generator_fubini", "integrator_crespo2021_infinite", "integrator_adaptive_fubini_variance_reduction_parallel",
]


# ------------------------------------------------------------------------------------ ranges
@dataclass
class Range:
    """viltrum::Range<float,DIM> (src/range.h:17-139)."""
    min: np.ndarray
    max: np.ndarray

    def __post_init__(self):
        self.min = np.asarray(self.min, dtype=np.float32).ravel()
        self.max = np.asarray(self.max, dtype=np.float32).ravel()
        if self.min.shape != self.max.shape or not 1 <= self.min.size <= 6:
            raise ValueError("range bounds must have the same dimension, 1..6")

    @property
    def dim(self) -> int:
        return int(self.min.size)


def range_(a, b) -> Range:
    return Range(np.atleast_1d(a), np.atleast_1d(b))


def range_all(n: int, a: float, b: float) -> Range:
    return Range(np.full(n, a), np.full(n, b))


def range_primary(n: int) -> Range:
    """range_primary<N>(): [0,1]^N (src/range.h:196-199)."""
    return range_all(n, 0.0, 1.0)


def range_infinite(a, b) -> Range:
    """range_infinite(a, b) (src/range-infinite.h:91-120): the listed leading dimensions; every
    further one is [0,1].  For integrands of unbounded dimension (Integrand.walk2), which draw the
    further coordinates themselves."""
    return range_(a, b)


# ------------------------------------------------------------------------------------ integrands
@dataclass
class Integrand:
    """A built-in integrand of libviltrum_cuda (include/vcu_integrands.h) with its parameters."""
    kind: int
    params: np.ndarray | None = None
    dim: int = 0

    @property
    def channels(self) -> int:
        return scenes.CHANNELS.get(self.kind, 1)

    @classmethod
    def poly2(cls):
        return cls(scenes.POLY2, None, 2)

    @classmethod
    def sin1(cls):
        return cls(scenes.SIN1, None, 1)

    @classmethod
    def sphere3(cls):
        return cls(scenes.SPHERE3, None, 3)

    @classmethod
    def wave2(cls):
        return cls(scenes.WAVE2, None, 2)

    @classmethod
    def scene2(cls, params=None, seed: int = 7):
        return cls(scenes.SCENE2, scenes.scene2(seed) if params is None else np.asarray(params, np.float32), 2)

    @classmethod
    def moving_scene3(cls, params=None, seed: int = 7):
        p = scenes.moving_scene3(seed) if params is None else np.asarray(params, np.float32)
        return cls(scenes.MOVING_SCENE3, p, 3)

    @classmethod
    def halfspace(cls, params):
        p = np.asarray(params, np.float32)
        return cls(scenes.HALFSPACE, p, int(p[0]))

    @classmethod
    def occluded_scene5(cls, params=None, seed: int = 7):
        p = scenes.occluded_scene5(seed) if params is None else np.asarray(params, np.float32)
        return cls(scenes.OCCLUDED_SCENE5, p, 5)

    @classmethod
    def walk2(cls, params=None, seed: int = 7):
        """The random walk over the 2-D scene: an integrand of unbounded dimension; integrate it over
        range_infinite(a, b) (its first two coordinates; the rest are [0,1) and drawn per sample)."""
        p = scenes.walk2(seed) if params is None else np.asarray(params, np.float32)
        return cls(scenes.WALK2, p, 2)


# ------------------------------------------------------------------------------------ rules
@dataclass(frozen=True)
class Rule:
    name: str
    samples: int


trapezoidal = Rule("trapezoidal", 2)
simpson = Rule("simpson", 3)
boole = Rule("boole", 5)


@dataclass(frozen=True)
class NestedRule:
    """nested(H, L) (src/nested/nested.h:42-45)."""
    high: Rule
    low: Rule

    def __post_init__(self):
        if (self.high.samples - 1) % (self.low.samples - 1) != 0:
            raise ValueError("Quadrature rules are not compatible for a nested rule")


def nested(high: Rule, low: Rule) -> NestedRule:
    return NestedRule(high, low)


@dataclass(frozen=True)
class error_metric_absolute:  # noqa: N801  (reference name)
    relative = False
    min_val = 1e-37


@dataclass(frozen=True)
class error_metric_relative:  # noqa: N801
    min_val: float = 1e-37
    relative = True


@dataclass(frozen=True)
class error_heuristic_default:  # noqa: N801
    metric: object = field(default_factory=error_metric_absolute)
    size = False
    size_weight = 1e-5
    min_size = 1e-37


@dataclass(frozen=True)
class error_heuristic_size:  # noqa: N801
    metric: object = field(default_factory=error_metric_absolute)
    size_weight: float = 1e-5
    min_size: float = 1e-37
    size = True


def _nested_struct(rule: NestedRule, heur) -> Nested:
    m = heur.metric
    return Nested(rule.high.samples, rule.low.samples, 1 if heur.size else 0, 1 if m.relative else 0,
                  float(heur.size_weight), float(heur.min_size), float(m.min_val))


# ------------------------------------------------------------------------------------ integrators
@dataclass
class MonteCarlo:
    """monte_carlo(samples, seed) (src/monte-carlo/monte-carlo.h:88-95)."""
    samples: int
    seed: int


@dataclass
class MonteCarloPerBinParallel:
    """monte_carlo_per_bin_parallel(samples, seed): per-bin samples, accumulated into the bins."""
    samples: int
    seed: int

    def integrate(self, bins, res, f, rng, logger=None, ctx=None, device_bins=False):
        return _run(self, bins, res, f, rng, logger, ctx, device_bins, accumulate=True)


@dataclass
class AdaptiveIterations:
    """integrator_adaptive_iterations(nested, heuristic, iterations).  Wrapped in
    integrator_per_bin_parallel it runs per bin; used directly it is viltrum's global form: one heap
    over the whole range, regions added into the bins (accumulates)."""
    rule: NestedRule
    heuristic: object
    iterations: int

    def integrate(self, bins, res, f, rng, logger=None, ctx=None, device_bins=False):
        return _run_global(self, bins, res, f, rng, logger, ctx, device_bins)


@dataclass
class PerBinParallel:
    """integrator_per_bin_parallel(inner) (src/integrator-per-bin-parallel.h:11-47)."""
    inner: object

    def integrate(self, bins, res, f, rng, logger=None, ctx=None, device_bins=False):
        return _run(self, bins, res, f, rng, logger, ctx, device_bins, accumulate=False)


def monte_carlo(samples: int, seed: int = 0) -> MonteCarlo:
    return MonteCarlo(int(samples), int(seed))


def monte_carlo_per_bin_parallel(samples: int, seed: int = 0) -> MonteCarloPerBinParallel:
    return MonteCarloPerBinParallel(int(samples), int(seed))


def integrator_adaptive_iterations(rule: NestedRule, heuristic_or_iterations, iterations: int | None = None):
    if iterations is None:
        return AdaptiveIterations(rule, error_heuristic_default(error_metric_absolute()), int(heuristic_or_iterations))
    return AdaptiveIterations(rule, heuristic_or_iterations, int(iterations))


@dataclass
class AdaptiveTolerance:
    """integrator_adaptive_tolerance(nested, heuristic, tolerance) (src/nested/integrator-adaptive-
    tolerance.h:9-56): accumulates into the bins, depth first."""
    rule: NestedRule
    heuristic: object
    tolerance: float
    max_regions: int = 0

    def integrate(self, bins, res, f, rng, logger=None, ctx=None, device_bins=False):
        return _run_global(self, bins, res, f, rng, logger, ctx, device_bins)


def integrator_adaptive_tolerance(rule: NestedRule, heuristic_or_tolerance=1e-3, tolerance: float | None = None,
                                  max_regions: int = 0):
    if tolerance is None and not hasattr(heuristic_or_tolerance, "metric"):
        return AdaptiveTolerance(rule, error_heuristic_default(error_metric_absolute()), float(heuristic_or_tolerance),
                                 max_regions)
    return AdaptiveTolerance(rule, heuristic_or_tolerance, float(1e-3 if tolerance is None else tolerance), max_regions)


def integrator_adaptive_iterations_parallel(rule: NestedRule, heuristic_or_iterations, iterations: int | None = None):
    """integrator_adaptive_iterations_parallel: the same regions and, on one host thread, the same
    bins as integrator_adaptive_iterations (regions-integrator-parallel-regions.h)."""
    return integrator_adaptive_iterations(rule, heuristic_or_iterations, iterations)


def integrator_per_bin_parallel(inner) -> PerBinParallel:
    return PerBinParallel(inner)


# control variates (src/control-variates/)
@dataclass(frozen=True)
class rr_uniform_region:  # noqa: N801  (reference name)
    """Uniform choice of the residual's region, weight = number of regions (region-russian-roulette.h:9-28)."""
    code = RR_UNIFORM


@dataclass(frozen=True)
class rr_integral_region:  # noqa: N801
    """The residual's region chosen with probability proportional to the norm (sum of |channel|) of the
    control variate's integral over bin n region, floored at 1% of the mean weight; sample weight
    1/probability (region-russian-roulette.h:30-68)."""
    code = RR_INTEGRAL


@dataclass(frozen=True)
class rr_error_region:  # noqa: N801
    """The residual's region chosen with probability proportional to norm(region error estimate) x
    volume(bin n region) / volume(region), floored at 1% of the mean weight; sample weight
    1/probability (region-russian-roulette.h:70-110)."""
    code = RR_ERROR


@dataclass(frozen=True)
class rr_pdf_region:  # noqa: N801
    """The residual's region chosen with probability proportional to the integral of its polynomial's
    pdf over bin n region, floored at factor_prob of the mean weight; sample weight 1/probability
    (region-russian-roulette.h:112-149).  Simpson high rule only."""
    factor_prob: float = 0.01
    code = RR_PDF


@dataclass(frozen=True)
class region_sampling_uniform:  # noqa: N801
    """Uniform point in bin n region, weight = its volume (region-sampling.h:9-20)."""
    code = RS_UNIFORM


@dataclass(frozen=True)
class region_sampling_importance:  # noqa: N801
    """Point drawn from the region polynomial's pdf over bin n region (uniform when that range's volume
    is below 1e-5), weight 1/pdf (region-sampling.h:22-43).  Simpson high rule only."""
    code = RS_IMPORTANCE


@dataclass(frozen=True)
class region_sampling_russian_roulette:  # noqa: N801
    """Pdf point or uniform point, chosen by the pdf's integral against the volume; weight 1/pdf of the
    strategy taken (region-sampling.h:47-81).  Simpson high rule only."""
    code = RS_RUSSIAN_ROULETTE


@dataclass(frozen=True)
class region_sampling_mis:  # noqa: N801
    """Pdf point kept or replaced by a uniform one with the power heuristic's probabilities
    (region-sampling.h:84-135).  Simpson high rule only."""
    power: float = 1.0
    cutoff: float = 0.0
    code = RS_MIS


@dataclass(frozen=True)
class cv_optimize_weight:  # noqa: N801
    """Control-variate weight alpha = clamp(cov/var) from the samples (weight-strategy.h:171-241)."""
    fixed = False
    alpha = 1.0


@dataclass(frozen=True)
class cv_fixed_weight:  # noqa: N801
    """Fixed control-variate weight (weight-strategy.h:7-35)."""
    alpha: float = 1.0
    fixed = True


@dataclass
class AdaptiveHeapGenerator:
    """regions_generator_adaptive_heap(rule, heuristic, iterations) (regions-generator-adaptive-heap.h:8-51)."""
    rule: NestedRule
    heuristic: object
    iterations: int


@dataclass
class VarianceReduction:
    """regions_integrator_parallel_variance_reduction(rr, cv, sampling, seed, samples)."""
    rr: object
    cv: object
    sampling: object
    seed: int
    samples: int


@dataclass
class RegionBased:
    """integrator_region_based(generator, regions_integrator) (integrator-region-based.h:5-29)."""
    generator: AdaptiveHeapGenerator
    integrator: VarianceReduction

    def integrate(self, bins, res, f, rng, logger=None, ctx=None, device_bins=False, replay=None,
                  approximation=None, regions=None):
        return _run_cv(self, bins, res, f, rng, logger, ctx, device_bins, replay, approximation, regions)


def regions_generator_adaptive_heap(rule: NestedRule, heuristic, iterations: int) -> AdaptiveHeapGenerator:
    return AdaptiveHeapGenerator(rule, heuristic, int(iterations))


@dataclass
class FubiniGenerator:
    """regions_generator_fubini<N>(generator, monte_carlo(samples, seed)) (regions-generator-fubini.h:7-28):
    regions over the first N dimensions, the others integrated by Monte Carlo in every evaluation."""
    dims: int
    generator: AdaptiveHeapGenerator
    rest: MonteCarlo


def regions_generator_fubini(dims: int, generator: AdaptiveHeapGenerator, rest) -> FubiniGenerator:
    if not isinstance(rest, MonteCarlo):
        raise NotImplementedError("the CUDA Fubini tail integrates the remaining dimensions by monte_carlo(n, seed)")
    if int(dims) != 2:
        raise NotImplementedError("the CUDA Fubini tail takes regions over the first 2 dimensions")
    return FubiniGenerator(int(dims), generator, rest)


def regions_integrator_parallel_variance_reduction(rr, cv, *args) -> VarianceReduction:
    """(rr, cv, sampling, seed, samples) or (rr, cv, samples, seed) as the reference's overloads."""
    if len(args) == 3:
        sampling, seed, samples = args
    elif len(args) == 2:
        sampling, (samples, seed) = region_sampling_uniform(), args
    else:
        raise TypeError("regions_integrator_parallel_variance_reduction(rr, cv, [sampling,] ...)")
    if not isinstance(rr, (rr_uniform_region, rr_integral_region, rr_error_region, rr_pdf_region)):
        raise NotImplementedError("the CUDA control variates implement rr_uniform_region, rr_integral_region, "
                                  "rr_error_region and rr_pdf_region")
    if not isinstance(sampling, (region_sampling_uniform, region_sampling_importance,
                                 region_sampling_russian_roulette, region_sampling_mis)):
        raise NotImplementedError("the CUDA control variates implement region_sampling_uniform, _importance, "
                                  "_russian_roulette and _mis")
    return VarianceReduction(rr, cv, sampling, int(seed), int(samples))


def integrator_region_based(generator, integrator: VarianceReduction) -> RegionBased:
    return RegionBased(generator, integrator)


def integrator_crespo2021_infinite(dims: int, iterations: int, mc_samples: int, spp: int, seed: int = 0) -> RegionBased:
    """integrator_crespo2021_infinite<dims>(iterations, mc_samples, spp, seed) (integrator-crespo2021.h:24-44)
    over a finite range: crespo2021's regions over the first `dims` dimensions, the others integrated by
    monte_carlo(mc_samples, 2*seed+1) inside every evaluation."""
    return integrator_region_based(
        regions_generator_fubini(dims, regions_generator_adaptive_heap(
            nested(simpson, trapezoidal), error_heuristic_size(error_metric_relative(), 1e-5), iterations),
            monte_carlo(mc_samples, 2 * seed + 1)),
        regions_integrator_parallel_variance_reduction(rr_uniform_region(), cv_optimize_weight(),
                                                       region_sampling_uniform(), seed, spp))


def integrator_adaptive_fubini_variance_reduction_parallel(dims: int, rule: NestedRule, heuristic, iterations: int,
                                                           mc_samples: int, rr, cv, sampler, spp: int,
                                                           seed: int = 0) -> RegionBased:
    """integrator_adaptive_fubini_variance_reduction_parallel<dims>(rule, heuristic, iterations, mc_samples, rr,
    cv, sampler, spp, seed) (integrator-adaptive-fubini-variance-reduction.h:28-41)."""
    return integrator_region_based(
        regions_generator_fubini(dims, regions_generator_adaptive_heap(rule, heuristic, iterations),
                                 monte_carlo(mc_samples, 2 * seed + 1)),
        regions_integrator_parallel_variance_reduction(rr, cv, sampler, seed, spp))


def integrator_adaptive_variance_reduction_parallel(rule: NestedRule, *args) -> RegionBased:
    """integrator_adaptive_variance_reduction_parallel(rule, [error_heuristic,] iterations, rr, cv,
    [region_sampler,] samples, [seed]) (integrator-adaptive-variance-reduction.h:12-41): the adaptive
    heap generator (default heuristic with the absolute metric when none is given) followed by
    regions_integrator_parallel_variance_reduction."""
    args = list(args)
    heur = error_heuristic_default(error_metric_absolute())
    if args and not isinstance(args[0], (int, np.integer)):
        heur = args.pop(0)
    if len(args) < 4:
        raise TypeError("integrator_adaptive_variance_reduction_parallel(rule, [heuristic,] iterations, rr, cv, "
                        "[sampler,] samples, [seed])")
    iterations, rr, cv = args[0], args[1], args[2]
    rest = args[3:]
    sampling = region_sampling_uniform()
    if rest and not isinstance(rest[0], (int, np.integer)):
        sampling = rest.pop(0)
    if not rest or len(rest) > 2:
        raise TypeError("samples (and optionally seed) expected after the cv strategy")
    samples, seed = int(rest[0]), int(rest[1]) if len(rest) > 1 else 0
    return integrator_region_based(regions_generator_adaptive_heap(rule, heur, iterations),
                                   regions_integrator_parallel_variance_reduction(rr, cv, sampling, seed, samples))


def integrator_crespo2021(iterations: int, spp: int, seed: int = 0) -> RegionBased:
    """integrator_crespo2021(iterations, spp, seed) (src/control-variates/integrator-crespo2021.h:7-22)."""
    return integrator_region_based(
        regions_generator_adaptive_heap(nested(simpson, trapezoidal),
                                        error_heuristic_size(error_metric_relative(), 1e-5), iterations),
        regions_integrator_parallel_variance_reduction(rr_uniform_region(), cv_optimize_weight(),
                                                       region_sampling_uniform(), seed, spp))


# ------------------------------------------------------------------------------------ integrate
def _as_integrand(f) -> Integrand:
    if isinstance(f, Integrand):
        return f
    raise TypeError("integrands are built-in functors of the CUDA library: pass a viltrum_gb300.Integrand")


def _run(integrator, bins, res, f, rng, logger, ctx, device_bins, accumulate):
    f = _as_integrand(f)
    ctx = ctx or default_context()
    res = [int(r) for r in res]
    if f.dim and f.dim != rng.dim:
        raise ValueError(f"integrand dimension {f.dim} does not match range dimension {rng.dim}")
    ch = f.channels
    nb = int(np.prod(res))
    if logger is not None:
        logger.log_progress(0, 1)
    mem = MEM_DEVICE if device_bins else MEM_HOST
    p = Context.problem(f.kind, f.params, rng.min, rng.max, res, mem)
    # a flat float32 buffer in viltrum's linear order is written in place (assign semantics)
    flat = (not device_bins and not accumulate and isinstance(bins, np.ndarray) and bins.ndim == 1
            and bins.dtype == np.float32 and bins.size == nb * ch and bins.flags.c_contiguous)
    out = bins if (device_bins or flat) else np.empty(nb * ch, dtype=np.float32)
    inner = integrator.inner if isinstance(integrator, PerBinParallel) else integrator
    if isinstance(inner, MonteCarloPerBinParallel):
        # monte_carlo_per_bin_parallel's own factor, added on the device to the current values
        if not device_bins:
            arr = np.asarray(bins, dtype=np.float32).reshape(tuple(res) + ((ch,) if ch > 1 else ()))
            axes = tuple(range(len(res) - 1, -1, -1)) + ((len(res),) if ch > 1 else ())
            out[...] = np.ascontiguousarray(arr.transpose(axes)).ravel()
        stats = ctx.per_bin_monte_carlo_accumulate(p, inner.samples, inner.seed, out)
        accumulate = False
    elif isinstance(inner, MonteCarlo):
        stats = ctx.per_bin_monte_carlo(p, inner.samples, inner.seed, out)
    elif isinstance(inner, AdaptiveIterations):
        stats = ctx.per_bin_adaptive_nested(p, _nested_struct(inner.rule, inner.heuristic), inner.iterations, out)
    else:
        raise NotImplementedError(f"no CUDA implementation of per-bin {type(inner).__name__}")
    if not device_bins and not flat:
        vals = out.reshape(tuple(reversed(res)) + (ch,)).transpose(tuple(range(len(res) - 1, -1, -1)) + (len(res),))
        if ch == 1:
            vals = vals[..., 0]
        target = bins
        if accumulate:
            target += vals.astype(target.dtype).reshape(target.shape)
        else:
            target[...] = vals.reshape(target.shape)
    if logger is not None:
        logger.log_progress(1, 1)
    return stats


def _run_global(ai, bins, res, f, rng, logger, ctx, device_bins):
    f = _as_integrand(f)
    ctx = ctx or default_context()
    res = [int(r) for r in res]
    ch = f.channels
    nb = int(np.prod(res))
    if logger is not None:
        logger.log_progress(0, 1)
    mem = MEM_DEVICE if device_bins else MEM_HOST
    p = Context.problem(f.kind, f.params, rng.min, rng.max, res, mem)
    flat = (not device_bins and isinstance(bins, np.ndarray) and bins.ndim == 1 and bins.dtype == np.float32
            and bins.size == nb * ch and bins.flags.c_contiguous)
    if device_bins or flat:
        out = bins
    else:
        # the caller's bins in viltrum's linear order (dim 0 fastest, channels last)
        arr = np.asarray(bins, dtype=np.float32).reshape(tuple(res) + ((ch,) if ch > 1 else ()))
        axes = tuple(range(len(res) - 1, -1, -1)) + ((len(res),) if ch > 1 else ())
        out = np.ascontiguousarray(arr.transpose(axes)).ravel()
    if isinstance(ai, AdaptiveTolerance):
        stats, _ = ctx.adaptive_tolerance(p, _nested_struct(ai.rule, ai.heuristic), ai.tolerance, out, ai.max_regions)
    else:
        stats = ctx.adaptive_iterations_global(p, _nested_struct(ai.rule, ai.heuristic), ai.iterations, out)
    if not device_bins and not flat:
        vals = out.reshape(tuple(reversed(res)) + (ch,)).transpose(tuple(range(len(res) - 1, -1, -1)) + (len(res),))
        if ch == 1:
            vals = vals[..., 0]
        bins[...] = vals.reshape(bins.shape)
    if logger is not None:
        logger.log_progress(1, 1)
    return stats


def _run_cv(rb: RegionBased, bins, res, f, rng, logger, ctx, device_bins, replay, approximation, regions):
    from ._lib import CvOpts
    f = _as_integrand(f)
    ctx = ctx or default_context()
    res = [int(r) for r in res]
    ch = f.channels
    nb = int(np.prod(res))
    if logger is not None:
        logger.log_progress(0, 1)
    g, vr = rb.generator, rb.integrator
    fubini_dims, tail = 0, 0
    if isinstance(g, FubiniGenerator):
        fubini_dims, tail, g = g.dims, int(g.rest.samples), g.generator
    mem = MEM_DEVICE if device_bins else MEM_HOST
    p = Context.problem(f.kind, f.params, rng.min, rng.max, res, mem)
    flat = (not device_bins and isinstance(bins, np.ndarray) and bins.ndim == 1 and bins.dtype == np.float32
            and bins.size == nb * ch and bins.flags.c_contiguous)
    out = bins if (device_bins or flat) else np.empty(nb * ch, dtype=np.float32)
    opts = CvOpts(vr.samples, vr.seed, 1 if vr.cv.fixed else 0, 0, float(vr.cv.alpha), vr.rr.code, vr.sampling.code,
                  float(getattr(vr.rr, "factor_prob", 0.01)), 0, float(getattr(vr.sampling, "power", 1.0)),
                  float(getattr(vr.sampling, "cutoff", 0.0)), fubini_dims, tail)
    stats = ctx.control_variates(p, _nested_struct(g.rule, g.heuristic), g.iterations, opts, out, approximation,
                                 regions, replay)
    if not device_bins and not flat:
        vals = out.reshape(tuple(reversed(res)) + (ch,)).transpose(tuple(range(len(res) - 1, -1, -1)) + (len(res),))
        if ch == 1:
            vals = vals[..., 0]
        bins[...] = vals.reshape(bins.shape)
    if logger is not None:
        logger.log_progress(1, 1)
    return stats


def integrate(integrator, *args, logger=None, ctx=None, device_bins=False):
    """integrate(integrator, bins, f, range) or integrate(integrator, f, range) (single value).

    bins: numpy array of shape `resolution` (+ (channels,) for multi-channel integrands), or,
    with device_bins=True, a CUDA buffer (torch tensor or pointer) of prod(resolution)*channels
    floats in viltrum's linear order (dim 0 fastest, channels interleaved).
    Returns the call's vcu_stats as a dict (single-value form: the value)."""
    if len(args) == 2:
        f, rng = args
        f = _as_integrand(f)
        sol = np.zeros((1, f.channels) if f.channels > 1 else (1,), dtype=np.float32)
        integrator.integrate(sol, [1], f, rng, logger, ctx, False) if hasattr(integrator, "integrate") \
            else _run(integrator, sol, [1], f, rng, logger, ctx, False, False)
        return sol[0]
    bins, f, rng = args
    f = _as_integrand(f)
    if device_bins:
        raise ValueError("device bins need an explicit resolution: use integrate_into(...)")
    res = list(bins.shape[:-1] if f.channels > 1 else bins.shape)
    if hasattr(integrator, "integrate"):
        st = integrator.integrate(bins, res, f, rng, logger, ctx, False)
    else:
        raise NotImplementedError(f"{type(integrator).__name__} is not a per-bin integrator")
    return st.as_dict()


def integrate_into(integrator, bins, resolution, f, rng, logger=None, ctx=None, device_bins=True):
    """integrate with an explicit resolution (viltrum's integrate(I, bins, res, f, range) form,
    src/integrate.h:72-79); with device_bins=True `bins` is a device buffer."""
    st = integrator.integrate(bins, list(resolution), _as_integrand(f), rng, logger, ctx, device_bins)
    return st.as_dict()
