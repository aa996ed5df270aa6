"""The Python factories mirror the reference's integrator constructors (no device use): the
argument forms resolve to the same strategy objects, and forms the CUDA path does not implement
are refused at construction."""
import pytest

import viltrum_gb300 as v
from viltrum_gb300 import _lib


def test_variance_reduction_overloads():
    st = v.nested(v.simpson, v.trapezoidal)
    a = v.integrator_adaptive_variance_reduction_parallel(st, 127, v.rr_integral_region(), v.cv_fixed_weight(0.0), 64)
    assert a.generator.iterations == 127 and a.integrator.samples == 64 and a.integrator.seed == 0
    assert isinstance(a.generator.heuristic, v.error_heuristic_default)
    b = v.integrator_adaptive_variance_reduction_parallel(
        st, v.error_heuristic_size(v.error_metric_relative(), 1e-5), 255, v.rr_pdf_region(0.05), v.cv_optimize_weight(),
        v.region_sampling_mis(2.0, 0.1), 16, 9)
    assert b.integrator.seed == 9 and b.integrator.sampling.power == 2.0 and b.integrator.rr.factor_prob == 0.05
    assert b.integrator.rr.code == _lib.RR_PDF and b.integrator.sampling.code == _lib.RS_MIS
    with pytest.raises(TypeError):
        v.integrator_adaptive_variance_reduction_parallel(st, 127, v.rr_uniform_region())


def test_fubini_forms():
    c = v.integrator_crespo2021_infinite(2, 1023, 8, 16, 4)
    assert isinstance(c.generator, v.FubiniGenerator)
    assert c.generator.dims == 2 and c.generator.rest.samples == 8 and c.generator.rest.seed == 9
    with pytest.raises(NotImplementedError):
        v.regions_generator_fubini(3, c.generator.generator, v.monte_carlo(4, 1))


def test_unsupported_strategies_are_refused():
    class rr_custom:  # noqa: N801
        pass
    with pytest.raises(NotImplementedError):
        v.regions_integrator_parallel_variance_reduction(rr_custom(), v.cv_optimize_weight(), 16, 0)
    assert v.range_infinite([0, 0], [1, 1]).dim == 2
