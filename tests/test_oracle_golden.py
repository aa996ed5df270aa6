"""The CPU oracle reproduces every golden fixture of the reference bit for bit.

The fixtures were produced by the unmodified reference headers (oracle/_ref, see
tests/golden/make_golden.py); this pins the C++ restatement the GPU is later compared to."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc


def cv_strategy(g):
    """The residual strategy a control-variate fixture was made with (uniform when absent)."""
    out = {k: int(g[k]) for k in ("rr", "sampling") if k in g}
    out.update({k: float(g[k]) for k in ("mis_power", "mis_cutoff") if k in g})
    return out


def _nested(g):
    hi, lo, heur, met = [str(x) for x in g["nested"]]
    return orc.Nested.make(hi, lo, heur, met)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_golden(port, name):
    g = load_golden(name)
    method = str(g["method"])
    params = g.get("params")
    if method == "mc":
        bins, pts = port.per_bin_monte_carlo(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"], int(g["spp"]),
                                             int(g["seed"]), int(g["flavour"]), record="out_points" in g)
        assert np.array_equal(bins.view(np.uint32), g["out_bins"].view(np.uint32))
        if "out_points" in g:
            assert np.array_equal(pts.view(np.uint32), g["out_points"].view(np.uint32))
    elif method == "nc":
        bins, _ = port.per_bin_adaptive_nested(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"], _nested(g),
                                               int(g["iterations"]))
        assert np.array_equal(bins.view(np.uint32), g["out_bins"].view(np.uint32))
    elif method == "cv":
        r = port.control_variates(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"],
                                  orc.Nested.make("simpson", "trapezoidal", "size", "relative"), int(g["iterations"]),
                                  int(g["spp"]), int(g["seed"]), int(g["weight"]), float(g["alpha"]), regions=True,
                                  replay=True, **cv_strategy(g))
        assert np.array_equal(r["bins"].view(np.uint32), g["out_bins"].view(np.uint32))
        assert np.array_equal(r["regions"].view(np.uint32), g["out_regions"].view(np.uint32))
        dim = len(g["rmin"])
        assert np.array_equal(r["replay"][:, :, 1:1 + dim].view(np.uint32), g["out_points"].view(np.uint32))
    elif method == "global":
        out = port.adaptive_global(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"], _nested(g), int(g["iterations"]),
                                   initial=g["initial"])
        assert np.array_equal(out.view(np.uint32), g["out_bins"].view(np.uint32))
    elif method == "tolerance":
        out, _ = port.adaptive_tolerance(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"], _nested(g),
                                         float(g["tolerance"]), initial=g["initial"])
        assert np.array_equal(out.view(np.uint32), g["out_bins"].view(np.uint32))
    elif method == "fubini":
        # statistical fixture (the reference's own outputs for several seeds): each seed's bins are
        # near the FP64 truth and the seeds differ, as Monte Carlo estimates do
        from viltrum_gb300 import scenes
        exact = scenes.exact_bins(int(g["kind"]), params, g["rmin"], g["rmax"], g["res"], t_nodes=96)
        mse = [float(np.mean((b - exact) ** 2)) for b in g["out_bins"]]
        assert max(mse) < 2e-3 and len(set(np.round(mse, 12))) == len(mse)
    elif method == "per_bin_fubini":
        # statistical fixture (the reference's own outputs for several seeds).  Bins over (x, y): near
        # the FP64 truth.  Bins over (x, t) (integrator_fubini({0, 2}, ...)): each column of x-bins,
        # averaged over t, matches the truth's column averaged over y (both are the integral over
        # the x-bin); in both the seeds differ, as Monte Carlo estimates do
        from viltrum_gb300 import scenes
        res = [int(r) for r in g["res"]]
        exact = scenes.exact_bins(int(g["kind"]), params, g["rmin"], g["rmax"], res, t_nodes=96)
        b = g["out_bins"].astype(np.float64)
        assert np.isfinite(b).all() and len({float(x) for x in b.mean(axis=(1, 2))}) == b.shape[0]
        if bool(g["swap_xt"]):
            col_ref = b.mean(axis=0).reshape(res[1], res[0], 3).mean(axis=0)
            col_exact = exact.reshape(res[1], res[0], 3).mean(axis=0)
            assert np.max(np.abs(col_ref - col_exact)) < 0.05
        else:
            assert max(float(np.mean((x - exact) ** 2)) for x in b) < 2e-3
    elif method == "walk":
        # statistical fixture of the unbounded-dimension walk (the reference's own outputs for several
        # seeds): finite, non-negative scene values (the control-variate estimate may dip a little
        # below 0), and the seeds differ as Monte Carlo estimates do
        b = g["out_bins"]
        assert np.isfinite(b).all() and (b >= -0.01).all() and b.mean() > 0
        assert len({float(x) for x in b.mean(axis=1)}) == b.shape[0]
    elif method == "batch":
        from viltrum_gb300 import scenes
        items = scenes.batch_items(int(g["n"]), int(g["seed"]), int(g["budget_lo"]), int(g["budget_hi"]))
        nested = orc.Nested.make("simpson", "trapezoidal")
        out = np.array([port.integrate_single(scenes.HALFSPACE, it["params"], it["rmin"], it["rmax"], it["method"],
                                              it["budget"], it["seed"], nested) for it in items], dtype=np.float32)
        assert np.array_equal(out.view(np.uint32), g["out_values"].view(np.uint32))
    elif method == "pieces":
        from golden.make_golden import run_pieces  # the fixture's own probe loop
        out = run_pieces(port, g)
        for k in ("moments", "pdf", "samples"):
            assert np.array_equal(out[k].view(np.uint8), g["out_" + k].view(np.uint8)), k
    else:
        pytest.fail(method)


def test_known_answers(port):
    """Known answers printed by the reference's examples (main/doc/*.cc)."""
    # Boole reproduces x^2+y^2 exactly: 5 bins of 5*int x^2 dx + 1/3 (main/doc/integrators.cc:57-63)
    bins, _ = port.per_bin_adaptive_nested(1, None, [0, 0], [1, 1], [5], orc.Nested.make(), 0)
    exact = np.array([5 * ((i + 1) ** 3 - i ** 3) / 375.0 + 1.0 / 3.0 for i in range(5)])
    assert np.allclose(bins[:, 0], exact, rtol=1e-5)  # float coefficient rounding of the reference
    # sin over [0, pi] = 2 (main/doc/montecarlo-1d.cc:6-12), 4096 samples
    b, _ = port.per_bin_monte_carlo(2, None, [0.0], [3.14159265], [1], 4096, 5)
    assert abs(b[0, 0] - 2.0) < 0.05
    # sphere volume 4pi/3 (main/doc/integrands.cc:34)
    b, _ = port.per_bin_monte_carlo(3, None, [-1, -1, -1], [1, 1, 1], [1], 1 << 15, 3)
    assert abs(b[0, 0] - 4 * np.pi / 3) < 0.05
