"""Generate the golden fixtures that pin the CPU oracle to the viltrum reference.

Run where the reference sources are available (the fixtures are committed; the GPU machine never
runs this):

    make -C oracle ref          # builds oracle/_ref/libvref.so from the unmodified headers
    python tests/golden/make_golden.py

Each case is executed by the reference driver (oracle/_ref) and its outputs are stored in
tests/golden/<name>.npz.  The script also runs the C++ restatement (oracle/liboracle.so) on the
same case and refuses to write a fixture the restatement does not reproduce bit for bit.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from viltrum_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

SCENE_SMALL = scenes.scene2(seed=7)
MOVING_SMALL = scenes.moving_scene3(seed=7, n_gauss=8, n_disk=8)
HALF3 = scenes.halfspace(seed=11, dim=3)

# (name, method, kwargs)
CASES = [
    ("mc_wave2_bins16_spp64_seed1", "mc", dict(kind=scenes.WAVE2, params=None, rmin=[0, 0], rmax=[1, 1], res=[16],
                                             spp=64, seed=1, flavour=0, record=True)),
    ("mc_wave2_bins1024_spp1024_seed1", "mc", dict(kind=scenes.WAVE2, params=None, rmin=[0, 0], rmax=[1, 1],
                                                 res=[1024], spp=1024, seed=1, flavour=0, record=False)),
    ("mc_poly2_bins4x3_spp16_seed2_single", "mc", dict(kind=scenes.POLY2, params=None, rmin=[0, 0], rmax=[1, 1],
                                                     res=[4, 3], spp=16, seed=2, flavour=1, record=True)),
    ("mc_sin1_pi_spp64_seed5", "mc", dict(kind=scenes.SIN1, params=None, rmin=[0.0], rmax=[3.14159265], res=[1],
                                        spp=64, seed=5, flavour=0, record=True)),
    ("mc_sphere3_spp1024_seed3", "mc", dict(kind=scenes.SPHERE3, params=None, rmin=[-1, -1, -1], rmax=[1, 1, 1],
                                          res=[1], spp=1024, seed=3, flavour=0, record=False)),
    ("mc_moving3_rgb_bins4x4_spp8_seed9", "mc", dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL, rmin=[0, 0, 0],
                                                   rmax=[1, 1, 1], res=[4, 4], spp=8, seed=9, flavour=0,
                                                   record=True)),
    ("nc_scene2_bins16x16_bs_abs_it15", "nc", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1],
                                                  res=[16, 16], nested=("boole", "simpson", "default", "absolute"),
                                                  iterations=15)),
    ("nc_scene2_bins8x8_bs_rel_it15", "nc", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1],
                                                res=[8, 8], nested=("boole", "simpson", "default", "relative"),
                                                iterations=15)),
    ("nc_scene2_bins8x8_st_size_rel_it7", "nc", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0],
                                                    rmax=[1, 1], res=[8, 8],
                                                    nested=("simpson", "trapezoidal", "size", "relative"),
                                                    iterations=7)),
    ("nc_poly2_bins5_bs_abs_it4", "nc", dict(kind=scenes.POLY2, params=None, rmin=[0, 0], rmax=[1, 1], res=[5],
                                            nested=("boole", "simpson", "default", "absolute"), iterations=4)),
    ("nc_wave2_bins32_bs_abs_it15", "nc", dict(kind=scenes.WAVE2, params=None, rmin=[0, 0], rmax=[1, 1], res=[32],
                                              nested=("boole", "simpson", "default", "absolute"), iterations=15)),
    ("nc_wave2_bins4x4_bt_abs_it5", "nc", dict(kind=scenes.WAVE2, params=None, rmin=[0, 0], rmax=[1, 1],
                                              res=[4, 4], nested=("boole", "trapezoidal", "default", "absolute"),
                                              iterations=5)),
    ("nc_halfspace3_bins4_st_abs_it10", "nc", dict(kind=scenes.HALFSPACE, params=HALF3, rmin=[0, 0, 0],
                                                  rmax=[1, 1, 1], res=[4],
                                                  nested=("simpson", "trapezoidal", "default", "absolute"),
                                                  iterations=10)),
    ("nc_moving3_rgb_bins4x4_st_size_rel_it7", "nc", dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL,
                                                         rmin=[0, 0, 0], rmax=[1, 1, 1], res=[4, 4],
                                                         nested=("simpson", "trapezoidal", "size", "relative"),
                                                         iterations=7)),
    ("cv_moving3_rgb_bins16x16_it255_spp16_seed3", "cv", dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL,
                                                             rmin=[0, 0, 0], rmax=[1, 1, 1], res=[16, 16],
                                                             iterations=255, spp=16, seed=3, weight=0, alpha=1.0)),
    ("cv_scene2_bins16x16_it127_spp8_seed4", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0],
                                                       rmax=[1, 1], res=[16, 16], iterations=127, spp=8, seed=4,
                                                       weight=0, alpha=1.0)),
    ("cv_scene2_fixed_bins8x8_it63_spp4_seed6", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0],
                                                          rmax=[1, 1], res=[8, 8], iterations=63, spp=4, seed=6,
                                                          weight=1, alpha=0.75)),
    ("cv_poly2_crespo_bins1_it16_spp64_seed0", "cv", dict(kind=scenes.POLY2, params=None, rmin=[0, 0], rmax=[1, 1],
                                                         res=[1], iterations=16, spp=64, seed=0, weight=0,
                                                         alpha=1.0)),
    # residual region choice by importance: rr_integral_region / rr_error_region (rr = 1 / 2)
    ("cv_scene2_rrintegral_bins16x16_it127_spp8_seed9", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL,
                                                                  rmin=[0, 0], rmax=[1, 1], res=[16, 16],
                                                                  iterations=127, spp=8, seed=9, weight=0, alpha=1.0,
                                                                  rr=1)),
    ("cv_scene2_rrintegral_fixed0_bins8x8_it63_spp8_seed10", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL,
                                                                       rmin=[0, 0], rmax=[1, 1], res=[8, 8],
                                                                       iterations=63, spp=8, seed=10, weight=1,
                                                                       alpha=0.0, rr=1)),
    ("cv_scene2_rrerror_bins16x16_it127_spp8_seed11", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL,
                                                                rmin=[0, 0], rmax=[1, 1], res=[16, 16],
                                                                iterations=127, spp=8, seed=11, weight=0, alpha=1.0,
                                                                rr=2)),
    ("cv_moving3_rgb_rrerror_bins16x16_it255_spp16_seed12", "cv", dict(kind=scenes.MOVING_SCENE3,
                                                                      params=MOVING_SMALL, rmin=[0, 0, 0],
                                                                      rmax=[1, 1, 1], res=[16, 16], iterations=255,
                                                                      spp=16, seed=12, weight=0, alpha=1.0, rr=2)),
    ("cv_moving3_rgb_rrintegral_bins8x8_it127_spp16_seed13", "cv", dict(kind=scenes.MOVING_SCENE3,
                                                                       params=MOVING_SMALL, rmin=[0, 0, 0],
                                                                       rmax=[1, 1, 1], res=[8, 8], iterations=127,
                                                                       spp=16, seed=13, weight=0, alpha=1.0, rr=1)),
    # the Simpson pdf of the control variate: rr_pdf_region (rr = 3) and the point samplers
    # region_sampling_importance / _russian_roulette / _mis (sampling = 1 / 2 / 3)
    ("cv_scene2_rrpdf_bins16x16_it127_spp8_seed14", "cv", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0],
                                                              rmax=[1, 1], res=[16, 16], iterations=127, spp=8,
                                                              seed=14, weight=0, alpha=1.0, rr=3)),
    ("cv_scene2_importance_rrpdf_fixed0_bins8x8_it63_spp8_seed15", "cv",
     dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1], res=[8, 8], iterations=63, spp=8,
          seed=15, weight=1, alpha=0.0, rr=3, sampling=1)),
    ("cv_scene2_importance_bins16x16_it127_spp8_seed16", "cv",
     dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1], res=[16, 16], iterations=127, spp=8,
          seed=16, weight=0, alpha=1.0, sampling=1)),
    ("cv_scene2_rrsampling_rrpdf_bins16x16_it127_spp8_seed17", "cv",
     dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1], res=[16, 16], iterations=127, spp=8,
          seed=17, weight=0, alpha=1.0, rr=3, sampling=2)),
    ("cv_scene2_mis_p2_c005_bins16x16_it127_spp8_seed18", "cv",
     dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1], res=[16, 16], iterations=127, spp=8,
          seed=18, weight=0, alpha=1.0, sampling=3, mis_power=2.0, mis_cutoff=0.05)),
    ("cv_moving3_rgb_importance_rrpdf_bins16x16_it255_spp16_seed19", "cv",
     dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL, rmin=[0, 0, 0], rmax=[1, 1, 1], res=[16, 16],
          iterations=255, spp=16, seed=19, weight=0, alpha=1.0, rr=3, sampling=1)),
    ("cv_poly2_mis_bins1_it16_spp64_seed20", "cv", dict(kind=scenes.POLY2, params=None, rmin=[0, 0], rmax=[1, 1],
                                                        res=[1], iterations=16, spp=64, seed=20, weight=0, alpha=1.0,
                                                        sampling=3)),
]

CV_STRATEGY_KEYS = ("rr", "sampling", "mis_power", "mis_cutoff")

CRESPO = ("simpson", "trapezoidal", "size", "relative")

# integrator_adaptive_iterations used directly (one heap over the range, regions added into bins
# that start from a non-zero image)
GLOBAL_CASES = [
    ("global_scene2_bins16x16_st_abs_it255", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1],
                                                  res=[16, 16], nested=("simpson", "trapezoidal", "default", "absolute"),
                                                  iterations=255)),
    ("global_moving3_rgb_bins8x8_bs_abs_it127", dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL, rmin=[0, 0, 0],
                                                     rmax=[1, 1, 1], res=[8, 8],
                                                     nested=("boole", "simpson", "default", "absolute"), iterations=127)),
    ("global_halfspace3_bins4_st_size_rel_it63", dict(kind=scenes.HALFSPACE, params=HALF3, rmin=[0, 0, 0],
                                                      rmax=[1, 1, 1], res=[4],
                                                      nested=("simpson", "trapezoidal", "size", "relative"),
                                                      iterations=63)),
]


def global_initial(kw) -> np.ndarray:
    nb = int(np.prod(kw["res"]))
    ch = 3 if kw["kind"] == scenes.MOVING_SCENE3 else 1
    return (0.125 + 0.001 * np.arange(nb * ch)).astype(np.float32)


def run_global(lib: orc.Oracle, kw: dict) -> dict:
    hi, lo, heur, met = kw["nested"]
    return {"bins": lib.adaptive_global(kw["kind"], kw["params"], kw["rmin"], kw["rmax"], kw["res"],
                                        orc.Nested.make(hi, lo, heur, met), kw["iterations"],
                                        initial=global_initial(kw))}


# integrator_adaptive_tolerance: depth first, leaves added into bins that start from a non-zero image
TOL_CASES = [
    ("tolerance_scene2_bins16x16_bs_abs_1e-6", dict(kind=scenes.SCENE2, params=SCENE_SMALL, rmin=[0, 0], rmax=[1, 1],
                                                    res=[16, 16], nested=("boole", "simpson", "default", "absolute"),
                                                    tolerance=1e-6)),
    ("tolerance_moving3_rgb_bins8x8_st_abs_1e-4", dict(kind=scenes.MOVING_SCENE3, params=MOVING_SMALL, rmin=[0, 0, 0],
                                                       rmax=[1, 1, 1], res=[8, 8],
                                                       nested=("simpson", "trapezoidal", "default", "absolute"),
                                                       tolerance=1e-4)),
]


def run_tolerance(lib: orc.Oracle, kw: dict) -> dict:
    hi, lo, heur, met = kw["nested"]
    bins, n = lib.adaptive_tolerance(kw["kind"], kw["params"], kw["rmin"], kw["rmax"], kw["res"],
                                     orc.Nested.make(hi, lo, heur, met), kw["tolerance"], initial=global_initial(kw))
    return {"bins": bins}


# independent single-value integrals (the batched-integrals workload at small budgets)
# integrator_crespo2021_infinite<2> over the finite range of the moving-disk scene: regions over
# (x, y), time integrated by Monte Carlo in every evaluation.  The reference draws those tail
# samples from one sequential std::mt19937 stream, so the device is compared with these outputs
# statistically (the reference's bins for several seeds, against the FP64 truth).
FUBINI_CASES = [
    ("fubini_moving3_rgb_bins32x32_it511_mc8_spp16", dict(params=scenes.moving_scene3(seed=7, n_gauss=16, n_disk=16),
                                                          rmin=[0, 0, 0], rmax=[1, 1, 1], res=[32, 32],
                                                          iterations=511, mc_samples=8, spp=16,
                                                          seeds=list(range(1, 9)))),
]


# the random walk over the scene (an integrand of unbounded dimension) over range_infinite: the
# reference's per-bin Monte Carlo and crespo2021_infinite<2>, several seeds each (statistical)
WALK_CASES = [
    ("walk_mc_bins16x16_spp256", dict(params=scenes.walk2(), rmin=[0, 0], rmax=[1, 1], res=[16, 16], walk_method=0,
                                     spp=256, iterations=0, mc_samples=0, seeds=list(range(1, 9)))),
    ("walk_crespo_infinite_bins16x16_it255_mc8_spp16", dict(params=scenes.walk2(), rmin=[0, 0], rmax=[1, 1],
                                                            res=[16, 16], walk_method=1, spp=16, iterations=255,
                                                            mc_samples=8, seeds=list(range(1, 9)))),
]


def run_walk(ref: orc.Oracle, kw: dict) -> np.ndarray:
    return np.stack([ref.walk(kw["params"], kw["rmin"], kw["rmax"], kw["res"], kw["walk_method"], kw["spp"], seed,
                              kw["iterations"], kw["mc_samples"]) for seed in kw["seeds"]])


def run_fubini(ref: orc.Oracle, kw: dict) -> np.ndarray:
    return np.stack([ref.crespo2021_infinite(scenes.MOVING_SCENE3, kw["params"], kw["rmin"], kw["rmax"], kw["res"],
                                             kw["iterations"], kw["mc_samples"], kw["spp"], seed)
                     for seed in kw["seeds"]])


# integrator_fubini<2> over a per-bin integrator with a Monte Carlo tail, without and with the
# reorder of integrator_fubini({0, 2}, ...): the reference's bins for several seeds (statistical:
# the tail draws from one sequential std::mt19937 stream)
PER_BIN_FUBINI_CASES = [
    ("fubini_perbin_nested_moving3_bins16x16_it15_mc8", dict(params=scenes.moving_scene3(seed=7, n_gauss=16, n_disk=16),
                                                             rmin=[0, 0, 0], rmax=[1, 1, 1], res=[16, 16], method=1,
                                                             spp=0, iterations=15, mc_samples=8, swap_xt=False,
                                                             seeds=list(range(1, 9)))),
    ("fubini_perbin_nested_moving3_xt_bins16x16_it15_mc8", dict(params=scenes.moving_scene3(seed=7, n_gauss=16,
                                                                                              n_disk=16),
                                                                rmin=[0, 0, 0], rmax=[1, 1, 1], res=[16, 16], method=1,
                                                                spp=0, iterations=15, mc_samples=8, swap_xt=True,
                                                                seeds=list(range(1, 9)))),
    ("fubini_perbin_mc_moving3_xt_bins16x16_spp16_mc4", dict(params=scenes.moving_scene3(seed=7, n_gauss=16, n_disk=16),
                                                             rmin=[0, 0, 0], rmax=[1, 1, 1], res=[16, 16], method=0,
                                                             spp=16, iterations=0, mc_samples=4, swap_xt=True,
                                                             seeds=list(range(1, 9)))),
]


def run_per_bin_fubini(ref: orc.Oracle, kw: dict) -> np.ndarray:
    return np.stack([ref.per_bin_fubini(kw["params"], kw["rmin"], kw["rmax"], kw["res"], kw["method"], kw["spp"],
                                        kw["iterations"], kw["mc_samples"], seed, kw["swap_xt"])
                     for seed in kw["seeds"]])


BATCH_CASES = [
    ("batch_halfspace_n64_seed5", dict(n=64, seed=5, budget_lo=1, budget_hi=400)),
]


def run_batch(lib: orc.Oracle, kw: dict) -> dict:
    items = scenes.batch_items(kw["n"], kw["seed"], kw["budget_lo"], kw["budget_hi"])
    nested = orc.Nested.make("simpson", "trapezoidal")
    out = np.array([lib.integrate_single(scenes.HALFSPACE, it["params"], it["rmin"], it["rmax"], it["method"],
                                         it["budget"], it["seed"], nested) for it in items], dtype=np.float32)
    return {"values": out}


def visit_to_linear(res, parallel: bool) -> np.ndarray:
    """Bin (dim-0-fastest linear index) visited at each step of the reference's bin loop.

    for_each(parallel, ...) walks dim 0 in the outer loop and the remaining dims, dim 1 fastest,
    inside it (src/foreach.h:98-120); for_each(sequential, ...) walks dim-0 fastest."""
    res = [int(r) for r in res]
    nb = int(np.prod(res))
    lin = np.arange(nb)
    if not parallel or len(res) == 1:
        return lin
    idx = np.array(np.unravel_index(lin, res[::-1]))[::-1]  # idx[d] for linear order
    # visit key: dims 1..D-1 dim-1 fastest, then dim 0 slowest
    key = np.zeros(nb, dtype=np.int64)
    mul = 1
    for d in list(range(1, len(res))) + [0]:
        key += idx[d] * mul
        mul *= res[d]
    order = np.empty(nb, dtype=np.int64)
    order[key] = lin
    return order


def run(lib: orc.Oracle, method: str, kw: dict) -> dict:
    kw = dict(kw)
    if method == "mc":
        bins, pts = lib.per_bin_monte_carlo(kw["kind"], kw["params"], kw["rmin"], kw["rmax"], kw["res"], kw["spp"],
                                            kw["seed"], kw["flavour"], record=kw["record"])
        out = {"bins": bins}
        if pts is not None:
            if lib.kind == "reference":
                fixed = np.empty_like(pts)
                fixed[visit_to_linear(kw["res"], True)] = pts
                pts = fixed
            out["points"] = pts
        return out
    if method == "nc":
        hi, lo, heur, met = kw["nested"]
        nested = orc.Nested.make(hi, lo, heur, met)
        bins, _ = lib.per_bin_adaptive_nested(kw["kind"], kw["params"], kw["rmin"], kw["rmax"], kw["res"], nested,
                                              kw["iterations"])
        return {"bins": bins}
    if method == "cv":
        nested = orc.Nested.make(*CRESPO)
        r = lib.control_variates(kw["kind"], kw["params"], kw["rmin"], kw["rmax"], kw["res"], nested,
                                 kw["iterations"], kw["spp"], kw["seed"], kw["weight"], kw["alpha"], regions=True,
                                 replay=True, **{k: kw[k] for k in CV_STRATEGY_KEYS if k in kw})
        pts = r["replay"]
        if lib.kind == "port":
            pts = pts[:, :, 1:1 + len(kw["rmin"])]
        else:
            fixed = np.empty_like(pts)
            fixed[visit_to_linear(kw["res"], int(kw["res"][0]) >= 4)] = pts
            pts = fixed
        return {"bins": r["bins"], "regions": r["regions"], "points": pts}
    raise ValueError(method)


def pieces_inputs() -> dict:
    """Inputs of the single-piece probes: the control-variate weight accumulator on paired samples
    (the shape of main/compilation-tests/covariance.cc, plus constant, anti-correlated and one-sample
    series) and the 1-D Simpson pdf / sampler (the node values of main/compilation-tests/region-sample.cc
    and inverse.cc, plus lifted, constant and edge-peaked parabolas) over three sub-ranges."""
    rng = np.random.default_rng(21)
    x = rng.uniform(0, 2 * np.pi, 1000).astype(np.float32)
    v0 = np.sin(x).astype(np.float32)
    series = []
    for n, noise in ((20, 0.1), (1000, 0.5)):
        g = v0[:n]
        f = (g + rng.uniform(-noise, noise, n)).astype(np.float32)
        series.append((f, g))
    series.append((v0[:50].copy(), np.full(50, 0.25, np.float32)))          # variance 0: alpha 1
    series.append(((1.5 - np.abs(v0[:50])).astype(np.float32), v0[:50].copy()))  # |f|, |g| anti-correlated: alpha 0
    series.append((v0[:1].copy(), v0[1:2].copy()))                          # one sample: the approximation
    cv_len = np.array([len(f) for f, _ in series], np.int64)
    nodes = np.array([[1, 0.2, 1], [0.43, 0.9, 0.42], [0, 0, 1], [1, -0.5, 1], [2, 2, 2], [0, 1, 0],
                      [0.1, 3.0, 0.05]], np.float32)
    ranges = np.array([[0, 1], [0, 0.125], [0.3, 0.7]], np.float32)
    t = np.linspace(0.0, 1.0, 9).astype(np.float32)
    s = np.concatenate([np.arange(10) * np.float32(0.1), rng.uniform(0, 1, 6)]).astype(np.float32)
    return {"cv_f": np.concatenate([f for f, _ in series]), "cv_g": np.concatenate([g for _, g in series]),
            "cv_len": cv_len, "cv_approx": np.float32(0.7), "nodes": nodes, "ranges": ranges, "t": t, "s": s}


def run_pieces(lib: orc.Oracle, kw: dict) -> dict:
    moments, off = [], 0
    for n in kw["cv_len"]:
        moments.append(lib.cv_optimize_moments(kw["cv_f"][off:off + n], kw["cv_g"][off:off + n], float(kw["cv_approx"])))
        off += int(n)
    pdf = np.zeros((len(kw["nodes"]), len(kw["ranges"]), len(kw["t"])), np.float32)
    smp = np.zeros((len(kw["nodes"]), len(kw["ranges"]), len(kw["s"])), np.float32)
    for i, nd in enumerate(kw["nodes"]):
        for j, (t0, t1) in enumerate(kw["ranges"]):
            # the pdf is read inside the sub-range: t mapped onto [t0, t1]
            tt = (np.float32(t0) + kw["t"] * np.float32(t1 - t0)).astype(np.float32)
            pdf[i, j] = lib.simpson_pdf_1d(nd, tt, float(t0), float(t1))
            smp[i, j] = lib.simpson_sample_1d(nd, kw["s"], float(t0), float(t1))
    return {"moments": np.array(moments, np.float64), "pdf": pdf, "samples": smp}


def main() -> int:
    """Regenerates every fixture, or only those whose names start with one of the arguments."""
    only = sys.argv[1:]

    def wanted(name: str) -> bool:
        return not only or any(name.startswith(o) for o in only)

    ref = orc.reference()
    if ref is None:
        print("oracle/_ref/libvref.so is missing: run `make -C oracle ref` where the reference exists")
        return 1
    port = orc.port()
    bad = 0
    for name, method, kw in CASES:
        if not wanted(name):
            continue
        r = run(ref, method, kw)
        p = run(port, method, kw)
        same = all(np.array_equal(r[k].view(np.uint32), p[k].view(np.uint32)) for k in r)
        if not same:
            bad += 1
            for k in r:
                if not np.array_equal(r[k], p[k]):
                    diff = np.abs(r[k].astype(np.float64) - p[k].astype(np.float64))
                    print(f"MISMATCH {name}.{k}: max |diff| {diff.max():.3e} at {np.unravel_index(diff.argmax(), diff.shape)}"
                          f" ({int((diff > 0).sum())} of {diff.size} differ)")
            continue
        meta = {k: np.asarray(v) for k, v in kw.items() if v is not None and k not in ("params",)}
        if kw.get("params") is not None:
            meta["params"] = np.asarray(kw["params"], dtype=np.float32)
        if method == "nc":
            meta["nested"] = np.array(kw["nested"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method=method, **meta, **{"out_" + k: v for k, v in r.items()})
        print(f"ok {name}")
    for name, kw in GLOBAL_CASES:
        if not wanted(name):
            continue
        r, p = run_global(ref, kw), run_global(port, kw)
        if not np.array_equal(r["bins"].view(np.uint32), p["bins"].view(np.uint32)):
            bad += 1
            d = np.abs(r["bins"].astype(np.float64) - p["bins"])
            print(f"MISMATCH {name}: max |diff| {d.max():.3e} ({int((d > 0).sum())} differ)")
            continue
        meta = {k: np.asarray(v) for k, v in kw.items() if k not in ("params", "nested")}
        meta["params"] = np.asarray(kw["params"], dtype=np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="global", nested=np.array(kw["nested"]),
                            initial=global_initial(kw), **meta, out_bins=r["bins"])
        print(f"ok {name}")
    for name, kw in TOL_CASES:
        if not wanted(name):
            continue
        r, p = run_tolerance(ref, kw), run_tolerance(port, kw)
        if not np.array_equal(r["bins"].view(np.uint32), p["bins"].view(np.uint32)):
            bad += 1
            print(f"MISMATCH {name}")
            continue
        meta = {k: np.asarray(v) for k, v in kw.items() if k not in ("params", "nested")}
        meta["params"] = np.asarray(kw["params"], dtype=np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="tolerance", nested=np.array(kw["nested"]),
                            initial=global_initial(kw), **meta, out_bins=r["bins"])
        print(f"ok {name}")
    for name, kw in BATCH_CASES:
        if not wanted(name):
            continue
        r, p = run_batch(ref, kw), run_batch(port, kw)
        if not np.array_equal(r["values"].view(np.uint32), p["values"].view(np.uint32)):
            bad += 1
            print(f"MISMATCH {name}: {int((r['values'] != p['values']).sum())} items differ")
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="batch", **{k: np.asarray(v) for k, v in kw.items()},
                            out_values=r["values"])
        print(f"ok {name}")
    for name, kw in FUBINI_CASES:
        if not wanted(name):
            continue
        out = run_fubini(ref, kw)
        meta = {k: np.asarray(v) for k, v in kw.items() if k != "params"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="fubini", kind=scenes.MOVING_SCENE3,
                            params=np.asarray(kw["params"], np.float32), **meta, out_bins=out)
        print(f"ok {name} (reference outputs, compared statistically)")
    for name, kw in PER_BIN_FUBINI_CASES:
        if not wanted(name):
            continue
        out = run_per_bin_fubini(ref, kw)
        meta = {("first" if k == "method" else k): np.asarray(v) for k, v in kw.items() if k != "params"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="per_bin_fubini", kind=scenes.MOVING_SCENE3,
                            params=np.asarray(kw["params"], np.float32), **meta, out_bins=out)
        print(f"ok {name} (reference outputs, compared statistically)")
    for name, kw in WALK_CASES:
        if not wanted(name):
            continue
        out = run_walk(ref, kw)
        meta = {k: np.asarray(v) for k, v in kw.items() if k != "params"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), method="walk", kind=scenes.WALK2,
                            params=np.asarray(kw["params"], np.float32), **meta, out_bins=out)
        print(f"ok {name} (reference outputs, compared statistically)")
    if wanted("pieces_cv_moments_simpson_pdf"):
        kw = pieces_inputs()
        r, p = run_pieces(ref, kw), run_pieces(port, kw)
        if all(np.array_equal(r[k].view(np.uint8), p[k].view(np.uint8)) for k in r):
            np.savez_compressed(os.path.join(HERE, "pieces_cv_moments_simpson_pdf.npz"), method="pieces", **kw,
                                **{"out_" + k: v for k, v in r.items()})
            print("ok pieces_cv_moments_simpson_pdf")
        else:
            bad += 1
            print("MISMATCH pieces_cv_moments_simpson_pdf: " +
                  ", ".join(k for k in r if not np.array_equal(r[k].view(np.uint8), p[k].view(np.uint8))))
    total = sum(wanted(n) for n in [c[0] for c in CASES] + [c[0] for c in BATCH_CASES + GLOBAL_CASES + TOL_CASES]
                + ["pieces_cv_moments_simpson_pdf"])
    print(f"{total - bad} of {total} cases bit-identical")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
