"""Batched independent integrals (one persistent, graph-captured launch) against the reference.

Each item is a single-value integrate(I, f, range).  Nested items (adaptive nested(simpson,
trapezoidal) with `budget` regions) are deterministic and must equal the reference's value: the
committed golden fixture holds values of the unmodified reference, and larger cases are compared
with the oracle.  Tolerance: relative 1e-5 per item in FP32 (the region integrals are rounded as the
reference rounds them, so the values are in fact bit-identical, which the golden case asserts).
Monte Carlo items draw Philox points instead of the reference's std::mt19937, so they are checked
statistically against an FP64 truth: |est - truth| <= 3 sigma for all but a few items."""
import os

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as orc
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ST = _lib.Nested(orc.RULE["simpson"], orc.RULE["trapezoidal"], orc.HEUR["default"], orc.METRIC["absolute"],
                 1e-5, 1e-37, 1e-37)


def _halfspace_np(params, x):
    """FP64 evaluation of the half-space family at points x[n, dim]."""
    dim = int(params[0])
    a, b, nrm, c = params[1:7][:dim], params[7:13][:dim], params[13:19][:dim], params[19]
    v = np.prod(np.exp(-a * x) * np.cos(b * x), axis=1)
    return np.where(x @ nrm.astype(np.float64) < c, v, 0.0)


def _oracle_values(port, items):
    nested = orc.Nested.make("simpson", "trapezoidal")
    return np.array([port.integrate_single(scenes.HALFSPACE, it["params"], it["rmin"], it["rmax"], it["method"],
                                           it["budget"], it["seed"], nested) for it in items], np.float32)


def _close(gpu, ref):
    ref = np.asarray(ref, np.float64)
    tol = RTOL * np.abs(ref) + 1e-30
    return np.abs(np.asarray(gpu, np.float64) - ref) <= tol


def test_batch_nested_matches_reference_golden(ctx):
    g = load_golden("batch_halfspace_n64_seed5")
    items = scenes.batch_items(int(g["n"]), int(g["seed"]), int(g["budget_lo"]), int(g["budget_hi"]))
    out, st, rep = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
    nested = np.array([it["method"] == 1 for it in items])
    ref = g["out_values"]
    assert nested.sum() > 20
    assert np.all(_close(out[nested], ref[nested]))
    assert np.array_equal(out[nested].view(np.uint32), ref[nested].view(np.uint32))
    assert st.evaluations > 0 and st.kernel_launches >= 1 and rep.blocks >= 1


def test_batch_nested_matches_oracle_uneven(ctx, port):
    """Dimensions 2-6, budgets 256..2048 regions (S^dim up to 729 nodes per region)."""
    items = scenes.batch_items(40, seed=21, budget_lo=256, budget_hi=2048, methods=(1,))
    out, st, rep = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
    ref = _oracle_values(port, items)
    ok = _close(out, ref)
    assert ok.all(), [(i, items[i]["dim"], items[i]["budget"], out[i], ref[i]) for i in np.flatnonzero(~ok)]
    assert rep.nested_regions == sum(it["budget"] for it in items)


def test_batch_boole_simpson_matches_oracle(ctx, port):
    """Another rule pair (boole over simpson, 5^dim nodes: dimensions 2-4)."""
    items = scenes.batch_items(12, seed=8, budget_lo=16, budget_hi=300, dims=(2, 4), methods=(1,))
    nb = _lib.Nested(orc.RULE["boole"], orc.RULE["simpson"], orc.HEUR["default"], orc.METRIC["relative"],
                     1e-5, 1e-37, 1e-37)
    out, _, _ = ctx.integrate_batch(scenes.HALFSPACE, items, nb)
    nested = orc.Nested.make("boole", "simpson", "default", "relative")
    ref = np.array([port.integrate_single(scenes.HALFSPACE, it["params"], it["rmin"], it["rmax"], 1, it["budget"], 0,
                                          nested) for it in items], np.float32)
    assert np.all(_close(out, ref))


def test_batch_monte_carlo_statistics(ctx):
    """Philox Monte Carlo items: within 3 sigma of the FP64 truth for all but a few of 48 items,
    sigma from the integrand's variance over the range and the item's sample count."""
    items = scenes.batch_items(48, seed=33, budget_lo=4096, budget_hi=65536, methods=(0,))
    out, _, _ = ctx.integrate_batch(scenes.HALFSPACE, items)
    rng = np.random.default_rng(1)
    exceed = 0
    for i, it in enumerate(items):
        x = rng.random((1 << 19, it["dim"]))
        fx = _halfspace_np(np.asarray(it["params"], np.float64), x)
        truth, sd = fx.mean(), fx.std()
        sigma = np.hypot(sd / np.sqrt(it["budget"]), sd / np.sqrt(x.shape[0]))
        exceed += abs(float(out[i]) - truth) > 3 * sigma + 1e-9
    assert exceed <= 3


def test_batch_launch_shape_does_not_change_results(ctx):
    items = scenes.batch_items(32, seed=4, budget_lo=64, budget_hi=4096)
    runs = []
    for t in ("256", "1024"):
        os.environ["VCU_BATCH_THREADS"] = t
        try:
            out, _, rep = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
        finally:
            del os.environ["VCU_BATCH_THREADS"]
        assert rep.threads == int(t)
        runs.append(out.copy())
    assert np.array_equal(runs[0].view(np.uint32), runs[1].view(np.uint32))


def test_batch_resident_replay_and_item_times(ctx):
    items = scenes.batch_items(64, seed=6, budget_lo=256, budget_hi=8192)
    first, _, _ = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
    again = np.empty_like(first)
    ms = np.zeros(len(items), np.float32)
    st, rep = ctx.integrate_batch_resident(again, item_ms=ms)
    assert np.array_equal(first.view(np.uint32), again.view(np.uint32))
    assert np.all(ms > 0) and np.all(ms <= st.device_ms * 1.01 + 0.01)
    import torch
    dev = torch.empty(len(items), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.integrate_batch_resident(dev, mem=_lib.MEM_DEVICE)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), first.view(np.uint32))


def test_batch_edge_cases(ctx, port):
    # budget 1: the root region alone; one-sample Monte Carlo; a 1-D item
    p2 = scenes.halfspace(5, 2)
    p1 = scenes.halfspace(9, 1)
    items = [dict(dim=2, method=1, budget=1, seed=0, params=p2, rmin=[0, 0], rmax=[1, 1]),
             dict(dim=2, method=0, budget=1, seed=3, params=p2, rmin=[0, 0], rmax=[1, 1]),
             dict(dim=1, method=1, budget=7, seed=0, params=p1, rmin=[0.25], rmax=[0.75]),
             dict(dim=2, method=1, budget=2, seed=0, params=p2, rmin=[-1, 0.5], rmax=[2, 0.5])]  # zero-volume range
    out, _, _ = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
    for i in (0, 2, 3):
        ref = _oracle_values(port, [items[i]])[0]
        assert out[i].view(np.uint32) == np.float32(ref).view(np.uint32), (i, out[i], ref)
    assert np.isfinite(out[1])
    # invalid requests are refused before any launch
    bad = [
        [dict(dim=2, method=1, budget=0, params=p2, rmin=[0, 0], rmax=[1, 1])],              # zero budget
        [dict(dim=2, method=5, budget=4, params=p2, rmin=[0, 0], rmax=[1, 1])],              # bad method
        [dict(dim=2, method=1, budget=4, params=p2, rmin=[1, 0], rmax=[0, 1])],              # min > max
        [dict(dim=3, method=1, budget=4, params=p2, rmin=[0, 0, 0], rmax=[1, 1, 1])],        # params of 2-D
        [dict(dim=2, method=1, budget=1 << 24, params=p2, rmin=[0, 0], rmax=[1, 1])],        # too many regions
    ]
    for b in bad:
        with pytest.raises(_lib.VcuError) as e:
            ctx.integrate_batch(scenes.HALFSPACE, b, ST)
        assert e.value.code == 1
    six = [dict(dim=6, method=1, budget=4, params=scenes.halfspace(1, 6), rmin=[0] * 6, rmax=[1] * 6)]
    nb = _lib.Nested(orc.RULE["boole"], orc.RULE["simpson"], 0, 0, 1e-5, 1e-37, 1e-37)
    with pytest.raises(_lib.VcuError) as e:
        ctx.integrate_batch(scenes.HALFSPACE, six, nb)  # 5^6 nodes per region
    assert e.value.code == 8
    with pytest.raises(_lib.VcuError):
        ctx.integrate_batch_resident(np.empty(1, np.float32))  # failed uploads leave no batch


def test_batch_fixed_arity_family(ctx, port):
    """Items of a fixed-arity family (the 2-D scene, different scene per item)."""
    items = []
    for i in range(6):
        prm = scenes.scene2(seed=40 + i, n_gauss=8, n_disk=4)
        items.append(dict(dim=2, method=1, budget=50 + 30 * i, seed=0, params=prm, rmin=[0, 0], rmax=[1, 1]))
    out, _, _ = ctx.integrate_batch(scenes.SCENE2, items, ST)
    nested = orc.Nested.make("simpson", "trapezoidal")
    ref = np.array([port.integrate_single(scenes.SCENE2, it["params"], it["rmin"], it["rmax"], 1, it["budget"], 0,
                                          nested) for it in items], np.float32)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_batch_full_size_properties(ctx, port):
    """The 4096-integral workload (dimensions 2-6, budgets 256..65536): every value finite, a
    deterministic re-run, and the smallest nested items identical to the oracle."""
    items = scenes.batch_items(4096, seed=11)
    out, st, rep = ctx.integrate_batch(scenes.HALFSPACE, items, ST)
    assert np.all(np.isfinite(out))
    again = np.empty_like(out)
    ctx.integrate_batch_resident(again)
    assert np.array_equal(out.view(np.uint32), again.view(np.uint32))
    small = [i for i, it in enumerate(items) if it["method"] == 1 and it["budget"] * 3 ** it["dim"] < 60000][:24]
    assert len(small) >= 8
    ref = _oracle_values(port, [items[i] for i in small])
    assert np.all(_close(out[small], ref))
