"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE, not the product.

`port()` loads oracle/liboracle.so, the C++ restatement of viltrum's per-bin integration path
(oracle.cc); `reference()` loads oracle/_ref/libvref.so, the driver over the unmodified reference
headers, which exists only where the reference sources were available to build it.

Only tests/, bench.py's cpu_baseline leg and __graft_entry__.smoke() use this module, and only as
the checker the CUDA library is compared against.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvref.so")

RULE = {"trapezoidal": 2, "simpson": 3, "boole": 5}
HEUR = {"default": 0, "size": 1}
METRIC = {"absolute": 0, "relative": 1}
CV_OPTIMIZE, CV_FIXED = 0, 1
RR_UNIFORM, RR_INTEGRAL, RR_ERROR, RR_PDF = 0, 1, 2, 3  # rr_{uniform,integral,error,pdf}_region
# region_sampling_{uniform,importance,russian_roulette,mis}
RS_UNIFORM, RS_IMPORTANCE, RS_RUSSIAN_ROULETTE, RS_MIS = 0, 1, 2, 3


def replay_width(dim, sampling=RS_UNIFORM):
    """Floats per residual sample of the oracle's replay records (orc_replay_width)."""
    return 1 + dim + (1 if sampling == RS_RUSSIAN_ROULETTE else 1 + dim if sampling == RS_MIS else 0)
MC_PER_BIN_PARALLEL, MC_PER_BIN_PARALLEL_SINGLE = 0, 1

_f32p = ctypes.POINTER(ctypes.c_float)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)


class CvStrategy(ctypes.Structure):
    """orc_cv: the control-variate integrator's residual strategy."""
    _fields_ = [("weight", ctypes.c_int32), ("rr", ctypes.c_int32), ("alpha", ctypes.c_double),
                ("rr_factor", ctypes.c_float), ("sampling", ctypes.c_int32), ("mis_power", ctypes.c_double),
                ("mis_cutoff", ctypes.c_double)]


class Nested(ctypes.Structure):
    """orc_nested: a Nested<H,L> rule with its error heuristic and metric."""

    _fields_ = [
        ("rule_hi", ctypes.c_int32),
        ("rule_lo", ctypes.c_int32),
        ("heuristic", ctypes.c_int32),
        ("metric", ctypes.c_int32),
        ("size_weight", ctypes.c_double),
        ("min_size", ctypes.c_double),
        ("min_val", ctypes.c_double),
    ]

    @classmethod
    def make(cls, hi="boole", lo="simpson", heuristic="default", metric="absolute", size_weight=1e-5,
             min_size=1e-37, min_val=1e-37):
        return cls(RULE[hi], RULE[lo], HEUR[heuristic], METRIC[metric], size_weight, min_size, min_val)


def reference_sources() -> str | None:
    """Directory of the viltrum sources (viltrum.h and src/) that the reference driver and the
    header-compatibility test compile against: $VILTRUM_REFERENCE, else the checkout this oracle
    was pinned against; None where neither holds the sources (e.g. the GPU hosts)."""
    for cand in (os.environ.get("VILTRUM_REFERENCE"), "/root/reference"):
        if cand and os.path.exists(os.path.join(cand, "viltrum.h")):
            return cand
    return None


def build_reference() -> str | None:
    """Build oracle/_ref/libvref.so (oracle/Makefile `ref`) where the reference sources exist."""
    src = reference_sources()
    if src is None:
        return None
    subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFERENCE={src}"])
    return REF_SO


def build(force: bool = False) -> str:
    """Compile liboracle.so from oracle.cc with the flags of oracle/Makefile."""
    src = os.path.join(HERE, "oracle.cc")
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in ("oracle.cc", "oracle_impl.h", "oracle.h", "vrgb.h")):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-o", PORT_SO, src, "-lpthread"]
        subprocess.check_call(cmd)
    return PORT_SO


def _ptr(a, t=_f32p):
    return None if a is None else a.ctypes.data_as(t)


class Oracle:
    def __init__(self, path: str, prefix: str):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        self.kind = "reference" if prefix == "ref_" else "port"
        L = self.lib
        if prefix == "orc_":
            L.orc_channels.restype = ctypes.c_int
            L.orc_channels.argtypes = [ctypes.c_int32]
            L.orc_eval.restype = ctypes.c_int
            L.orc_eval.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, ctypes.c_int64,
                                   _f32p]
            L.orc_per_bin_adaptive_nested_threads.restype = ctypes.c_int
            L.orc_per_bin_adaptive_nested_threads.argtypes = [
                ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                ctypes.POINTER(Nested), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, _f32p, _i32p]
        f = getattr(L, prefix + "per_bin_monte_carlo")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, _f32p, _f32p]
        f = getattr(L, prefix + "per_bin_adaptive_nested")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.POINTER(Nested), ctypes.c_uint64, _f32p, _i32p]
        f = getattr(L, prefix + "adaptive_global")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.POINTER(Nested), ctypes.c_uint64, _f32p]
        f = getattr(L, prefix + "adaptive_tolerance")
        f.restype = ctypes.c_int64
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.POINTER(Nested), ctypes.c_float, ctypes.c_uint64, _f32p]
        f = getattr(L, prefix + "integrate_single")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32,
                      ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(Nested), _f32p]
        f = getattr(L, prefix + "cv_optimize_moments")
        f.restype = ctypes.c_int
        f.argtypes = [_f32p, _f32p, ctypes.c_uint64, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]
        for name in ("simpson_pdf_1d", "simpson_sample_1d"):
            f = getattr(L, prefix + name)
            f.restype = ctypes.c_int
            f.argtypes = [_f32p, ctypes.c_float, ctypes.c_float, ctypes.c_float, _f32p]
        f = getattr(L, prefix + "control_variates")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.POINTER(Nested), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                      ctypes.POINTER(CvStrategy), _f32p, _f32p, _f32p, _f32p]

    # ------------------------------------------------------------------ helpers
    @staticmethod
    def _problem(params, rmin, rmax, res):
        params = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float32)
        rmin = np.ascontiguousarray(rmin, dtype=np.float32)
        rmax = np.ascontiguousarray(rmax, dtype=np.float32)
        res = np.ascontiguousarray(res, dtype=np.uint64)
        return params, rmin, rmax, res

    @staticmethod
    def channels(kind: int) -> int:
        return 3 if kind == 6 else 1

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{self.prefix}{what} failed with status {rc}")

    # ------------------------------------------------------------------ API
    def eval(self, kind, params, x):
        params = np.ascontiguousarray(params if params is not None else np.zeros(1), dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32)
        n, dim = x.shape
        out = np.zeros((n, self.channels(kind)), dtype=np.float32)
        self._check(self.lib.orc_eval(kind, _ptr(params), params.size, dim, _ptr(x), n, _ptr(out)), "eval")
        return out

    def per_bin_monte_carlo(self, kind, params, rmin, rmax, res, spp, seed, flavour=MC_PER_BIN_PARALLEL,
                            record=False, initial=None):
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32) if initial is None else np.array(initial, dtype=np.float32).ravel()
        pts = np.zeros(nb * spp * rmin.size, dtype=np.float32) if record else None
        rc = getattr(self.lib, self.prefix + "per_bin_monte_carlo")(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p), spp,
            seed, flavour, _ptr(out), _ptr(pts))
        self._check(rc, "per_bin_monte_carlo")
        return out.reshape(nb, ch), (pts.reshape(nb, spp, rmin.size) if record else None)

    def per_bin_adaptive_nested(self, kind, params, rmin, rmax, res, nested: Nested, iterations, trace=False):
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32)
        tr = np.zeros(nb * iterations * 2, dtype=np.int32) if trace else None
        rc = getattr(self.lib, self.prefix + "per_bin_adaptive_nested")(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
            ctypes.byref(nested), iterations, _ptr(out), _ptr(tr, _i32p))
        self._check(rc, "per_bin_adaptive_nested")
        return out.reshape(nb, ch), (tr.reshape(nb, iterations, 2) if trace else None)

    def per_bin_adaptive_nested_threads(self, kind, params, rmin, rmax, res, nested, iterations, bin_begin,
                                        bin_end, nthreads, trace=False):
        """bins [bin_begin, bin_end) on `nthreads` host threads; with trace=True also the split trace
        (dimension, popped error bits) of those bins, as per_bin_adaptive_nested returns it."""
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32)
        tr = np.zeros(nb * iterations * 2, dtype=np.int32) if trace else None
        rc = self.lib.orc_per_bin_adaptive_nested_threads(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
            ctypes.byref(nested), iterations, bin_begin, bin_end, nthreads, _ptr(out), _ptr(tr, _i32p))
        self._check(rc, "per_bin_adaptive_nested_threads")
        bins = out.reshape(nb, ch)[bin_begin:bin_end]
        if not trace:
            return bins
        return bins, tr.reshape(nb, iterations, 2)[bin_begin:bin_end]

    def adaptive_global(self, kind, params, rmin, rmax, res, nested: Nested, iterations, initial=None):
        """integrator_adaptive_iterations used directly: one heap over the range, regions added into
        the bins (which start from `initial`, zeros by default)."""
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32) if initial is None else np.array(initial, np.float32).ravel().copy()
        rc = getattr(self.lib, self.prefix + "adaptive_global")(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
            ctypes.byref(nested), iterations, _ptr(out))
        self._check(rc, "adaptive_global")
        return out.reshape(nb, ch)

    def adaptive_tolerance(self, kind, params, rmin, rmax, res, nested: Nested, tolerance, initial=None,
                           max_regions=1 << 24):
        """integrator_adaptive_tolerance: returns (bins, number of leaf regions)."""
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32) if initial is None else np.array(initial, np.float32).ravel().copy()
        n = getattr(self.lib, self.prefix + "adaptive_tolerance")(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
            ctypes.byref(nested), tolerance, max_regions, _ptr(out))
        if n < -1:
            raise RuntimeError(f"{self.prefix}adaptive_tolerance failed ({n})")
        return out.reshape(nb, ch), int(n)

    def integrate_single(self, kind, params, rmin, rmax, method, budget, seed=0, nested: Nested | None = None):
        """One single-value integrate(I, f, range): method 0 = monte_carlo(budget, seed), 1 = adaptive
        nested quadrature with `budget` regions."""
        params, rmin, rmax, _ = self._problem(params, rmin, rmax, [1])
        out = np.zeros(1, dtype=np.float32)
        rc = getattr(self.lib, self.prefix + "integrate_single")(
            kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), method, budget, seed,
            ctypes.byref(nested) if nested is not None else None, _ptr(out))
        self._check(rc, "integrate_single")
        return float(out[0])

    def walk(self, params, rmin, rmax, res, method, spp, seed, iterations=0, mc_samples=0):
        """The random walk over the scene (an integrand of unbounded dimension) over
        range_infinite(rmin, rmax): per-bin Monte Carlo (method 0) or crespo2021_infinite<2> (method
        1), the unmodified reference only."""
        params = np.ascontiguousarray(params, np.float32)
        rmin = np.ascontiguousarray(rmin, np.float32)
        rmax = np.ascontiguousarray(rmax, np.float32)
        res = np.ascontiguousarray(res, np.uint64)
        out = np.zeros(int(np.prod(res)), dtype=np.float32)
        f = getattr(self.lib, self.prefix + "walk")
        f.restype = ctypes.c_int
        f.argtypes = [_f32p, ctypes.c_int32, _f32p, _f32p, _u64p, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64,
                      ctypes.c_uint64, ctypes.c_uint64, _f32p]
        rc = f(_ptr(params), params.size, _ptr(rmin), _ptr(rmax), _ptr(res, _u64p), method, spp, seed, iterations,
               mc_samples, _ptr(out))
        self._check(rc, "walk")
        return out

    def crespo2021_infinite(self, kind, params, rmin, rmax, res, iterations, mc_samples, spp, seed):
        """integrator_crespo2021_infinite<2> over a finite range (the unmodified reference only)."""
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        out = np.zeros(nb * ch, dtype=np.float32)
        f = getattr(self.lib, self.prefix + "crespo2021_infinite")
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int32, _f32p, ctypes.c_int32, ctypes.c_int32, _f32p, _f32p, ctypes.c_int32, _u64p,
                      ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _f32p]
        rc = f(kind, _ptr(params), params.size, rmin.size, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
               iterations, mc_samples, spp, seed, _ptr(out))
        self._check(rc, "crespo2021_infinite")
        return out.reshape(nb, ch)

    def per_bin_fubini(self, params, rmin, rmax, res, method, spp, iterations, mc_samples, seed, swap_xt=False):
        """integrator_fubini<2>(integrator_per_bin_parallel(first), monte_carlo(mc_samples, seed + 1)) over the
        moving-disk scene, first = monte_carlo(spp, seed) (method 0) or adaptive nested(simpson,
        trapezoidal) with `iterations` splits (method 1); swap_xt: integrator_fubini({0, 2}, ...), bins
        over dimensions 0 and 2 (the unmodified reference only)."""
        params = np.ascontiguousarray(params, np.float32)
        rmin = np.ascontiguousarray(rmin, np.float32)
        rmax = np.ascontiguousarray(rmax, np.float32)
        res = np.ascontiguousarray(res, np.uint64)
        out = np.zeros(int(np.prod(res)) * 3, dtype=np.float32)
        f = getattr(self.lib, self.prefix + "per_bin_fubini")
        f.restype = ctypes.c_int
        f.argtypes = [_f32p, ctypes.c_int32, _f32p, _f32p, _u64p, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64,
                      ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, _f32p]
        rc = f(_ptr(params), params.size, _ptr(rmin), _ptr(rmax), _ptr(res, _u64p), method, spp, iterations,
               mc_samples, seed, 1 if swap_xt else 0, _ptr(out))
        self._check(rc, "per_bin_fubini")
        return out.reshape(-1, 3)

    def control_variates(self, kind, params, rmin, rmax, res, nested: Nested, iterations, spp, seed,
                         weight=CV_OPTIMIZE, alpha=1.0, regions=False, replay=False, approx=False, rr=RR_UNIFORM,
                         sampling=RS_UNIFORM, rr_factor=0.01, mis_power=1.0, mis_cutoff=0.0):
        params, rmin, rmax, res = self._problem(params, rmin, rmax, res)
        nb = int(np.prod(res))
        ch = self.channels(kind)
        dim = rmin.size
        out = np.zeros(nb * ch, dtype=np.float32)
        ap = np.zeros(nb * ch, dtype=np.float32) if approx else None
        rg = np.zeros((iterations + 1) * 2 * dim, dtype=np.float32) if regions else None
        width = replay_width(dim, sampling) if self.prefix == "orc_" else dim
        strategy = CvStrategy(weight, rr, alpha, rr_factor, sampling, mis_power, mis_cutoff)
        rp = np.zeros(nb * spp * width, dtype=np.float32) if replay else None
        rc = getattr(self.lib, self.prefix + "control_variates")(
            kind, _ptr(params), params.size, dim, _ptr(rmin), _ptr(rmax), res.size, _ptr(res, _u64p),
            ctypes.byref(nested), iterations, spp, seed, ctypes.byref(strategy), _ptr(out), _ptr(ap), _ptr(rg),
            _ptr(rp))
        self._check(rc, "control_variates")
        return {
            "bins": out.reshape(nb, ch),
            "approximation": None if ap is None else ap.reshape(nb, ch),
            "regions": None if rg is None else rg.reshape(iterations + 1, 2, dim),
            "replay": None if rp is None else rp.reshape(nb, spp, width),
        }
    # ------------------------------------------------------------------ probes of single pieces
    def cv_optimize_moments(self, f, g, approximation=0.0):
        """cv_optimize_weight's accumulator fed (f[i], g[i]) in order ->
        (variance of g, covariance of f and g, alpha, integral(approximation))."""
        f = np.ascontiguousarray(f, dtype=np.float32)
        g = np.ascontiguousarray(g, dtype=np.float32)
        assert f.shape == g.shape
        out = np.zeros(4, dtype=np.float64)
        rc = getattr(self.lib, self.prefix + "cv_optimize_moments")(
            _ptr(f), _ptr(g), f.size, approximation, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self._check(rc, "cv_optimize_moments")
        return tuple(float(v) for v in out)

    def _simpson_1d(self, name, nodes, u, t0, t1):
        nodes = np.ascontiguousarray(nodes, dtype=np.float32)
        assert nodes.size == 3
        out = np.zeros(1, dtype=np.float32)
        fn = getattr(self.lib, self.prefix + name)
        res = np.empty(len(u), dtype=np.float32)
        for i, v in enumerate(u):
            self._check(fn(_ptr(nodes), float(v), t0, t1, _ptr(out)), name)
            res[i] = out[0]
        return res

    def simpson_pdf_1d(self, nodes, t, t0, t1):
        """pdf_subrange at each t over [t0,t1] of a 1-D Simpson region over [0,1] with these nodes."""
        return self._simpson_1d("simpson_pdf_1d", nodes, t, t0, t1)

    def simpson_sample_1d(self, nodes, s, t0, t1):
        """sample_subrange over [t0,t1] for each uniform s, same region."""
        return self._simpson_1d("simpson_sample_1d", nodes, s, t0, t1)


_port = None



def port() -> Oracle:
    """The C++ restatement (built on demand)."""
    global _port
    if _port is None:
        build()
        _port = Oracle(PORT_SO, "orc_")
    return _port


def reference() -> Oracle | None:
    """The unmodified reference driver, if it was built here (oracle/Makefile `ref`)."""
    if not os.path.exists(REF_SO):
        return None
    return Oracle(REF_SO, "ref_")
