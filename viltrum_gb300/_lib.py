"""ctypes binding of libviltrum_cuda.so (include/viltrum_cuda.h).

The library is built in-tree (viltrum_gb300/build.py).  There is no CPU fallback: if the library
is missing or no CUDA device is present, loading or creating a context raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libviltrum_cuda.so")

VCU_MAX_DIM = 6
VCU_MAX_DIMBINS = 4
MEM_HOST, MEM_DEVICE = 0, 1
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "QUEUE_OVERFLOW", 4: "DEVICE_TIMEOUT", 5: "NAN_DETECTED",
          6: "CUDA_ERROR", 7: "NO_DEVICE", 8: "UNSUPPORTED"}
FLAG_NAN, FLAG_TIMEOUT, FLAG_OVERFLOW = 1, 2, 4

EXPORTS = ["vcu_abi_version", "vcu_create", "vcu_destroy", "vcu_last_error", "vcu_channels", "vcu_eval",
           "vcu_per_bin_monte_carlo", "vcu_per_bin_monte_carlo_replay", "vcu_per_bin_monte_carlo_accumulate",
           "vcu_per_bin_adaptive_nested",
           "vcu_control_variates", "vcu_learned_control_variates", "vcu_mlp_eval", "vcu_integrate_batch",
           "vcu_integrate_batch_resident", "vcu_adaptive_iterations_global", "vcu_adaptive_tolerance",
           "vcu_cv_replay_width", "vcu_set_device_memory_limit", "vcu_device_memory_held", "vcu_per_bin_fubini"]
BATCH_MONTE_CARLO, BATCH_NESTED = 0, 1
CV_OPTIMIZE, CV_FIXED = 0, 1
RR_UNIFORM, RR_INTEGRAL, RR_ERROR, RR_PDF = 0, 1, 2, 3  # residual region choice
RS_UNIFORM, RS_IMPORTANCE, RS_RUSSIAN_ROULETTE, RS_MIS = 0, 1, 2, 3  # residual point sampling


def cv_replay_width(dim: int, sampling: int = RS_UNIFORM) -> int:
    """Floats per residual sample of vcu_control_variates' replay records."""
    return 1 + dim + (1 if sampling == RS_RUSSIAN_ROULETTE else 1 + dim if sampling == RS_MIS else 0)


class VcuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


class Integrand(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("n_params", ctypes.c_int32), ("params", ctypes.POINTER(ctypes.c_float))]


class Problem(ctypes.Structure):
    _fields_ = [("f", Integrand), ("dim", ctypes.c_int32), ("dimbins", ctypes.c_int32),
                ("range_min", ctypes.c_float * VCU_MAX_DIM), ("range_max", ctypes.c_float * VCU_MAX_DIM),
                ("resolution", ctypes.c_uint64 * VCU_MAX_DIMBINS), ("mem", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Nested(ctypes.Structure):
    _fields_ = [("rule_hi", ctypes.c_int32), ("rule_lo", ctypes.c_int32), ("heuristic", ctypes.c_int32),
                ("metric", ctypes.c_int32), ("size_weight", ctypes.c_double), ("min_size", ctypes.c_double),
                ("min_val", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("evaluations", ctypes.c_uint64), ("regions", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint32), ("flags", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class CvOpts(ctypes.Structure):
    _fields_ = [("samples_per_bin", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("weight", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("alpha", ctypes.c_double), ("rr", ctypes.c_int32),
                ("sampling", ctypes.c_int32), ("rr_factor", ctypes.c_float), ("reserved2", ctypes.c_int32),
                ("mis_power", ctypes.c_double), ("mis_cutoff", ctypes.c_double), ("fubini_dims", ctypes.c_int32),
                ("tail_samples", ctypes.c_uint32), ("variance", ctypes.c_void_p)]


FUBINI_MONTE_CARLO, FUBINI_NESTED = 0, 1


class FubiniOpts(ctypes.Structure):
    """vcu_fubini"""
    _fields_ = [("dims", ctypes.c_int32), ("tail_samples", ctypes.c_uint32), ("tail_seed", ctypes.c_uint64),
                ("method", ctypes.c_int32), ("n_order", ctypes.c_int32), ("order", ctypes.c_int32 * (2 * VCU_MAX_DIM)),
                ("samples_per_bin", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("nested", Nested),
                ("iterations", ctypes.c_uint64)]

    @classmethod
    def make(cls, tail_samples, tail_seed, method, samples_per_bin=0, seed=0, nested=None, iterations=0, order=()):
        """order: (to, from) pairs of integrator_reorder; integrator_fubini({d0, d1}, ...) is ((0, d0), (1, d1))"""
        o = cls()
        o.dims = 2
        o.tail_samples = tail_samples
        o.tail_seed = tail_seed
        o.method = method
        o.samples_per_bin = samples_per_bin
        o.seed = seed
        if nested is not None:
            o.nested = nested
        o.iterations = iterations
        o.n_order = len(order)
        for k, (to, frm) in enumerate(order):
            o.order[2 * k] = to
            o.order[2 * k + 1] = frm
        return o


class LearnedOpts(ctypes.Structure):
    """vcu_learned.  Positional: samples_per_bin, seed, train_steps, batch, learning_rate,
    check_every, fallback, cells, theta_out, cells_unbinned, pilot, poly_bins, poly_variance."""
    _fields_ = [("samples_per_bin", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("train_steps", ctypes.c_uint32),
                ("batch", ctypes.c_uint32), ("learning_rate", ctypes.c_float), ("check_every", ctypes.c_uint32),
                ("fallback", ctypes.c_int32), ("cells", ctypes.c_int32), ("theta_out", ctypes.c_void_p),
                ("cells_unbinned", ctypes.c_int32), ("pilot", ctypes.c_uint32), ("poly_bins", ctypes.c_void_p),
                ("poly_variance", ctypes.c_void_p)]


class LearnedReport(ctypes.Structure):
    _fields_ = [("train_ms", ctypes.c_double), ("integral_ms", ctypes.c_double), ("residual_ms", ctypes.c_double),
                ("heldout_mse", ctypes.c_double), ("fallback_bins", ctypes.c_uint32),
                ("polynomial_bins", ctypes.c_uint32), ("train_steps_run", ctypes.c_uint32),
                ("nodes_per_bin", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchItem(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("method", ctypes.c_int32), ("budget", ctypes.c_uint64),
                ("seed", ctypes.c_uint64), ("range_min", ctypes.c_float * VCU_MAX_DIM),
                ("range_max", ctypes.c_float * VCU_MAX_DIM), ("n_params", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("params", ctypes.c_void_p)]


class BatchReport(ctypes.Structure):
    _fields_ = [("item_ms", ctypes.c_void_p), ("threads", ctypes.c_int32), ("blocks", ctypes.c_uint32),
                ("nested_regions", ctypes.c_uint64)]


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_int32), ("stream", ctypes.c_void_p)]


_lib = None
_lib_lock = threading.Lock()


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m viltrum_gb300.build` "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        f32p = ctypes.POINTER(ctypes.c_float)
        L.vcu_abi_version.restype = ctypes.c_int
        L.vcu_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Opts)]
        L.vcu_destroy.argtypes = [vp]
        L.vcu_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
        L.vcu_channels.argtypes = [ctypes.c_int32]
        L.vcu_set_device_memory_limit.argtypes = [vp, ctypes.c_uint64]
        L.vcu_per_bin_fubini.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(FubiniOpts), vp,
                                         ctypes.POINTER(Stats)]
        L.vcu_device_memory_held.argtypes = [vp]
        L.vcu_device_memory_held.restype = ctypes.c_uint64
        L.vcu_eval.argtypes = [vp, ctypes.POINTER(Integrand), ctypes.c_int32, vp, ctypes.c_int64, vp, ctypes.c_int32]
        L.vcu_per_bin_monte_carlo.argtypes = [vp, ctypes.POINTER(Problem), ctypes.c_uint64, ctypes.c_uint64, vp,
                                              ctypes.POINTER(Stats)]
        L.vcu_per_bin_monte_carlo_replay.argtypes = [vp, ctypes.POINTER(Problem), ctypes.c_uint64, vp, vp,
                                                     ctypes.POINTER(Stats)]
        L.vcu_per_bin_monte_carlo_accumulate.argtypes = [vp, ctypes.POINTER(Problem), ctypes.c_uint64,
                                                         ctypes.c_uint64, vp, vp, ctypes.POINTER(Stats)]
        L.vcu_per_bin_adaptive_nested.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(Nested),
                                                  ctypes.c_uint64, vp, vp, ctypes.POINTER(Stats)]
        L.vcu_control_variates.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(Nested), ctypes.c_uint64,
                                           ctypes.POINTER(CvOpts), vp, vp, vp, vp, ctypes.POINTER(Stats)]
        L.vcu_learned_control_variates.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(LearnedOpts), vp, vp,
                                                   ctypes.POINTER(LearnedReport), ctypes.POINTER(Stats)]
        L.vcu_mlp_eval.argtypes = [vp, ctypes.c_int32, vp, vp, vp, ctypes.c_int64, vp, vp]
        L.vcu_adaptive_iterations_global.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(Nested),
                                                     ctypes.c_uint64, vp, ctypes.POINTER(Stats)]
        L.vcu_adaptive_tolerance.argtypes = [vp, ctypes.POINTER(Problem), ctypes.POINTER(Nested), ctypes.c_float,
                                             ctypes.c_uint64, vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(Stats)]
        L.vcu_integrate_batch.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(Nested), ctypes.POINTER(BatchItem),
                                          ctypes.c_uint64, vp, ctypes.c_int32, ctypes.POINTER(BatchReport),
                                          ctypes.POINTER(Stats)]
        L.vcu_integrate_batch_resident.argtypes = [vp, vp, ctypes.c_int32, ctypes.POINTER(BatchReport),
                                                   ctypes.POINTER(Stats)]
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        del f32p
        _lib = L
        return L


def _ptr(a) -> int | None:
    """Address of a numpy array, torch tensor or raw integer pointer."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


class Context:
    """One vcu_ctx: a CUDA stream plus the library's device buffers on one device."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        h = ctypes.c_void_p()
        opts = Opts(device, 0, stream)
        rc = self.lib.vcu_create(ctypes.byref(h), ctypes.byref(opts))
        if rc != 0:
            raise VcuError(rc, "vcu_create failed (no CUDA device or driver?)")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.vcu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(512)
        self.lib.vcu_last_error(self.handle, buf, 512)
        return buf.value.decode()

    def check(self, rc: int):
        if rc != 0:
            raise VcuError(rc, self.last_error())

    # ----------------------------------------------------------------- entry points
    @staticmethod
    def problem(kind, params, rmin, rmax, res, mem=MEM_HOST):
        params = np.ascontiguousarray(params if params is not None else np.zeros(0), dtype=np.float32)
        p = Problem()
        p.f = Integrand(int(kind), int(params.size),
                        params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if params.size else None)
        p.dim = len(rmin)
        p.dimbins = len(res)
        for d in range(len(rmin)):
            p.range_min[d] = float(rmin[d])
            p.range_max[d] = float(rmax[d])
        for d in range(len(res)):
            p.resolution[d] = int(res[d])
        p.mem = mem
        p._keep = params  # keep the parameter array alive with the struct
        return p

    def channels(self, kind: int) -> int:
        c = self.lib.vcu_channels(int(kind))
        if c < 0:
            raise VcuError(-c, f"unknown integrand kind {kind}")
        return c

    def eval(self, kind, params, x, mem=MEM_HOST, out=None):
        params = np.ascontiguousarray(params if params is not None else np.zeros(0), dtype=np.float32)
        f = Integrand(int(kind), int(params.size),
                      params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if params.size else None)
        if mem == MEM_HOST:
            x = np.ascontiguousarray(x, dtype=np.float32)
            npts, dim = x.shape
            out = np.empty((npts, self.channels(kind)), dtype=np.float32)
        else:
            npts, dim = x.shape
        self.check(self.lib.vcu_eval(self.handle, ctypes.byref(f), dim, _ptr(x), npts, _ptr(out), mem))
        return out

    def set_device_memory_limit(self, nbytes: int) -> None:
        """cap the bytes the context's device buffers may hold (0: no cap)"""
        self.check(self.lib.vcu_set_device_memory_limit(self.handle, int(nbytes)))

    def device_memory_held(self) -> int:
        return int(self.lib.vcu_device_memory_held(self.handle))

    def per_bin_monte_carlo(self, p: Problem, spp: int, seed: int, bins) -> Stats:
        st = Stats()
        self.check(self.lib.vcu_per_bin_monte_carlo(self.handle, ctypes.byref(p), spp, seed, _ptr(bins),
                                                    ctypes.byref(st)))
        return st

    def per_bin_monte_carlo_replay(self, p: Problem, spp: int, points, bins) -> Stats:
        st = Stats()
        self.check(self.lib.vcu_per_bin_monte_carlo_replay(self.handle, ctypes.byref(p), spp, _ptr(points),
                                                           _ptr(bins), ctypes.byref(st)))
        return st

    def per_bin_monte_carlo_accumulate(self, p: Problem, spp: int, seed: int, bins, points=None) -> Stats:
        """monte_carlo_per_bin_parallel: bins (read and written) += volume(range)/spp * sum f."""
        st = Stats()
        self.check(self.lib.vcu_per_bin_monte_carlo_accumulate(self.handle, ctypes.byref(p), spp, seed, _ptr(points),
                                                               _ptr(bins), ctypes.byref(st)))
        return st

    def per_bin_fubini(self, p: Problem, opts: "FubiniOpts", bins) -> Stats:
        """integrator_fubini<2>(per-bin integrator, monte_carlo(K)) with an optional reorder; assigns"""
        st = Stats()
        self.check(self.lib.vcu_per_bin_fubini(self.handle, ctypes.byref(p), ctypes.byref(opts), _ptr(bins),
                                               ctypes.byref(st)))
        return st

    def per_bin_adaptive_nested(self, p: Problem, nested: Nested, iterations: int, bins, trace=None) -> Stats:
        st = Stats()
        self.check(self.lib.vcu_per_bin_adaptive_nested(self.handle, ctypes.byref(p), ctypes.byref(nested),
                                                        iterations, _ptr(bins), _ptr(trace), ctypes.byref(st)))
        return st


def _cv_method(self, p: Problem, nested: Nested, iterations: int, cv: CvOpts, bins, approximation=None,
               regions=None, replay=None) -> Stats:
    st = Stats()
    self.check(self.lib.vcu_control_variates(self.handle, ctypes.byref(p), ctypes.byref(nested), iterations,
                                             ctypes.byref(cv), _ptr(replay), _ptr(bins), _ptr(approximation),
                                             _ptr(regions), ctypes.byref(st)))
    return st


Context.control_variates = _cv_method


def _global_method(self, p: Problem, nested: Nested, iterations: int, bins) -> Stats:
    """integrator_adaptive_iterations used directly: accumulates into bins"""
    st = Stats()
    self.check(self.lib.vcu_adaptive_iterations_global(self.handle, ctypes.byref(p), ctypes.byref(nested), iterations,
                                                       _ptr(bins), ctypes.byref(st)))
    return st


Context.adaptive_iterations_global = _global_method


def _tolerance_method(self, p: Problem, nested: Nested, tolerance: float, bins, max_regions: int = 0):
    """integrator_adaptive_tolerance: accumulates into bins; returns (stats, number of leaf regions)"""
    st = Stats()
    leaves = ctypes.c_uint64(0)
    self.check(self.lib.vcu_adaptive_tolerance(self.handle, ctypes.byref(p), ctypes.byref(nested), tolerance,
                                               max_regions, _ptr(bins), ctypes.byref(leaves), ctypes.byref(st)))
    return st, int(leaves.value)


Context.adaptive_tolerance = _tolerance_method


def _learned_method(self, p: Problem, opts: LearnedOpts, bins, network_integral=None):
    st, rep = Stats(), LearnedReport()
    self.check(self.lib.vcu_learned_control_variates(self.handle, ctypes.byref(p), ctypes.byref(opts), _ptr(bins),
                                                     _ptr(network_integral), ctypes.byref(rep), ctypes.byref(st)))
    return st, rep


def _mlp_eval_method(self, dim: int, theta, u, y=None, grad=False):
    theta = np.ascontiguousarray(theta, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    n = u.shape[0]
    out = np.empty(n, np.float32)
    g = np.empty(theta.size, np.float32) if grad else None
    yy = None if y is None else np.ascontiguousarray(y, np.float32)
    self.check(self.lib.vcu_mlp_eval(self.handle, dim, _ptr(theta), _ptr(u), _ptr(yy), n, _ptr(out), _ptr(g)))
    return out, g


def batch_items(items) -> tuple:
    """ctypes array of vcu_batch_item from dicts (dim, method, budget, seed, params, rmin, rmax); the
    parameter arrays are returned too, since the items point into them."""
    arr = (BatchItem * len(items))()
    keep = []
    for i, it in enumerate(items):
        b = arr[i]
        b.dim = int(it["dim"])
        b.method = int(it["method"])
        b.budget = int(it["budget"])
        b.seed = int(it.get("seed", 0))
        for d in range(b.dim):
            b.range_min[d] = float(it["rmin"][d])
            b.range_max[d] = float(it["rmax"][d])
        prm = it.get("params")
        if prm is not None:
            prm = np.ascontiguousarray(prm, np.float32)
            keep.append(prm)
            b.params = prm.ctypes.data
            b.n_params = prm.size
    return arr, keep


def _batch_method(self, kind: int, items, nested: Nested | None = None, results=None, mem=MEM_HOST,
                  item_ms=None):
    """vcu_integrate_batch over a list of item dicts (or a prepared (array, keep) pair)."""
    arr, keep = items if isinstance(items, tuple) else batch_items(items)
    n = len(arr)
    if results is None:
        results = np.empty(n, np.float32)
    st, rep = Stats(), BatchReport()
    rep.item_ms = _ptr(item_ms)
    self.check(self.lib.vcu_integrate_batch(self.handle, kind, ctypes.byref(nested) if nested is not None else None,
                                            arr, n, _ptr(results), mem, ctypes.byref(rep), ctypes.byref(st)))
    del keep
    return results, st, rep


def _batch_resident_method(self, results, mem=MEM_HOST, item_ms=None):
    st, rep = Stats(), BatchReport()
    rep.item_ms = _ptr(item_ms)
    self.check(self.lib.vcu_integrate_batch_resident(self.handle, _ptr(results), mem, ctypes.byref(rep),
                                                     ctypes.byref(st)))
    return st, rep


Context.learned_control_variates = _learned_method
Context.mlp_eval = _mlp_eval_method
Context.integrate_batch = _batch_method
Context.integrate_batch_resident = _batch_resident_method

_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
