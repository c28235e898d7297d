"""Python host interface of the GB300 domain propagator (ctypes over libgdp_gb300.so).

Two layers:

* ``propagateGPUAtomic`` / ``propagateGPUReduction`` mirror the reference's
  Python driver (fileReader/GPUDomPropInterface.py:35-145): same names, same
  argument order ``(n_vars, n_cons, nnz, csr_col_indices, csr_row_ptrs,
  csr_vals, lhss, rhss, lbs, ubs, vartypes, ...)``, same return value
  ``(lbs, ubs)`` as lists. They call the reference-named C symbols.
* ``Context`` / ``propagate`` use the extended C API (gdp_ext.h) with numpy
  arrays, options and statistics (rounds, infeasibility, device time).

The library must be built (``build.build()``); there is no fallback: loading
fails loudly when libgdp_gb300.so is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path
from typing import List, Optional, Tuple

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libgdp_gb300.so"

GDP_OKAY, GDP_ERROR, GDP_NOTIMPLEMENTED = 1, 0, -18
CPU_LOOP, GPU_LOOP, MEGAKERNEL = 0, 1, 2
GDP_BINARY, GDP_INTEGER, GDP_CONTINUOUS = 0, 1, 3
GDP_INF = 1e20


class GDPError(RuntimeError):
    pass


class MpsProblem(C.Structure):
    _fields_ = [("n_cons", C.c_int), ("n_vars", C.c_int), ("nnz", C.c_int),
                ("row_ptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int)),
                ("val", C.POINTER(C.c_double)), ("lhs", C.POINTER(C.c_double)), ("rhs", C.POINTER(C.c_double)),
                ("lb", C.POINTER(C.c_double)), ("ub", C.POINTER(C.c_double)), ("vartype", C.POINTER(C.c_int))]


class TuneTrial(C.Structure):
    _fields_ = [("thread_row_max", C.c_int), ("split_tile", C.c_int), ("sync_type", C.c_int),
                ("ctas_per_sm", C.c_int), ("rounds", C.c_int), ("cta_threads", C.c_int), ("ms", C.c_double)]


class Options(C.Structure):
    _fields_ = [
        ("max_rounds", C.c_int),
        ("sync_type", C.c_int),
        ("thread_row_max", C.c_int),
        ("split_tile", C.c_int),
        ("device", C.c_int),
        ("use_marking", C.c_int),
        ("ctas_per_sm", C.c_int),
        ("barrier_wait_kcycles", C.c_int),
        ("cta_threads", C.c_int),
        ("reserved", C.c_int * 4),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("rounds", C.c_int),
        ("converged", C.c_int),
        ("infeasible", C.c_int),
        ("infeasible_var", C.c_int),
        ("device_error", C.c_int),
        ("kernel_launches", C.c_int),
        ("changed_vars", C.c_longlong),
        ("rows_processed", C.c_longlong),
        ("nnz_processed", C.c_longlong),
        ("bytes_algorithmic", C.c_double),
        ("device_ms", C.c_double),
        ("total_ms", C.c_double),
        ("nnz_exact", C.c_longlong),
        ("rows_deferred", C.c_longlong),
        ("full_rounds", C.c_int),
        ("infeasible_row", C.c_int),
        ("divisions", C.c_longlong),
        ("rows_exact", C.c_longlong),
        ("rows_go", C.c_longlong),
        ("rows_seqmax", C.c_longlong),
        ("rows_drift", C.c_longlong),
        ("nnz_drift", C.c_longlong),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib: Optional[C.CDLL] = None

_P_INT = C.POINTER(C.c_int)
_P_DBL = C.POINTER(C.c_double)
_LEGACY_ARGS = [C.c_int, C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL, _P_DBL, _P_INT]


def load_library(path: Optional[os.PathLike] = None, make_default: bool = False) -> C.CDLL:
    """Loads libgdp_gb300.so (once) and declares the C signatures. A library
    at another path (the phase-timer build) is loaded as given, and becomes the
    one every later call of this module uses with make_default=True."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise GDPError(f"{p} is missing: build it with gpu-domain-propagator_gb300/build.py "
                       "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    lib.gdp_last_error.restype = C.c_char_p
    lib.gdp_default_options.argtypes = [C.POINTER(Options)]
    lib.gdp_context_create.argtypes = [C.c_int, C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL,
                                       _P_INT, C.POINTER(Options), C.POINTER(C.c_void_p)]
    lib.gdp_context_destroy.argtypes = [C.c_void_p]
    lib.gdp_propagate.argtypes = [C.c_void_p, _P_DBL, _P_DBL, C.POINTER(Stats)]
    lib.gdp_propagate_into.argtypes = [C.c_void_p, _P_DBL, _P_DBL, _P_DBL, _P_DBL, C.POINTER(Stats)]
    lib.gdp_propagate_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Stats)]
    lib.gdp_context_set_options.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.gdp_context_layout.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    lib.gdp_propagate_once.argtypes = _LEGACY_ARGS + [C.POINTER(Options), C.POINTER(Stats)]
    lib.propagateConstraintsGPUAtomicDouble.argtypes = _LEGACY_ARGS + [C.c_int]
    lib.propagateConstraintsGPUReductionDouble.argtypes = _LEGACY_ARGS
    lib.gdp_propagate_noalloc.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 8 + \
        [C.c_int, C.c_void_p, C.POINTER(Stats)]
    lib.gdp_propagate_noalloc.restype = C.c_int
    _PP_INT, _PP_DBL = C.POINTER(_P_INT), C.POINTER(_P_DBL)
    lib.gdp_batch_create.argtypes = [C.c_int, _P_INT, _P_INT, _P_INT, _PP_INT, _PP_INT, _PP_DBL, _PP_DBL,
                                     _PP_DBL, _PP_INT, C.POINTER(Options), C.POINTER(C.c_void_p)]
    lib.gdp_batch_create_nodes.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
    lib.gdp_batch_propagate.argtypes = [C.c_void_p, _PP_DBL, _PP_DBL, C.POINTER(Stats), C.POINTER(Stats)]
    lib.gdp_batch_propagate_into.argtypes = [C.c_void_p, _PP_DBL, _PP_DBL, _PP_DBL, _PP_DBL, C.POINTER(Stats),
                                             C.POINTER(Stats)]
    lib.gdp_batch_uses_graph.argtypes = [C.c_void_p]
    lib.gdp_batch_destroy.argtypes = [C.c_void_p]
    for name in ("gdp_batch_create", "gdp_batch_create_nodes", "gdp_batch_propagate", "gdp_batch_propagate_into",
                 "gdp_batch_uses_graph", "gdp_batch_destroy"):
        getattr(lib, name).restype = C.c_int
    _P_F = C.POINTER(C.c_float)
    lib.gdp_mlp_create.argtypes = [C.c_ulonglong, C.c_int, C.POINTER(C.c_void_p)]
    lib.gdp_mlp_destroy.argtypes = [C.c_void_p]
    lib.gdp_mlp_get_params.argtypes = [C.c_void_p, _P_F]
    lib.gdp_mlp_set_params.argtypes = [C.c_void_p, _P_F]
    lib.gdp_mlp_forward.argtypes = [C.c_void_p, C.c_int, _P_F, _P_F]
    lib.gdp_mlp_gradient.argtypes = [C.c_void_p, C.c_int, _P_F, _P_F, _P_F, _P_F, _P_F]
    lib.gdp_mlp_train.argtypes = [C.c_void_p, C.c_int, _P_F, _P_F, _P_F, C.c_int, C.c_int, C.c_float,
                                  C.c_ulonglong, _P_F]
    lib.gdp_context_set_model.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_int]
    lib.gdp_batch_set_model.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_int]
    lib.gdp_autotune.argtypes = _LEGACY_ARGS[:8] + [_P_DBL, _P_DBL, _P_INT, C.POINTER(Options), C.c_int,
                                                    C.POINTER(Options), C.POINTER(C.c_double),
                                                    C.POINTER(TuneTrial), C.c_int, C.POINTER(C.c_int)]
    lib.gdp_autotune_clear_cache.restype = C.c_int
    lib.gdp_autotune.restype = C.c_int
    lib.gdp_mps_parse.argtypes = [C.c_char_p, C.c_longlong, C.POINTER(MpsProblem)]
    lib.gdp_mps_parse.restype = C.c_int
    lib.gdp_mps_free.argtypes = [C.POINTER(MpsProblem)]
    lib.gdp_mps_free.restype = None
    _P_U64 = C.POINTER(C.c_ulonglong)
    lib.gdp_phase_timers_read.argtypes = [_P_U64, _P_U64, _P_U64, C.c_int]
    lib.gdp_phase_timers_read.restype = C.c_int
    lib.gdp_phase_timers_clear.argtypes = []
    lib.gdp_phase_timers_clear.restype = C.c_int
    lib.gdp_context_trace.argtypes = [C.c_void_p, _P_DBL, _P_DBL, C.c_int, _P_F, _P_F, C.POINTER(C.c_int),
                                      C.POINTER(Stats)]
    for name in ("gdp_mlp_create", "gdp_mlp_destroy", "gdp_mlp_get_params", "gdp_mlp_set_params",
                 "gdp_mlp_forward", "gdp_mlp_gradient", "gdp_mlp_train", "gdp_context_set_model",
                 "gdp_context_trace", "gdp_batch_set_model"):
        getattr(lib, name).restype = C.c_int
    for name in ("gdp_default_options", "gdp_context_create", "gdp_context_destroy", "gdp_propagate",
                 "gdp_propagate_device", "gdp_context_set_options", "gdp_context_layout",
                 "gdp_propagate_once", "propagateConstraintsGPUAtomicDouble",
                 "propagateConstraintsGPUReductionDouble"):
        getattr(lib, name).restype = C.c_int
    if path is None or make_default:
        _lib = lib
    return lib


def last_error() -> str:
    return load_library().gdp_last_error().decode(errors="replace")


def release_cached_memory() -> None:
    """Frees the device memory that destroyed contexts and batches left cached
    for later ones (gdp_release_cached_memory)."""
    _check(load_library().gdp_release_cached_memory(), "gdp_release_cached_memory")


def _check(rc: int, what: str) -> None:
    if rc != GDP_OKAY:
        raise GDPError(f"{what} returned {rc}: {last_error()}")


def default_options(**kw) -> Options:
    o = Options()
    load_library().gdp_default_options(C.byref(o))
    for k, v in kw.items():
        if v is not None:
            setattr(o, k, int(v))
    return o


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _pi(a: np.ndarray):
    return a.ctypes.data_as(_P_INT)


def _pd(a: np.ndarray):
    return a.ctypes.data_as(_P_DBL)


@dataclass
class MIP:
    """A MIP in the reference's CSR argument convention."""
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    lhs: np.ndarray
    rhs: np.ndarray
    lb: np.ndarray
    ub: np.ndarray
    vartype: np.ndarray

    @property
    def m(self) -> int:
        return len(self.row_ptr) - 1

    @property
    def n(self) -> int:
        return len(self.lb)

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1]) if len(self.row_ptr) else 0

    def normalized(self) -> "MIP":
        return MIP(_i32(self.row_ptr), _i32(self.col), _f64(self.val), _f64(self.lhs), _f64(self.rhs),
                   _f64(self.lb), _f64(self.ub), _i32(self.vartype))


def propagate(mip: MIP, sync_type: int = CPU_LOOP, max_rounds: int = 0, thread_row_max: int = 0,
              split_tile: int = 0, lb=None, ub=None, use_marking: int = -1) -> Tuple[np.ndarray, np.ndarray, dict]:
    """One-shot propagation (upload, propagate, download) with statistics."""
    lib = load_library()
    p = mip.normalized()
    if p.m and p.n and p.nnz:  # a context for one call (the library copies the bounds in)
        with Context(p, sync_type=sync_type, max_rounds=max_rounds, thread_row_max=thread_row_max,
                     split_tile=split_tile, use_marking=use_marking) as ctx:
            return ctx.propagate(lb, ub)
    lbo = _f64(p.lb if lb is None else lb).copy()
    ubo = _f64(p.ub if ub is None else ub).copy()
    o = default_options(sync_type=sync_type, max_rounds=max_rounds, thread_row_max=thread_row_max,
                        split_tile=split_tile, use_marking=use_marking)
    st = Stats()
    rc = lib.gdp_propagate_once(p.m, p.n, p.nnz, _pi(p.col), _pi(p.row_ptr), _pd(p.val), _pd(p.lhs),
                                _pd(p.rhs), _pd(lbo), _pd(ubo), _pi(p.vartype), C.byref(o), C.byref(st))
    _check(rc, "gdp_propagate_once")
    return lbo, ubo, st.as_dict()


class Context:
    """Persistent device context: upload once, propagate many bound vectors."""

    def __init__(self, mip: MIP, sync_type: int = CPU_LOOP, max_rounds: int = 0, thread_row_max: int = 0,
                 split_tile: int = 0, use_marking: int = -1, ctas_per_sm: int = 0, barrier_wait_kcycles: int = 0,
                 cta_threads: int = 0):
        self._lib = load_library()
        self.mip = mip.normalized()
        p = self.mip
        o = default_options(sync_type=sync_type, max_rounds=max_rounds, thread_row_max=thread_row_max,
                            split_tile=split_tile, use_marking=use_marking, ctas_per_sm=ctas_per_sm,
                            barrier_wait_kcycles=barrier_wait_kcycles, cta_threads=cta_threads)
        h = C.c_void_p()
        rc = self._lib.gdp_context_create(p.m, p.n, p.nnz, _pi(p.col), _pi(p.row_ptr), _pd(p.val),
                                          _pd(p.lhs), _pd(p.rhs), _pi(p.vartype), C.byref(o), C.byref(h))
        _check(rc, "gdp_context_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gdp_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_options(self, max_rounds: int = 0, sync_type: int = CPU_LOOP) -> None:
        _check(self._lib.gdp_context_set_options(self._h, int(max_rounds), int(sync_type)),
               "gdp_context_set_options")

    def layout(self) -> dict:
        out = (C.c_longlong * 6)()
        _check(self._lib.gdp_context_layout(self._h, out), "gdp_context_layout")
        keys = ("thread_rows", "slices", "split_rows", "split_tiles", "sell_elements", "mega_grid")
        return dict(zip(keys, [int(v) for v in out]))

    def propagate(self, lb=None, ub=None) -> Tuple[np.ndarray, np.ndarray, dict]:
        lbi = _f64(self.mip.lb if lb is None else lb)
        ubi = _f64(self.mip.ub if ub is None else ub)
        if len(lbi) != self.mip.n or len(ubi) != self.mip.n:
            raise GDPError(f"expected {self.mip.n} bounds")
        lbo, ubo = np.empty_like(lbi), np.empty_like(ubi)  # the library copies the inputs in
        st = Stats()
        _check(self._lib.gdp_propagate_into(self._h, _pd(lbi), _pd(ubi), _pd(lbo), _pd(ubo), C.byref(st)),
               "gdp_propagate_into")
        return lbo, ubo, st.as_dict()

    def set_model(self, model, threshold: float = 0.0, min_len: int = 8) -> None:
        """Learned marking with `model` (an Mlp; None turns it off), a logit
        threshold, and the shortest row length the model decides for."""
        self._model = model
        _check(self._lib.gdp_context_set_model(self._h, model._h if model is not None else None,
                                               float(threshold), int(min_len)), "gdp_context_set_model")

    def trace(self, lb=None, ub=None, capacity: int = 1 << 20):
        """Trace propagation: returns (features [k, 16], labels [k], lb, ub, stats)."""
        lbo = _f64(self.mip.lb if lb is None else lb).copy()
        ubo = _f64(self.mip.ub if ub is None else ub).copy()
        x = np.zeros((max(capacity, 1), 16), np.float32)
        y = np.zeros(max(capacity, 1), np.float32)
        k = C.c_int()
        st = Stats()
        _check(self._lib.gdp_context_trace(self._h, _pd(lbo), _pd(ubo), int(capacity),
                                           x.ctypes.data_as(C.POINTER(C.c_float)),
                                           y.ctypes.data_as(C.POINTER(C.c_float)), C.byref(k), C.byref(st)),
               "gdp_context_trace")
        return x[:k.value].copy(), y[:k.value].copy(), lbo, ubo, st.as_dict()

    def propagate_device(self, d_lb_ptr: int, d_ub_ptr: int, stream_ptr: int = 0) -> dict:
        """Propagates device-resident bounds (raw device pointers, e.g. torch data_ptr())."""
        st = Stats()
        _check(self._lib.gdp_propagate_device(self._h, C.c_void_p(d_lb_ptr), C.c_void_p(d_ub_ptr),
                                              C.c_void_p(stream_ptr or None), C.byref(st)),
               "gdp_propagate_device")
        return st.as_dict()


def parse_mps(text: bytes) -> MIP:
    """gdp_mps_parse on MPS text: a MIP in the reference's CSR convention."""
    lib = load_library()
    out = MpsProblem()
    _check(lib.gdp_mps_parse(text, len(text), C.byref(out)), "gdp_mps_parse")
    try:
        def arr(ptr, cnt, dt):
            return np.ctypeslib.as_array(ptr, shape=(max(cnt, 1),))[:cnt].astype(dt, copy=True)
        m, n, nnz = out.n_cons, out.n_vars, out.nnz
        return MIP(arr(out.row_ptr, m + 1, np.int32), arr(out.col, nnz, np.int32), arr(out.val, nnz, np.float64),
                   arr(out.lhs, m, np.float64), arr(out.rhs, m, np.float64), arr(out.lb, n, np.float64),
                   arr(out.ub, n, np.float64), arr(out.vartype, n, np.int32))
    finally:
        lib.gdp_mps_free(C.byref(out))


def read_mps(path) -> MIP:
    """Reads an .mps or .mps.gz file."""
    import gzip
    p = os.fspath(path)
    data = gzip.open(p, "rb").read() if p.endswith(".gz") else open(p, "rb").read()
    return parse_mps(data)


def autotune(mip: MIP, repeats: int = 2, max_rounds: int = 0, use_marking: int = -1):
    """gdp_autotune: the fastest (thread_row_max, split_tile, sync_type,
    ctas_per_sm, cta_threads) for `mip`, cached per problem shape. Returns
    (options dict, best ms, list of trials)."""
    lib = load_library()
    p = mip.normalized()
    base = default_options(max_rounds=max_rounds, use_marking=use_marking)
    best = Options()
    ms = C.c_double()
    trials = (TuneTrial * 64)()
    k = C.c_int()
    rc = lib.gdp_autotune(p.m, p.n, p.nnz, _pi(p.col), _pi(p.row_ptr), _pd(p.val), _pd(p.lhs), _pd(p.rhs),
                          _pd(p.lb), _pd(p.ub), _pi(p.vartype), C.byref(base), int(repeats), C.byref(best),
                          C.byref(ms), trials, 64, C.byref(k))
    _check(rc, "gdp_autotune")
    opts = {name: getattr(best, name) for name in ("thread_row_max", "split_tile", "sync_type", "ctas_per_sm",
                                                   "cta_threads", "use_marking", "max_rounds")}
    table = [{name: getattr(trials[i], name) for name, _ in TuneTrial._fields_} for i in range(k.value)]
    return opts, ms.value, table


def autotune_clear_cache() -> None:
    _check(load_library().gdp_autotune_clear_cache(), "gdp_autotune_clear_cache")


class Batch:
    """Many problems, or many node bound vectors of one Context's problem,
    propagated together in one persistent launch (gdp_batch_*)."""

    def __init__(self, handle, lib, sizes, keep=None):
        self._h, self._lib, self._sizes, self._keep = handle, lib, sizes, keep

    @classmethod
    def instances(cls, mips, max_rounds: int = 0, thread_row_max: int = 0, split_tile: int = 0,
                  use_marking: int = -1, ctas_per_sm: int = 0, autotune: bool = False) -> "Batch":
        """autotune: pick thread_row_max, split_tile and ctas_per_sm with
        gdp_autotune on the largest member (its schedule applies to the batch loop)."""
        lib = load_library()
        ps = [m.normalized() for m in mips]
        k = len(ps)
        tuned = None
        if autotune and ps:
            big = max(ps, key=lambda p: p.nnz)
            tuned, _, _ = globals()["autotune"](big, repeats=1, max_rounds=max_rounds, use_marking=use_marking)
            thread_row_max, split_tile = tuned["thread_row_max"], tuned["split_tile"]
            # the batch loop runs 256-thread CTAs: the tuned warps per SM, in its CTAs
            ctas_per_sm = (max(1, tuned["ctas_per_sm"] * tuned["cta_threads"] // 256)
                           if tuned["ctas_per_sm"] > 0 else 0)
        arr_i = lambda xs: (C.c_int * k)(*xs)
        col = (_P_INT * k)(*[_pi(p.col) for p in ps])
        rp = (_P_INT * k)(*[_pi(p.row_ptr) for p in ps])
        val = (_P_DBL * k)(*[_pd(p.val) for p in ps])
        lhs = (_P_DBL * k)(*[_pd(p.lhs) for p in ps])
        rhs = (_P_DBL * k)(*[_pd(p.rhs) for p in ps])
        vt = (_P_INT * k)(*[_pi(p.vartype) for p in ps])
        o = default_options(max_rounds=max_rounds, thread_row_max=thread_row_max, split_tile=split_tile,
                            use_marking=use_marking, ctas_per_sm=ctas_per_sm)
        h = C.c_void_p()
        rc = lib.gdp_batch_create(k, arr_i([p.m for p in ps]), arr_i([p.n for p in ps]),
                                  arr_i([p.nnz for p in ps]), col, rp, val, lhs, rhs, vt, C.byref(o), C.byref(h))
        _check(rc, "gdp_batch_create")
        b = cls(h, lib, [p.n for p in ps], keep=ps)
        b.mips = ps
        b.tuned = tuned
        return b

    @classmethod
    def nodes(cls, ctx: "Context", n_nodes: int) -> "Batch":
        lib = load_library()
        h = C.c_void_p()
        _check(lib.gdp_batch_create_nodes(ctx._h, int(n_nodes), C.byref(h)), "gdp_batch_create_nodes")
        return cls(h, lib, [ctx.mip.n] * int(n_nodes), keep=ctx)

    @property
    def uses_graph(self) -> bool:
        return bool(self._lib.gdp_batch_uses_graph(self._h))

    def set_model(self, model, threshold: float = 0.0, min_len: int = 8) -> None:
        """Learned marking for every member of an instance batch (`model` an
        Mlp, None turns it off): each member takes the rounds of its own
        learned propagation (Context.set_model) inside the one launch."""
        self._model = model
        _check(self._lib.gdp_batch_set_model(self._h, model._h if model is not None else None, float(threshold),
                                             int(min_len)), "gdp_batch_set_model")

    def propagate(self, lbs, ubs):
        """lbs, ubs: one array per member. Returns (lbs, ubs, member stats, total stats)."""
        k = len(self._sizes)
        lbi = [_f64(x) for x in lbs]
        ubi = [_f64(x) for x in ubs]
        for i in range(k):
            if len(lbi[i]) != self._sizes[i] or len(ubi[i]) != self._sizes[i]:
                raise GDPError(f"member {i}: expected {self._sizes[i]} bounds")
        lbo = [np.empty_like(x) for x in lbi]  # written by the library (host threads)
        ubo = [np.empty_like(x) for x in ubi]
        arr = lambda xs: (_P_DBL * k)(*[_pd(x) for x in xs])
        st = (Stats * k)()
        tot = Stats()
        _check(self._lib.gdp_batch_propagate_into(self._h, arr(lbi), arr(ubi), arr(lbo), arr(ubo), st,
                                                  C.byref(tot)), "gdp_batch_propagate_into")
        return lbo, ubo, [s.as_dict() for s in st], tot.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gdp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MLP_FEATURES = 16
MLP_PARAMS = 5313


def _pf(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class Mlp:
    """The row-marking MLP (gdp_mlp_*): 16 -> 64 -> 64 -> 1, BF16/FP32, on the GPU."""

    def __init__(self, seed: int = 0, device: int = 0):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.gdp_mlp_create(int(seed), int(device), C.byref(h)), "gdp_mlp_create")
        self._h = h

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(MLP_PARAMS, np.float32)
        _check(self._lib.gdp_mlp_get_params(self._h, _pf(out)), "gdp_mlp_get_params")
        return out

    @params.setter
    def params(self, p) -> None:
        p = _f32(p)
        if p.size != MLP_PARAMS:
            raise GDPError(f"expected {MLP_PARAMS} parameters")
        _check(self._lib.gdp_mlp_set_params(self._h, _pf(p)), "gdp_mlp_set_params")

    def forward(self, x) -> np.ndarray:
        x = _f32(x).reshape(-1, MLP_FEATURES)
        z = np.zeros(len(x), np.float32)
        _check(self._lib.gdp_mlp_forward(self._h, len(x), _pf(x), _pf(z)), "gdp_mlp_forward")
        return z

    def gradient(self, x, y, w=None):
        x = _f32(x).reshape(-1, MLP_FEATURES)
        y = _f32(y)
        w = _f32(np.ones(len(x)) if w is None else w)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        _check(self._lib.gdp_mlp_gradient(self._h, len(x), _pf(x), _pf(y), _pf(w), _pf(g), C.byref(loss)),
               "gdp_mlp_gradient")
        return float(loss.value), g

    def train(self, x, y, w=None, epochs: int = 5, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        x = _f32(x).reshape(-1, MLP_FEATURES)
        y = _f32(y)
        w = _f32(np.ones(len(x)) if w is None else w)
        loss = C.c_float()
        _check(self._lib.gdp_mlp_train(self._h, len(x), _pf(x), _pf(y), _pf(w), int(epochs), int(batch),
                                       float(lr), int(seed), C.byref(loss)), "gdp_mlp_train")
        return float(loss.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gdp_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NOALLOC_MAX_VARS = 1 << 20


def propagate_noalloc(n_cons: int, n_vars: int, nnz: int, d_col: int, d_row_ptr: int, d_val: int, d_lhs: int,
                      d_rhs: int, d_lb: int, d_ub: int, d_vartype: int, max_rounds: int = 0,
                      stream: int = 0) -> dict:
    """gdp_propagate_noalloc on device pointers (ints, e.g. torch data_ptr()):
    the library allocates nothing; bounds d_lb/d_ub are updated in place."""
    st = Stats()
    rc = load_library().gdp_propagate_noalloc(int(n_cons), int(n_vars), int(nnz), *(C.c_void_p(p) for p in (
        d_col, d_row_ptr, d_val, d_lhs, d_rhs, d_lb, d_ub, d_vartype)), int(max_rounds),
        C.c_void_p(stream or None), C.byref(st))
    _check(rc, "gdp_propagate_noalloc")
    return st.as_dict()


# ---- mirror of the reference's Python driver (fileReader/GPUDomPropInterface.py) ----

def _legacy_arrays(n_vars, n_cons, nnz, csr_col_indices, csr_row_ptrs, csr_vals, lhss, rhss, lbs, ubs,
                   vartypes):
    # same length checks as the reference's check_input (GPUDomPropInterface.py:12-32)
    assert len(csr_col_indices) == nnz
    assert len(csr_row_ptrs) == n_cons + 1
    assert len(csr_vals) == nnz
    assert len(lhss) == n_cons
    assert len(rhss) == n_cons
    assert len(lbs) == n_vars
    assert len(ubs) == n_vars
    assert len(vartypes) == n_vars
    return (_i32(csr_col_indices), _i32(csr_row_ptrs), _f64(csr_vals), _f64(lhss), _f64(rhss),
            _f64(lbs).copy(), _f64(ubs).copy(), _i32(vartypes))


def propagateGPUAtomic(n_vars: int, n_cons: int, nnz: int, csr_col_indices, csr_row_ptrs, csr_vals, lhss,
                       rhss, lbs, ubs, vartypes, synctype: int = 0,
                       datatype=C.c_double) -> Tuple[List[float], List[float]]:
    """Reference fileReader/GPUDomPropInterface.py:90-145, on this library."""
    if datatype is not C.c_double:
        raise GDPError("only c_double is supported (FP64 propagation)")
    lib = load_library()
    col, rp, val, lhs, rhs, lbo, ubo, vt = _legacy_arrays(n_vars, n_cons, nnz, csr_col_indices, csr_row_ptrs,
                                                          csr_vals, lhss, rhss, lbs, ubs, vartypes)
    rc = lib.propagateConstraintsGPUAtomicDouble(n_cons, n_vars, nnz, _pi(col), _pi(rp), _pd(val), _pd(lhs),
                                                 _pd(rhs), _pd(lbo), _pd(ubo), _pi(vt), int(synctype))
    _check(rc, "propagateConstraintsGPUAtomicDouble")
    return list(lbo), list(ubo)


def propagateGPUReduction(n_vars: int, n_cons: int, nnz: int, csr_col_indices, csr_row_ptrs, csr_vals, lhss,
                          rhss, lbs, ubs, vartypes, datatype=C.c_double) -> Tuple[List[float], List[float]]:
    """Reference fileReader/GPUDomPropInterface.py:35-87, on this library."""
    if datatype is not C.c_double:
        raise GDPError("only c_double is supported (FP64 propagation)")
    lib = load_library()
    col, rp, val, lhs, rhs, lbo, ubo, vt = _legacy_arrays(n_vars, n_cons, nnz, csr_col_indices, csr_row_ptrs,
                                                          csr_vals, lhss, rhss, lbs, ubs, vartypes)
    rc = lib.propagateConstraintsGPUReductionDouble(n_cons, n_vars, nnz, _pi(col), _pi(rp), _pd(val),
                                                    _pd(lhs), _pd(rhs), _pd(lbo), _pd(ubo), _pi(vt))
    _check(rc, "propagateConstraintsGPUReductionDouble")
    return list(lbo), list(ubo)
