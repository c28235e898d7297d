"""Seeded synthetic MIPs (ctypes over libgdpgen.so).

The reference benchmarks on MIPLIB 2017, which is not available here; these
generators produce instances with the same structure knobs (row-length skew,
coefficient ranges, integrality mix, infinite bounds) from a seed, identical
for every thread count.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from gdp import MIP

PKG = Path(__file__).resolve().parent
GEN_PATH = PKG / "lib" / "libgdpgen.so"


class _Instance(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("nnz", C.c_int),
                ("row_ptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int)), ("val", C.POINTER(C.c_double)),
                ("lhs", C.POINTER(C.c_double)), ("rhs", C.POINTER(C.c_double)),
                ("lb", C.POINTER(C.c_double)), ("ub", C.POINTER(C.c_double)),
                ("vartype", C.POINTER(C.c_int)), ("x0", C.POINTER(C.c_double))]


class GenParams(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("len_dist", C.c_int), ("len_min", C.c_int),
                ("len_max", C.c_int), ("zipf_s", C.c_double), ("n_dense_rows", C.c_int),
                ("dense_len", C.c_int), ("coef_dist", C.c_int), ("coef_min", C.c_double),
                ("coef_max", C.c_double), ("frac_int_coef", C.c_double), ("frac_int_vars", C.c_double),
                ("int_ub_max", C.c_int), ("frac_inf_vars", C.c_double), ("cont_bound_max", C.c_double),
                ("slack_max", C.c_double), ("frac_one_sided", C.c_double), ("frac_equality", C.c_double),
                ("seed", C.c_uint64)]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        if not GEN_PATH.exists():
            raise RuntimeError(f"{GEN_PATH} is missing: build it with gpu-domain-propagator_gb300/build.py")
        g = C.CDLL(str(GEN_PATH))
        g.gdp_gen_default_params.argtypes = [C.c_int, C.POINTER(GenParams)]
        g.gdp_gen_random_mip.argtypes = [C.POINTER(GenParams), C.POINTER(_Instance)]
        g.gdp_gen_cover_knapsack.argtypes = [C.c_int] * 8 + [C.c_uint64, C.POINTER(_Instance)]
        g.gdp_gen_chains.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                     C.c_uint64, C.POINTER(_Instance)]
        g.gdp_gen_free.argtypes = [C.POINTER(_Instance)]
        for f in ("gdp_gen_default_params", "gdp_gen_random_mip", "gdp_gen_cover_knapsack", "gdp_gen_chains"):
            getattr(g, f).restype = C.c_int
        _gen = g
    return _gen


def _take(inst: _Instance, with_x0: bool = False):
    m, n, nnz = inst.m, inst.n, inst.nnz

    def arr(ptr, count, dt):
        if count == 0:
            return np.zeros(0, dtype=dt)
        return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt, copy=True)

    mip = MIP(arr(inst.row_ptr, m + 1, np.int32), arr(inst.col, nnz, np.int32), arr(inst.val, nnz, np.float64),
              arr(inst.lhs, m, np.float64), arr(inst.rhs, m, np.float64), arr(inst.lb, n, np.float64),
              arr(inst.ub, n, np.float64), arr(inst.vartype, n, np.int32))
    x0 = arr(inst.x0, n, np.float64)
    _lib().gdp_gen_free(C.byref(inst))
    return (mip, x0) if with_x0 else mip


def default_params(workload: int) -> GenParams:
    p = GenParams()
    if _lib().gdp_gen_default_params(int(workload), C.byref(p)) != 0:
        raise ValueError(f"unknown workload {workload}")
    return p


def random_mip(workload: int = 0, seed: int = 0, m: int | None = None, n: int | None = None,
               with_x0: bool = False, **overrides):
    """Workload 0: small random MIP (m=2000, n=1500); workload 1: the large
    power-law MIP (m=2,000,000, n=1,500,000, Zipf(1.8) rows in [2, 20000] and
    32 rows of 100,000 non-zeros). m/n and any generator field can be
    overridden (for scaled-down parity cases)."""
    p = default_params(workload)
    p.seed = int(seed)
    if m is not None:
        p.m = int(m)
    if n is not None:
        p.n = int(n)
    for k, v in overrides.items():
        setattr(p, k, v)
    inst = _Instance()
    rc = _lib().gdp_gen_random_mip(C.byref(p), C.byref(inst))
    if rc != 0:
        raise RuntimeError(f"gdp_gen_random_mip failed ({rc})")
    return _take(inst, with_x0)


def cover_knapsack(n_cover_rows: int = 500_000, n_knap_rows: int = 50_000, n_bin: int = 400_000,
                   n_cont: int = 50_000, cover_min: int = 5, cover_max: int = 60, knap_min: int = 5,
                   knap_max: int = 60, seed: int = 0, with_x0: bool = False):
    inst = _Instance()
    rc = _lib().gdp_gen_cover_knapsack(n_cover_rows, n_knap_rows, n_bin, n_cont, cover_min, cover_max, knap_min,
                                       knap_max, int(seed), C.byref(inst))
    if rc != 0:
        raise RuntimeError(f"gdp_gen_cover_knapsack failed ({rc})")
    return _take(inst, with_x0)


def chains(m: int, n: int | None = None, chain_max: int = 5000, frac_int_vars: float = 0.6,
           frac_inf_vars: float = 0.15, infeasible: bool = False, seed: int = 0, with_x0: bool = False,
           frac_equality: float = 0.0):
    """Chain rows x_{i+1} - x_i <= c_i mixed 50/50 with power-law rows of the
    large random MIP. The power-law rows have no equality rows by default:
    equality rows tight at the generating point make the verdict depend on
    rounding (the reference's cpu_seq declares every such instance
    infeasible within a few rounds, Jacobi rounds about half of them), while
    without them exactly the members built infeasible (`infeasible`) are
    infeasible under both schedules."""
    n = int(0.75 * m) if n is None else n
    inst = _Instance()
    rc = _lib().gdp_gen_chains(int(m), int(n), int(chain_max), float(frac_int_vars), float(frac_inf_vars),
                               float(frac_equality), int(bool(infeasible)), int(seed), C.byref(inst))
    if rc != 0:
        raise RuntimeError(f"gdp_gen_chains failed ({rc})")
    return _take(inst, with_x0)
