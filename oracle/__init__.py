"""TEST INFRASTRUCTURE ONLY: ctypes access to the oracle.

* ``libgdporacle.so`` (oracle/gdp_oracle.c): the CPU restatement of the
  reference propagation, JACOBI (the reference's cpu_omp round function,
  order-independent) and SEQUENTIAL (the reference's cpu_seq) schedules.
* ``_ref/libgdpref.so`` (oracle/ref_harness.cpp): the reference's own round
  functions compiled from its sources; present only where those sources exist.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
package; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "build" / "libgdporacle.so"
REF_SO = HERE / "_ref" / "libgdpref.so"

JACOBI, SEQUENTIAL = 0, 1

_P_INT = C.POINTER(C.c_int)
_P_DBL = C.POINTER(C.c_double)


class _Result(C.Structure):
    _fields_ = [("rounds", C.c_int), ("converged", C.c_int), ("infeasible", C.c_int),
                ("infeasible_var", C.c_int), ("candidates", C.c_longlong), ("rows_processed", C.c_longlong),
                ("nnz_processed", C.c_longlong), ("rows_go", C.c_longlong), ("infeasible_row", C.c_int)]


class _Acts(C.Structure):
    _fields_ = [("minact", C.c_double), ("maxact", C.c_double), ("maxactdelta", C.c_double),
                ("minact_inf", C.c_int), ("maxact_inf", C.c_int)]


@dataclass
class Result:
    lb: np.ndarray
    ub: np.ndarray
    rounds: int
    converged: bool
    infeasible: bool
    infeasible_var: int
    seconds: float
    rows_processed: int = 0
    nnz_processed: int = 0
    rows_go: int = 0  # GPU mode: processed rows of at most split_tile non-zeros that passed their row test
    infeasible_row: int = -1  # smallest row the row rule found infeasible (-1: none)


_o = None
_r = None


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


def lib():
    global _o
    if _o is None:
        if not ORACLE_SO.exists():
            build()
        o = C.CDLL(str(ORACLE_SO))
        o.gdpo_propagate.argtypes = [C.c_int, C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL,
                                     _P_DBL, _P_INT, C.c_int, C.c_int, C.c_int, C.POINTER(_Result)]
        o.gdpo_propagate.restype = C.c_int
        o.gdpo_propagate_ex.argtypes = [C.c_int, C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL,
                                        _P_DBL, _P_INT, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(_Result)]
        o.gdpo_propagate_ex.restype = C.c_int
        o.gdpo_adjust_upper.argtypes = [C.c_int, C.c_double]
        o.gdpo_adjust_upper.restype = C.c_double
        o.gdpo_adjust_lower.argtypes = [C.c_int, C.c_double]
        o.gdpo_adjust_lower.restype = C.c_double
        o.gdpo_is_lb_better.argtypes = [C.c_double] * 3
        o.gdpo_is_ub_better.argtypes = [C.c_double] * 3
        o.gdpo_can_cons_be_tightened.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_double,
                                                 C.c_double, C.c_double]
        o.gdpo_is_cons_infeasible.argtypes = [C.c_double] * 4
        o.gdpo_tighten_var_upper.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                             C.c_double, C.c_int, _P_DBL]
        o.gdpo_tighten_var_lower.argtypes = o.gdpo_tighten_var_upper.argtypes
        o.gdpo_activities.argtypes = [C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL]
        o.gdpo_activities.restype = _Acts
        o.gdpo_var_infeasible.argtypes = [C.c_double, C.c_double]
        o.gdpo_row_infeasible.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]
        o.gdpo_jacobi_round.argtypes = [C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL, _P_DBL,
                                        _P_INT, C.POINTER(C.c_ubyte), _P_DBL, _P_DBL, C.POINTER(C.c_ubyte),
                                        C.c_int]
        _o = o
    return _o


def ref_available() -> bool:
    return REF_SO.exists()


def ref_lib():
    global _r
    if _r is None:
        if not REF_SO.exists():
            raise FileNotFoundError(f"{REF_SO} not built (needs the reference sources)")
        r = C.CDLL(str(REF_SO))
        r.gdpref_propagate.argtypes = [C.c_int, C.c_int, C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL,
                                       _P_DBL, _P_INT, C.c_int, C.c_int, _P_INT, _P_INT, _P_INT, _P_DBL]
        r.gdpref_propagate.restype = C.c_int
        r.gdpref_activities.argtypes = [C.c_int, _P_INT, _P_INT, _P_DBL, _P_DBL, _P_DBL, _P_DBL, _P_DBL, _P_DBL,
                                        _P_INT, _P_INT]
        _r = r
    return _r


def _arrays(mip):
    return (np.ascontiguousarray(mip.row_ptr, np.int32), np.ascontiguousarray(mip.col, np.int32),
            np.ascontiguousarray(mip.val, np.float64), np.ascontiguousarray(mip.lhs, np.float64),
            np.ascontiguousarray(mip.rhs, np.float64), np.ascontiguousarray(mip.vartype, np.int32))


def _pi(a):
    return a.ctypes.data_as(_P_INT)


def _pd(a):
    return a.ctypes.data_as(_P_DBL)


def propagate(mip, schedule: int = JACOBI, max_rounds: int = 0, nthreads: int = 1, lb=None, ub=None,
              split_len: int = 0, split_tile: int = 0) -> Result:
    """Oracle restatement (libgdporacle.so). split_len/split_tile > 0 sum rows
    longer than split_len in the GPU path's lane-group / warp-tile order
    instead of left to right (the row test and candidates stay the reference's)."""
    o = lib()
    rp, col, val, lhs, rhs, vt = _arrays(mip)
    lbo = np.array(mip.lb if lb is None else lb, dtype=np.float64, copy=True)
    ubo = np.array(mip.ub if ub is None else ub, dtype=np.float64, copy=True)
    res = _Result()
    m, n, nnz = len(rp) - 1, len(lbo), int(rp[-1]) if len(rp) else 0
    t0 = time.perf_counter()
    rc = o.gdpo_propagate_ex(m, n, nnz, _pi(col), _pi(rp), _pd(val), _pd(lhs), _pd(rhs), _pd(lbo), _pd(ubo),
                             _pi(vt), int(schedule), int(max_rounds), int(nthreads), int(split_len),
                             int(split_tile), C.byref(res))
    dt = time.perf_counter() - t0
    if rc != 0:
        raise ValueError(f"oracle rejected the input ({rc})")
    return Result(lbo, ubo, res.rounds, bool(res.converged), bool(res.infeasible), res.infeasible_var, dt,
                  res.rows_processed, res.nnz_processed, res.rows_go, res.infeasible_row)


def ref_propagate(mip, schedule: int = JACOBI, max_rounds: int = 0, lb=None, ub=None) -> Result:
    """The reference's own round functions (cpu_omp for JACOBI, cpu_seq for SEQUENTIAL)."""
    r = ref_lib()
    rp, col, val, lhs, rhs, vt = _arrays(mip)
    lbo = np.array(mip.lb if lb is None else lb, dtype=np.float64, copy=True)
    ubo = np.array(mip.ub if ub is None else ub, dtype=np.float64, copy=True)
    rounds, infeas, conv, secs = C.c_int(), C.c_int(), C.c_int(), C.c_double()
    m, n, nnz = len(rp) - 1, len(lbo), int(rp[-1]) if len(rp) else 0
    rc = r.gdpref_propagate(m, n, nnz, _pi(col), _pi(rp), _pd(val), _pd(lhs), _pd(rhs), _pd(lbo), _pd(ubo),
                            _pi(vt), int(schedule), int(max_rounds), C.byref(rounds), C.byref(infeas),
                            C.byref(conv), C.byref(secs))
    if rc != 0:
        raise ValueError(f"reference harness failed ({rc})")
    return Result(lbo, ubo, rounds.value, bool(conv.value), bool(infeas.value), -1, secs.value)


def activities(mip, row: int, lb=None, ub=None) -> dict:
    rp, col, val, _, _, _ = _arrays(mip)
    lbv = np.ascontiguousarray(mip.lb if lb is None else lb, np.float64)
    ubv = np.ascontiguousarray(mip.ub if ub is None else ub, np.float64)
    a = lib().gdpo_activities(int(row), _pi(col), _pi(rp), _pd(val), _pd(lbv), _pd(ubv))
    return {"minact": a.minact, "maxact": a.maxact, "maxactdelta": a.maxactdelta,
            "minact_inf": a.minact_inf, "maxact_inf": a.maxact_inf}
