"""CPU tests of the C-ABI library: it loads, exports every symbol that
include/*.h declares, and handles the calls that need no GPU (FP32 / CPU
entry points, empty problems, argument validation) like the reference."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import gdp

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:GDP_RETCODE|const char \*|int|void)\s+\*?(\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_reference_interface():
    names = set(_declared_symbols())
    # every entry point of the reference's include/interface.h
    ref = {"propagateConstraintsGPUReductionDouble", "propagateConstraintsGPUReductionFloat",
           "propagateConstraintsGPUAtomicDouble", "propagateConstraintsGPUAtomicFloat",
           "propagateConstraintsSequentialDouble", "propagateConstraintsSequentialFloat",
           "propagateConstraintsFullOMPDouble", "propagateConstraintsFullOMPFloat",
           "propagateConstraintsSequentialDisjointDouble", "sequentialPropagateWithMeasureDouble",
           "atomicPropagateWithMeasureDouble"}
    assert ref <= names


@pytest.mark.parametrize("name", _declared_symbols())
def test_library_exports(name):
    lib = gdp.load_library()
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def _tiny():
    return dict(n_cons=1, n_vars=2, nnz=2, col=np.array([0, 1], np.int32), rp=np.array([0, 2], np.int32),
                val=np.array([1.0, 1.0]), lhs=np.array([-1e20]), rhs=np.array([1.0]),
                lb=np.array([0.0, 0.0]), ub=np.array([5.0, 5.0]), vt=np.array([1, 1], np.int32))


def test_float_and_cpu_entry_points_not_implemented():
    lib = gdp.load_library()
    t = _tiny()
    f = np.zeros(2, np.float32)
    pf = f.ctypes.data_as(C.c_void_p)
    pi = t["col"].ctypes.data_as(C.c_void_p)
    for name in ("propagateConstraintsGPUReductionFloat", "propagateConstraintsSequentialFloat",
                 "propagateConstraintsFullOMPFloat"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        assert fn(1, 2, 2, pi, pi, pf, pf, pf, pf, pf, pi) == gdp.GDP_NOTIMPLEMENTED
    fn = lib.propagateConstraintsGPUAtomicFloat
    fn.restype = C.c_int
    assert fn(1, 2, 2, pi, pi, pf, pf, pf, pf, pf, pi, 0) == gdp.GDP_NOTIMPLEMENTED
    d = np.zeros(2)
    pd = d.ctypes.data_as(C.c_void_p)
    for name in ("propagateConstraintsSequentialDouble", "propagateConstraintsFullOMPDouble",
                 "propagateConstraintsSequentialDisjointDouble", "sequentialPropagateWithMeasureDouble",
                 "atomicPropagateWithMeasureDouble"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        assert fn(1, 2, 2, pi, pi, pd, pd, pd, pd, pd, pi) == gdp.GDP_NOTIMPLEMENTED
    assert "not implemented" in gdp.last_error()


def test_phase_timers_only_in_the_timer_build():
    """The plain library compiles no phase timers: both calls refuse without
    touching the device."""
    lib = gdp.load_library()
    assert lib.gdp_phase_timers_clear() == gdp.GDP_NOTIMPLEMENTED
    assert "GDP_PHASE_TIMERS" in gdp.last_error()
    assert lib.gdp_phase_timers_read(None, None, None, 4) == gdp.GDP_NOTIMPLEMENTED


def test_empty_problem_is_noop():
    # reference src/propagators/GPU_propagator.cuh:113-116
    lb, ub = gdp.propagateGPUAtomic(2, 0, 0, [], [0], [], [], [], [1.0, 2.0], [3.0, 4.0], [3, 3])
    assert lb == [1.0, 2.0] and ub == [3.0, 4.0]


def test_unknown_sync_type_is_error():
    t = _tiny()
    with pytest.raises(gdp.GDPError, match="Unknown sync type"):
        gdp.propagateGPUAtomic(2, 1, 2, t["col"], t["rp"], t["val"], t["lhs"], t["rhs"], t["lb"], t["ub"],
                               t["vt"], synctype=7)


@pytest.mark.parametrize("bad", ["row_ptr_start", "col_range", "vartype", "nan_coef"])
def test_invalid_csr_rejected(bad):
    t = _tiny()
    col, rp, val, vt = t["col"].copy(), t["rp"].copy(), t["val"].copy(), t["vt"].copy()
    if bad == "row_ptr_start":
        rp = np.array([1, 2], np.int32)
    elif bad == "col_range":
        col = np.array([0, 2], np.int32)
    elif bad == "vartype":
        vt = np.array([1, 2], np.int32)
    elif bad == "nan_coef":
        val = np.array([1.0, np.nan])
    with pytest.raises(gdp.GDPError):
        gdp.propagateGPUAtomic(2, 1, 2, col, rp, val, t["lhs"], t["rhs"], t["lb"], t["ub"], vt)


def test_non_monotone_row_ptr_rejected():
    # three rows, row_ptr = [0, 2, 1, 2]: starts at 0, ends at nnz, decreases in the middle
    with pytest.raises(gdp.GDPError, match="monotone"):
        gdp.propagateGPUAtomic(2, 3, 2, [0, 1], [0, 2, 1, 2], [1.0, 1.0], [0.0] * 3, [1.0] * 3, [0.0, 0.0],
                               [1.0, 1.0], [3, 3])


def test_legacy_length_checks():
    with pytest.raises(AssertionError):
        gdp.propagateGPUAtomic(2, 1, 2, [0], [0, 2], [1.0, 1.0], [0.0], [1.0], [0.0, 0.0], [1.0, 1.0], [3, 3])
