"""The bench's parity reporting (bench.compare_bounds, bench.parity_entry):
integer bounds must match bit for bit, continuous bounds within 1e-9 relative
plus 1e-12 absolute, and bounds at or beyond the reference's infinity (1e20)
compare as equal infinities."""
import math
from types import SimpleNamespace

import numpy as np

import bench

INT, BIN, CONT = 0, 1, 3


def test_integer_bounds_must_match_exactly():
    vt = [INT, BIN, INT]
    ref_lb, ref_ub = np.array([0.0, 0.0, -3.0]), np.array([5.0, 1.0, 4.0])
    lb, ub = ref_lb.copy(), ref_ub.copy()
    ub[0] = 5.0 + 1e-15  # an integer bound a few ulps off is a mismatch
    lb[2] = -2.0
    r = bench.compare_bounds(lb, ub, ref_lb, ref_ub, vt)
    assert r["int_mismatches"] == 2
    assert r["cont_beyond_tol"] == 0
    assert r["cont_max_abs"] == 0.0  # integer deviations are not continuous ones


def test_continuous_tolerance_is_1e9_relative_plus_1e12_absolute():
    vt = [CONT] * 5
    ref = np.array([1.0, 1000.0, 0.0, 0.0, -7.5])
    got = ref + np.array([0.9e-9,        # within 1e-9 relative
                          2.0e-6,        # 2e-9 relative: beyond
                          0.9e-12,       # within the absolute floor at zero
                          2.0e-12,       # beyond it
                          0.0])
    r = bench.compare_bounds(got, ref, ref, ref, vt)
    assert r["int_mismatches"] == 0
    assert r["cont_beyond_tol"] == 2
    assert math.isclose(r["cont_max_abs"], 2.0e-6, rel_tol=1e-6)
    assert math.isclose(r["cont_max_rel"], 2.0e-9, rel_tol=1e-3)


def test_bounds_beyond_the_reference_infinity_compare_equal():
    vt = [CONT, INT, CONT]
    ref_lb = np.array([-np.inf, -1e20, -1e25])
    ref_ub = np.array([np.inf, 1e20, 3.0])
    lb = np.array([-1e20, -np.inf, -np.inf])
    ub = np.array([1e30, np.inf, 3.0])
    r = bench.compare_bounds(lb, ub, ref_lb, ref_ub, vt)
    assert r == {"int_mismatches": 0, "cont_beyond_tol": 0, "cont_max_abs": 0.0, "cont_max_rel": 0.0}


def test_nan_is_beyond_tolerance():
    vt = [CONT]
    r = bench.compare_bounds(np.array([np.nan]), np.array([1.0]), np.array([0.0]), np.array([1.0]), vt)
    assert r["cont_beyond_tol"] == 1


def test_parity_entry_reports_rounds_verdicts_and_deviations():
    vt = [INT, CONT]
    ref = SimpleNamespace(lb=np.array([0.0, 0.5]), ub=np.array([2.0, 1.5]), rounds=7, infeasible=False)
    st = {"rounds": 7, "infeasible": 0}
    e = bench.parity_entry(np.array([0.0, 0.5]), np.array([2.0, 1.5 + 1e-6]), st, ref, vt, "Jacobi")
    assert e["schedule"] == "Jacobi"
    assert e["rounds"] == {"gpu": 7, "ref": 7}
    assert e["infeasible"] == {"gpu": False, "ref": False}
    assert e["int_mismatches"] == 0
    assert e["cont_beyond_tol"] == 1
    assert math.isclose(e["cont_max_abs"], 1e-6, rel_tol=1e-6)
