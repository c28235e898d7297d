"""Shared helpers of the test suite: golden fixtures and comparison rules."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from gdp import MIP

GOLDEN = Path(__file__).resolve().parent / "golden"

# Tolerance for continuous bounds of this project (relative 1e-9, absolute
# 1e-12); integer-variable bounds, round counts and infeasibility flags are
# compared exactly.
REL_TOL = 1e-9
ABS_TOL = 1e-12
# The reference's own end-to-end tolerance against analytical solutions
# (test/test_infra.cuh:15, TEST_EPS).
REF_TEST_EPS = 1e-4

GOLDEN_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name: str):
    z = np.load(GOLDEN / f"{name}.npz")
    mip = MIP(z["row_ptr"], z["col"], z["val"], z["lhs"], z["rhs"], z["lb"], z["ub"], z["vartype"])
    return mip, {k: z[k] for k in z.files}


def clamp_inf(x: np.ndarray) -> np.ndarray:
    """Values beyond +-1e20 are all infinite (the reference's GDP_INF)."""
    return np.clip(np.asarray(x, np.float64), -1e20, 1e20)


def bounds_close(a: np.ndarray, b: np.ndarray, vartype: np.ndarray, rel: float = REL_TOL,
                 abs_: float = ABS_TOL) -> tuple[bool, str]:
    a, b = clamp_inf(a), clamp_inf(b)
    is_int = np.asarray(vartype) != 3
    bad_int = is_int & (a != b)
    bad_cont = (~is_int) & ~(np.abs(a - b) <= abs_ + rel * np.abs(b))
    if bad_int.any() or bad_cont.any():
        idx = np.flatnonzero(bad_int | bad_cont)[:5]
        return False, f"{int(bad_int.sum())} integer / {int(bad_cont.sum())} continuous mismatches, e.g. " + \
            ", ".join(f"[{i}] {a[i]!r} vs {b[i]!r}" for i in idx)
    return True, ""


def assert_bounds_close(lb, ub, lb_ref, ub_ref, vartype, rel=REL_TOL, abs_=ABS_TOL, what=""):
    ok, msg = bounds_close(lb, lb_ref, vartype, rel, abs_)
    assert ok, f"{what} lower bounds: {msg}"
    ok, msg = bounds_close(ub, ub_ref, vartype, rel, abs_)
    assert ok, f"{what} upper bounds: {msg}"


def assert_bitexact(lb, ub, lb_ref, ub_ref, what=""):
    """Equal as numbers (+0.0 == -0.0), infinities clamped to +-1e20."""
    for name, x, y in (("lb", lb, lb_ref), ("ub", ub, ub_ref)):
        x, y = clamp_inf(x), clamp_inf(y)
        bad = np.flatnonzero(x != y)
        assert bad.size == 0, f"{what} {name}: {bad.size} differ, e.g. " + \
            ", ".join(f"[{i}] {x[i]!r} vs {y[i]!r}" for i in bad[:5])


def permute(mip: MIP, row_perm: np.ndarray | None = None, col_perm: np.ndarray | None = None) -> MIP:
    """Row/column permutation as in the reference's permute_mip
    (fileReader/run_propagation.py:28-51): new row i is old row row_perm[i],
    new column j is old column col_perm[j]; columns stay ascending in a row."""
    m, n = mip.m, mip.n
    rp = np.arange(m) if row_perm is None else np.asarray(row_perm)
    cp = np.arange(n) if col_perm is None else np.asarray(col_perm)
    inv_c = np.empty(n, np.int64)
    inv_c[cp] = np.arange(n)
    rows, cols, vals = [], [], []
    lens = np.diff(mip.row_ptr)
    for i_new, i_old in enumerate(rp):
        b, e = mip.row_ptr[i_old], mip.row_ptr[i_old + 1]
        c = inv_c[mip.col[b:e]]
        o = np.argsort(c, kind="stable")
        cols.append(c[o])
        vals.append(mip.val[b:e][o])
    row_ptr = np.concatenate([[0], np.cumsum(lens[rp])]).astype(np.int32)
    return MIP(row_ptr, np.concatenate(cols).astype(np.int32) if cols else np.zeros(0, np.int32),
               np.concatenate(vals) if vals else np.zeros(0), mip.lhs[rp].copy(), mip.rhs[rp].copy(),
               mip.lb[cp].copy(), mip.ub[cp].copy(), mip.vartype[cp].copy())
