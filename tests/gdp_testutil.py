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


def row_infeasible_mip() -> MIP:
    """x1 + x2 >= 1e-3 with x1 fixed at 1e4 and x2 at -1e4 (continuous): the
    row's maximum activity 0 is below its lhs (a row the row rule flags: 1e-3 >
    1e-6 * max(1, 0, 1e-3)), while the candidates move each bound by 1e-3 only,
    within the variable rule's tolerance 1e-6 * 1e4 -- no variable crosses."""
    return MIP(np.array([0, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]),
               np.array([1e-3]), np.array([1e20]), np.array([1e4, -1e4]), np.array([1e4, -1e4]),
               np.array([3, 3], np.int32))


def eps_band_mip(length: int = 64, blocker: bool = True, p: int | None = None, q: int | None = None) -> MIP:
    """One row sum_k x_k <= 1 over continuous x_k in [0, u_k] (lhs = -inf), so
    its slack is 1 and d_k = u_k. Every u_k is 0.5 except u_p = 1 + 1.5e-9,
    the row's maximum d, which exceeds the slack by 1.5e-9 -- inside the
    (EPS, 2.00001e-9] band where only the reference's sequential EPS-max
    decides the row test. With `blocker`, an earlier u_q = 1 + 0.7e-9 becomes
    that EPS-max and u_p never replaces it (it exceeds it by 0.8e-9 <= EPS):
    the reference skips the row. Without it the EPS-max is u_p, the row is
    processed and u_p tightens to 1."""
    p = length - 5 if p is None else p
    q = 3 if q is None else q
    u = np.full(length, 0.5)
    u[p] = 1.0 + 1.5e-9
    if blocker:
        u[q] = 1.0 + 0.7e-9
    return MIP(np.array([0, length], np.int32), np.arange(length, dtype=np.int32), np.ones(length),
               np.array([-1e20]), np.array([1.0]), np.zeros(length), u, np.full(length, 3, np.int32))
