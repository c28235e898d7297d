"""Generates the golden fixtures under tests/golden/ (run in the build container).

Inputs:
  * the reference's analytical test MIPs (test/test_setups.cuh of the
    reference: TwoLinesExample :126-182, AchterbergExample :185-243,
    SavelsberghExample1 :248-303, SavelsberghCFLP :309-368, ex1 :614-660,
    WeakestBoundsExample1 :662-712) transcribed as test vectors, with their
    analytical bounds;
  * the reference's two generators, restated: GeneralizedCFP(k)
    (:473-611, analytical solution) and ATMSynthetic(n) (:372-466, glibc
    srand/rand values as in test/test_infra.cu:9-19);
  * seeded small random MIPs from libgdpgen (random_mip workload 0).
Expected outputs: the reference's own round functions (oracle/_ref, cpu_omp =
JACOBI and cpu_seq = SEQUENTIAL schedules, reference round cap 100) -- rounds,
infeasibility and bounds. Each case is one compressed .npz.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "gpu-domain-propagator_gb300"))

import oracle  # noqa: E402
from gdp import MIP  # noqa: E402

INF = 1e20


def mip(vals, cols, rows, lhs, rhs, lb, ub, vt):
    return MIP(np.array(rows, np.int32), np.array(cols, np.int32), np.array(vals, np.float64),
               np.array(lhs, np.float64), np.array(rhs, np.float64), np.array(lb, np.float64),
               np.array(ub, np.float64), np.array(vt, np.int32))


def two_lines():
    m = mip([0.5, 1, 1, -1], [0, 1, 0, 1], [0, 2, 4], [1, 1], [1, 1], [-2, -2], [2, 2], [3, 3])
    return m, ([1.33333333209157, 0.3333333330228925], [1.333333333954215, 0.33333333395421505])


def achterberg():
    vals = [2, 3, 2, 9, -1, -2, -3, 5, -3, -3, 9, -2, 9, -1, 2, -4, -7, 2, 5, -2, -1, 5, 4, -5, 1, -1, 1, -2, 1,
            -1, -2, 1, -2, 4, 2, -1, 3, -2, -1, 5, 1, 2, -6, -2, -2, 1, 1, 1, 2, -2, 2, -2]
    cols = [0, 7, 8, 1, 7, 8, 1, 2, 3, 1, 3, 9, 4, 8, 9, 5, 6, 9, 6, 8, 4, 6, 8, 9, 0, 1, 2, 4, 5, 7, 8, 9, 10, 11,
            1, 3, 4, 5, 7, 8, 9, 10, 11, 0, 2, 3, 4, 7, 8, 9, 10, 11]
    rows = [0, 3, 6, 9, 12, 15, 18, 20, 24, 34, 43, 52]
    m = mip(vals, cols, rows, [-100] * 11, [9, 0, 4, 6, 8, 3, 2, 2, 1, 2, 1], [0] * 12, [1] * 7 + [100] * 5,
            [0] * 7 + [1] * 5)
    return m, ([0.0] * 12, [1, 1, 1, 1, 1, 1, 1, 3, 4, 6, 23, 15])


def savelsbergh1():
    m = mip([1, 3, 1, 2, 2, 1, -15, 1, -20, 1, -5, 1], [3, 4, 3, 4, 3, 4, 0, 3, 1, 4, 2, 5], [0, 2, 4, 6, 8, 10, 12],
            [15, 10, 20, -INF, -INF, -INF], [INF, INF, INF, 0, 0, 0], [0] * 6, [1, 1, 1, INF, INF, INF],
            [0, 0, 0, 3, 3, 3])
    return m, ([0.0] * 6, [1, 1, 1, 15, 20, 5])


def savelsbergh_cflp():
    vals = [1] * 15 + [-100, 1, 1, 1, -100, 1, 1, 1, -100, 1, 1, 1, -100]
    cols = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 0, 4, 8, 12, 1, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15]
    m = mip(vals, cols, [0, 4, 8, 12, 16, 20, 24, 28], [80, 70, 40, -INF, -INF, -INF, -INF], [80, 70, 40, 0, 0, 0, 0],
            [0] * 16, [INF] * 12 + [1] * 4, [3] * 12 + [0] * 4)
    return m, ([0.0] * 16, [80, 80, 80, 80, 70, 70, 70, 70, 40, 40, 40, 40, 1, 1, 1, 1])


def ex1():
    m = mip([-1.0, 1.0, 1.0, 10.0, 1.0, -3.0, 1.0, 1.0, -3.5], [0, 1, 2, 3, 0, 1, 2, 1, 3], [0, 4, 7, 9],
            [-1e100, -1e100, 0.0], [20.0, 30.0, 0.0], [0.0, 0.0, 0.0, 2.0],
            [40.0, 1.7976931348623157e+308, 1.7976931348623157e+308, 3.0], [3, 3, 3, 1])
    return m, None


def weakest_bounds1():
    m = mip([1.0, 1.0, -1.0, -1.0, -1.0, 1.0, -1.0, 1.0, 1.0], [0, 0, 2, 3, 1, 2, 1, 3, 1], [0, 1, 4, 6, 8, 9],
            [-INF] * 5, [1.0] * 5, [-INF] * 4, [INF] * 4, [3] * 4)
    return m, None


def generalized_cfp(k: int, capacity: int = 100):
    vals, cols, rows, lhs, rhs = [], [], [0], [], []
    for i in range(k):
        for idx in range(k):
            vals.append(1.0)
            cols.append(i * k + idx)
    for i in range(k, 2 * k):
        for idx in range(k):
            vals.append(1.0)
            cols.append(idx * k + i - k)
            if idx == k - 1:
                vals.append(-capacity)
                cols.append(idx * k + i)
    cur = 0
    for i in range(2 * k):
        cur += k if i < k else k + 1
        rows.append(cur)
        lhs.append((i + 1) % capacity if i < k else -INF)
        rhs.append((i + 1) % capacity if i < k else 0)
    n = k * k + k
    lb = [0.0] * n
    ub = [INF if i < k * k else 1.0 for i in range(n)]
    vt = [3 if i < k * k else 0 for i in range(n)]
    ub_an = [float((i + 1) % capacity) for i in range(k) for _ in range(k)] + [1.0] * k
    return mip(vals, cols, rows, lhs, rhs, lb, ub, vt), ([0.0] * n, ub_an)


_libc = ctypes.CDLL("libc.so.6")
_libc.srand.argtypes = [ctypes.c_uint]
RAND_MAX = 2147483647


def _rand10(seed: float) -> float:
    _libc.srand(ctypes.c_uint(int(seed)).value)
    v = _libc.rand() / RAND_MAX
    return v if int(seed) % 2 == 0 else -v


def _rand10pos(seed: float) -> float:
    _libc.srand(ctypes.c_uint(int(seed)).value)
    return _libc.rand() / RAND_MAX


def atm_synthetic(n: int):
    stride = 4
    vals, cols, rows = [], [], [0]
    cnt = 0
    for i in range(stride):
        cnt += n
        rows.append(cnt)
        for j in range(n):
            vals.append(_rand10((i * 5 + 9) * (j * 3)))
            cols.append(j)
    for i in range(stride, n, stride):
        for ii in range(stride):
            if i + ii < n:
                cnt += min(stride, n - i)
                rows.append(cnt)
            for jj in range(stride):
                x, y = i + ii, i + jj
                if x < n and y < n:
                    vals.append(_rand10(x * y * 2))
                    cols.append(y)
    lhs, rhs, lb, ub, vt = [], [], [], [], []
    for i in range(n):
        seed = (i * 3 + 26) * 6
        v = _rand10(seed)
        lhs.append(-abs(v))
        rhs.append(abs(v) * 2)
        is_int = not (i < n * 0.9)
        lo, hi = -_rand10pos(seed), _rand10pos(seed)
        if is_int:
            hi = float(np.floor(hi + 1e-9))
            lo = float(np.ceil(lo - 1e-9))
        lb.append(lo)
        ub.append(hi)
        vt.append(1 if is_int else 3)
    return mip(vals, cols, rows, lhs, rhs, lb, ub, vt), None


def save(name: str, m: MIP, analytical=None) -> None:
    out = dict(row_ptr=m.row_ptr, col=m.col, val=m.val, lhs=m.lhs, rhs=m.rhs, lb=m.lb, ub=m.ub,
               vartype=m.vartype)
    if analytical is not None:
        out["lb_analytical"] = np.array(analytical[0], np.float64)
        out["ub_analytical"] = np.array(analytical[1], np.float64)
    for tag, sched in (("omp", oracle.JACOBI), ("seq", oracle.SEQUENTIAL)):
        r = oracle.ref_propagate(m, sched)
        out[f"lb_{tag}"] = r.lb
        out[f"ub_{tag}"] = r.ub
        out[f"rounds_{tag}"] = np.int32(r.rounds)
        out[f"infeasible_{tag}"] = np.int32(r.infeasible)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: m={m.m} n={m.n} nnz={m.nnz} rounds omp={int(out['rounds_omp'])} seq={int(out['rounds_seq'])}")


def main() -> None:
    oracle.build(ref=True)
    import gdpgen
    save("two_lines", *two_lines())
    save("achterberg", *achterberg())
    save("savelsbergh1", *savelsbergh1())
    save("savelsbergh_cflp", *savelsbergh_cflp())
    save("ex1", *ex1())
    save("weakest_bounds1", *weakest_bounds1())
    save("generalized_cfp_40", *generalized_cfp(40))
    save("atm_synthetic_2000", *atm_synthetic(2000))
    for seed in (1, 2):
        save(f"random_mip_seed{seed}", gdpgen.random_mip(0, seed=seed))
    # a small infeasible instance: a random MIP whose first row is made unsatisfiable
    m = gdpgen.random_mip(0, seed=3, m=400, n=300)
    b, e = int(m.row_ptr[0]), int(m.row_ptr[1])
    acts = np.abs(m.val[b:e]) * np.maximum(np.abs(np.clip(m.lb[m.col[b:e]], -1e3, 1e3)),
                                            np.abs(np.clip(m.ub[m.col[b:e]], -1e3, 1e3)))
    m.lhs[0] = float(np.sum(acts) + 10.0)
    m.rhs[0] = INF
    save("random_mip_infeasible", m)


if __name__ == "__main__":
    main()
