"""Where a MEGAKERNEL propagation spends its time, phase by phase.

Builds (once) and loads libgdp_gb300_timers.so -- the library compiled with
-DGDP_PHASE_TIMERS -- propagates the power-law workload (m = 2,000,000 rows,
n = 1,500,000 variables, Zipf(1.8) row lengths in [2, 20000] plus 32 rows of
100,000 non-zeros; the same generator and seed as bench.py) and prints:

  * wall time per phase summed over the rounds (between the grid barriers:
    A = activities and screen, B = multi-tile rows and deferred exact rows,
    C = exact tiles, F = finalize);
  * warp busy time per phase (all warps' time inside each phase, divided by
    the number of warps), which shows how full each phase keeps the GPU;
  * warp time of the two passes of the exact pass of SELL rows by lane-group
    size (pass 1: FP64 activities and the row test; pass 2: candidates);
  * with --per-round, one line per round with the work it processed and, per
    phase group, the average warp's busy time and the longest single warp's
    (a long pole shows as a maximum near the phase's wall time).

    python gpu-domain-propagator_gb300/phase_split.py [--scale 1.0] [--per-round]

The timers add atomics and %globaltimer reads to every warp's phase: the
timer library's device time is a little above the plain library's.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics
import sys
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
sys.path.insert(0, str(PKG))

import build as _build  # noqa: E402
import gdp  # noqa: E402
import gdpgen  # noqa: E402

ROUNDS = 1024  # rounds the device timers hold
SLOTS = 8
PHASES = ("A_activity", "B_multitile_rows", "B_exact_rows", "C_exact_tiles", "F_finalize")


def workload(scale: float, seed: int):
    m, n = int(2_000_000 * scale), int(1_500_000 * scale)
    kw = {} if scale >= 1.0 else dict(len_max=max(16, int(20000 * scale)), dense_len=max(32, int(100_000 * scale)))
    return gdpgen.random_mip(1, seed=seed, m=m, n=n, **kw)


def read_timers(lib, rounds: int):
    wall = (C.c_ulonglong * (ROUNDS * SLOTS))()
    busy = (C.c_ulonglong * (ROUNDS * SLOTS))()
    passes = (C.c_ulonglong * 16)()
    if lib.gdp_phase_timers_read(wall, busy, passes, ROUNDS) != gdp.GDP_OKAY:
        raise gdp.GDPError(gdp.last_error())
    cut = lambda b: np.frombuffer(b, dtype=np.uint64).reshape(ROUNDS, SLOTS).astype(np.int64)[1:rounds + 1]
    return cut(wall), cut(busy), np.frombuffer(passes, dtype=np.uint64).astype(np.int64)


def split(scale: float = 1.0, seed: int = 1000, warmup: int = 3, per_round: bool = False,
          cta_threads: int = 256, keep_bounds: bool = False, use_marking: int = -1) -> dict:
    so = _build.build(phase_timers=True)["gdp"]
    lib = gdp.load_library(so, make_default=True)
    mip = workload(scale, seed)
    ctx = gdp.Context(mip, sync_type=gdp.MEGAKERNEL, cta_threads=cta_threads, use_marking=use_marking)
    ms = [ctx.propagate()[2]["device_ms"] for _ in range(warmup)]
    if lib.gdp_phase_timers_clear() != gdp.GDP_OKAY:
        raise gdp.GDPError(gdp.last_error())
    lb, ub, st = ctx.propagate()
    R = min(st["rounds"], ROUNDS - 1)
    wall, busy, passes = read_timers(lib, R)
    warps = ctx.layout()["mega_grid"] * cta_threads // 32
    a = wall[:, 1] - wall[:, 0]
    b = wall[:, 2] - wall[:, 1]
    cf = wall[:, 4] - wall[:, 2]  # C (when present) and F
    busy_ms = {k: float(busy[:, i].sum()) / warps / 1e6 for i, k in enumerate(PHASES)}
    # per round: the average warp's busy time and the longest single warp's, by phase group
    avg_a = busy[:, 0] / warps
    avg_b = (busy[:, 1] + busy[:, 2]) / warps
    avg_cf = (busy[:, 3] + busy[:, 4]) / warps
    total_busy = sum(busy_ms.values())
    out = {
        "workload": f"power-law MIP m={mip.m} n={mip.n} nnz={mip.nnz} seed={seed}",
        "rounds": st["rounds"], "device_ms": st["device_ms"],
        "device_ms_warmup_median": statistics.median(ms) if ms else None,
        "warps": warps,
        "wall_ms": {"A": float(a.sum()) / 1e6, "B": float(b.sum()) / 1e6, "C+F": float(cf.sum()) / 1e6},
        "busy_ms_per_warp": busy_ms,
        "busy_share": {k: v / total_busy for k, v in busy_ms.items()} if total_busy else {},
        "exact_pass_ms_per_warp": {f"g{1 << lg}": [float(passes[2 * lg]) / warps / 1e6,
                                                     float(passes[2 * lg + 1]) / warps / 1e6] for lg in range(6)},
        # one-lane exact rows: elements against 32 x the longest row of each warp
        "one_lane_row_utilisation": float(passes[12]) / float(passes[13]) if passes[13] else None,
        "stats": {k: st[k] for k in ("rows_processed", "nnz_processed", "nnz_exact", "rows_exact", "rows_go",
                                     "divisions", "changed_vars")},
    }
    if per_round:
        prev = np.zeros(3, np.int64)
        lines = []
        for r in range(R):
            d = wall[r, 5:8] - prev
            prev = wall[r, 5:8]
            lines.append({"round": r + 1, "A_us": a[r] / 1e3, "B_us": b[r] / 1e3, "CF_us": cf[r] / 1e3,
                          "rows": int(d[0]), "nnz": int(d[1]), "nnz_exact": int(d[2]),
                          "A_avg_us": avg_a[r] / 1e3, "A_max_us": busy[r, 5] / 1e3,
                          "B_avg_us": avg_b[r] / 1e3, "B_max_us": busy[r, 6] / 1e3,
                          "CF_avg_us": avg_cf[r] / 1e3, "CF_max_us": busy[r, 7] / 1e3})
        out["per_round"] = lines
    if keep_bounds:
        out["lb"], out["ub"] = lb, ub
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scale", type=float, default=1.0, help="shrink m and n (1.0: the 2M-row workload)")
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--per-round", action="store_true")
    ap.add_argument("--cta-threads", type=int, default=256, choices=[128, 256, 512])
    ap.add_argument("--marking", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="-1: library default; 0: full sweeps; 1: adaptive; 2: marked rows every round")
    args = ap.parse_args(argv)
    res = split(args.scale, args.seed, args.warmup, args.per_round, args.cta_threads, use_marking=args.marking)
    rounds = res.pop("per_round", None)
    print(json.dumps(res, indent=1))
    for r in rounds or []:
        print(f"round {r['round']:4d}  A {r['A_us']:8.1f} us  B {r['B_us']:8.1f} us  C+F {r['CF_us']:7.1f} us  "
              f"rows {r['rows']:9d}  nnz {r['nnz']:11d}  exact nnz {r['nnz_exact']:10d}  "
              f"warp avg/max: A {r['A_avg_us']:6.1f}/{r['A_max_us']:6.1f}  B {r['B_avg_us']:6.1f}/{r['B_max_us']:6.1f}  "
              f"C+F {r['CF_avg_us']:5.1f}/{r['CF_max_us']:5.1f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
