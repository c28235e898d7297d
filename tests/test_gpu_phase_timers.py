"""The phase-timer build (libgdp_gb300_timers.so, -DGDP_PHASE_TIMERS): the
same propagation as the plain library, with per-round phase times that
account for the round loop and per-round work counters that add up to the
propagation's statistics."""
import pytest

import gdp
from gdp_testutil import assert_bitexact

pytestmark = pytest.mark.gpu


def test_phase_timers_account_for_the_round_loop(monkeypatch):
    import phase_split
    plain = gdp.load_library()
    mip = phase_split.workload(0.05, 1000)
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL) as ctx:
        lb, ub, st = ctx.propagate()
    # the timer build becomes the module's library for this test only
    monkeypatch.setattr(gdp, "_lib", plain)
    res = phase_split.split(scale=0.05, seed=1000, warmup=1, per_round=True, keep_bounds=True)
    assert gdp._lib is not plain
    assert res["rounds"] == st["rounds"] and st["rounds"] > 5
    assert_bitexact(res["lb"], res["ub"], lb, ub, what="timer build")
    for k in ("rows_processed", "nnz_processed", "nnz_exact", "rows_exact", "rows_go", "divisions"):
        assert res["stats"][k] == st[k], k
    rounds = res["per_round"]
    assert len(rounds) == st["rounds"]
    assert sum(r["rows"] for r in rounds) == st["rows_processed"]
    assert sum(r["nnz"] for r in rounds) == st["nnz_processed"]
    assert sum(r["nnz_exact"] for r in rounds) == st["nnz_exact"]
    assert all(r["A_us"] > 0 and r["B_us"] >= 0 and r["CF_us"] > 0 for r in rounds)
    # the phases between the first round's start and the last barrier lie
    # inside the launch the device time brackets
    wall = sum(res["wall_ms"].values())
    assert 0.3 * res["device_ms"] < wall <= res["device_ms"] * 1.01
    busy = res["busy_ms_per_warp"]
    assert busy["A_activity"] > 0 and busy["F_finalize"] > 0
    assert sum(busy.values()) <= wall * 1.05  # no warp is much busier than the wall clock (skew of the stamps)
    assert sum(v[0] for v in res["exact_pass_ms_per_warp"].values()) > 0
