"""The autotuner times row bins, then loop schedules (driver, CTAs per SM,
megakernel CTA size) on the fastest bins, returns the fastest, and keeps the
result per problem shape; propagation under the chosen options stays
bit-exact with the oracle's GPU mode of the same layout."""
import time

import pytest

import gdp
import gdpgen
import oracle
from gdp_testutil import assert_bitexact

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_stays_exact():
    gdp.autotune_clear_cache()
    mip = gdpgen.random_mip(1, seed=41, m=40_000, n=30_000, n_dense_rows=2, dense_len=6_000)
    opts, ms, trials = gdp.autotune(mip, repeats=1)
    assert len(trials) == 9 + 5  # 9 row bins, then 5 schedules other than the base one
    assert ms == min(t["ms"] for t in trials) and ms > 0
    assert {t["cta_threads"] for t in trials} == {128, 256, 512}
    assert opts["thread_row_max"] in (16, 32, 64) and opts["split_tile"] in (512, 1024, 2048)
    assert opts["sync_type"] in (gdp.MEGAKERNEL, gdp.GPU_LOOP)
    with gdp.Context(mip, sync_type=opts["sync_type"], thread_row_max=opts["thread_row_max"],
                     split_tile=opts["split_tile"], ctas_per_sm=opts["ctas_per_sm"],
                     cta_threads=opts["cta_threads"]) as ctx:
        lb, ub, st = ctx.propagate()
    ref = oracle.propagate(mip, oracle.JACOBI, split_len=opts["thread_row_max"], split_tile=opts["split_tile"],
                           nthreads=8)
    assert st["rounds"] == ref.rounds
    assert_bitexact(lb, ub, ref.lb, ref.ub, what=str(opts))


def test_autotune_cache_per_shape():
    """A second call for a problem of the same shape (here the same matrix
    with other bounds) returns the cached result without timing anything."""
    gdp.autotune_clear_cache()
    mip = gdpgen.random_mip(1, seed=42, m=30_000, n=20_000, n_dense_rows=2, dense_len=4_000)
    t0 = time.perf_counter()
    a = gdp.autotune(mip, repeats=1)
    first = time.perf_counter() - t0
    other = gdp.MIP(mip.row_ptr, mip.col, mip.val, mip.lhs, mip.rhs, mip.lb, mip.ub * 2, mip.vartype)
    t0 = time.perf_counter()
    b = gdp.autotune(other, repeats=1)
    second = time.perf_counter() - t0
    assert a == b
    assert second < 0.1 * first


@pytest.mark.parametrize("cta_threads", [128, 256, 512])
def test_megakernel_cta_sizes_bitexact(cta_threads):
    """The megakernel's CTA size changes only the grid: results stay bit for bit."""
    mip = gdpgen.random_mip(1, seed=43, m=30_000, n=20_000, n_dense_rows=2, dense_len=4_000)
    ref = oracle.propagate(mip, oracle.JACOBI, split_len=32, split_tile=1024, nthreads=8)
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL, cta_threads=cta_threads) as ctx:
        lb, ub, st = ctx.propagate()
    assert st["rounds"] == ref.rounds
    assert_bitexact(lb, ub, ref.lb, ref.ub)


def test_bad_cta_threads_rejected():
    mip = gdpgen.random_mip(0, seed=44)
    with pytest.raises(gdp.GDPError, match="cta_threads"):
        gdp.Context(mip, sync_type=gdp.MEGAKERNEL, cta_threads=96)
