"""The autotuner times every candidate layout/schedule and returns the
fastest; propagation under the chosen options stays bit-exact with the
oracle's GPU mode of the same layout."""
import pytest

import gdp
import gdpgen
import oracle
from gdp_testutil import assert_bitexact

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_stays_exact():
    mip = gdpgen.random_mip(1, seed=41, m=40_000, n=30_000, n_dense_rows=2, dense_len=6_000)
    opts, ms, trials = gdp.autotune(mip, repeats=1)
    assert len(trials) == 36
    assert ms == min(t["ms"] for t in trials) and ms > 0
    assert opts["thread_row_max"] in (16, 32, 64) and opts["split_tile"] in (512, 1024, 2048)
    assert opts["sync_type"] in (gdp.MEGAKERNEL, gdp.GPU_LOOP)
    lb, ub, st = gdp.propagate(mip, sync_type=opts["sync_type"], thread_row_max=opts["thread_row_max"],
                               split_tile=opts["split_tile"])
    ref = oracle.propagate(mip, oracle.JACOBI, split_len=opts["thread_row_max"], split_tile=opts["split_tile"],
                           nthreads=8)
    assert st["rounds"] == ref.rounds
    assert_bitexact(lb, ub, ref.lb, ref.ub, what=str(opts))
