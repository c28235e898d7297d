"""GPU test of gdp_propagate_noalloc, the entry point for callers that cannot
call cudaMalloc (their device memory belongs to their own pool, e.g. a solver
propagating many branch-and-bound nodes in a loop). It allocates nothing: the
caller passes the problem and the bounds in device memory, and the library's
working memory is one fixed device array shared by every call.

The test calls it through the C-ABI twice in a row on different problems and
checks each result against the context entry point (gdp_propagate_once) with
the same comparison rule as the other parity tests (bit for bit: every row is
short enough to be summed left to right on both paths). The second call also
proves that the shared array is re-initialized between calls. This file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import numpy as np
import pytest

import gdp
import gdpgen
import oracle
from gdp_testutil import assert_bitexact, row_infeasible_mip

pytestmark = pytest.mark.gpu


def _device_arrays(torch, mip):
    dev = "cuda"
    return dict(col=torch.tensor(mip.col, dtype=torch.int32, device=dev),
                row_ptr=torch.tensor(mip.row_ptr, dtype=torch.int32, device=dev),
                val=torch.tensor(mip.val, dtype=torch.float64, device=dev),
                lhs=torch.tensor(mip.lhs, dtype=torch.float64, device=dev),
                rhs=torch.tensor(mip.rhs, dtype=torch.float64, device=dev),
                lb=torch.tensor(mip.lb, dtype=torch.float64, device=dev),
                ub=torch.tensor(mip.ub, dtype=torch.float64, device=dev),
                vartype=torch.tensor(mip.vartype, dtype=torch.int32, device=dev))


def _noalloc(torch, mip):
    d = _device_arrays(torch, mip)
    torch.cuda.synchronize()
    st = gdp.propagate_noalloc(mip.m, mip.n, mip.nnz, d["col"].data_ptr(), d["row_ptr"].data_ptr(),
                               d["val"].data_ptr(), d["lhs"].data_ptr(), d["rhs"].data_ptr(), d["lb"].data_ptr(),
                               d["ub"].data_ptr(), d["vartype"].data_ptr(), 0,
                               torch.cuda.current_stream().cuda_stream)
    return d["lb"].cpu().numpy(), d["ub"].cpu().numpy(), st


def test_noalloc_matches_context_path_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    first = gdpgen.random_mip(0, seed=301)
    second = gdpgen.random_mip(0, seed=302, m=1500, n=1200)
    for mip in (first, second):
        lb, ub, st = _noalloc(torch, mip)
        rlb, rub, rst = gdp.propagate(mip, sync_type=gdp.CPU_LOOP)
        assert st["rounds"] == rst["rounds"]
        assert st["infeasible"] == rst["infeasible"]
        assert st["converged"] == rst["converged"]
        assert_bitexact(lb, ub, rlb, rub, what="noalloc vs context path")


def test_noalloc_rejects_more_variables_than_its_scratch():
    n = gdp.NOALLOC_MAX_VARS + 1
    with pytest.raises(gdp.GDPError, match="at most"):
        gdp.propagate_noalloc(1, n, 1, 1, 1, 1, 1, 1, 1, 1, 1)


def test_noalloc_long_rows_follow_the_reference_order():
    """Rows longer than the context path's thread_row_max are still summed
    left to right by one thread here, with the reference's row test: the
    result equals the oracle's restatement of the reference's cpu_omp round
    function bit for bit, on a power-law instance with rows up to 5,000
    non-zeros."""
    torch = pytest.importorskip("torch")
    mip = gdpgen.random_mip(1, seed=303, m=20_000, n=15_000, len_max=2000, dense_len=5000, n_dense_rows=2)
    assert np.diff(mip.row_ptr).max() > 32
    lb, ub, st = _noalloc(torch, mip)
    ref = oracle.propagate(mip, oracle.JACOBI, nthreads=8)
    assert st["rounds"] == ref.rounds and bool(st["infeasible"]) == ref.infeasible
    assert_bitexact(lb, ub, ref.lb, ref.ub, what="noalloc vs reference order")


def test_noalloc_checks_its_input_before_indexing():
    """A column index outside [0, n) is reported as an error by the device
    check that runs before any round reads the CSR; a valid call afterwards
    works (the shared working array is re-initialized)."""
    torch = pytest.importorskip("torch")
    mip = gdpgen.random_mip(0, seed=304)
    bad = gdp.MIP(mip.row_ptr, mip.col.copy(), mip.val, mip.lhs, mip.rhs, mip.lb, mip.ub, mip.vartype)
    bad.col[5] = mip.n + 7
    with pytest.raises(gdp.GDPError, match="column index out of range at non-zero 5"):
        _noalloc(torch, bad)
    lb, ub, st = _noalloc(torch, mip)
    rlb, rub, rst = gdp.propagate(mip, sync_type=gdp.CPU_LOOP)
    assert st["rounds"] == rst["rounds"]
    assert_bitexact(lb, ub, rlb, rub, what="noalloc after a rejected call")


def test_noalloc_flags_an_infeasible_row():
    torch = pytest.importorskip("torch")
    lb, ub, st = _noalloc(torch, row_infeasible_mip())
    assert st["infeasible"] == 1 and st["infeasible_row"] == 0 and st["infeasible_var"] == -1
