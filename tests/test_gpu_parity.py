"""GPU parity: the CUDA path through the C-ABI against the oracle and the
reference's golden outputs.

The GPU runs the deterministic Jacobi schedule (the reference's cpu_omp round
function). Every row takes the reference's row test and candidates; rows up to
thread_row_max non-zeros are also summed left to right as the reference does,
longer rows in fixed lane groups and warp tiles, which the oracle's GPU mode
reproduces (split_len/split_tile). Every comparison against the oracle with the
same parameters is therefore bit for bit, comparisons against the reference's
own outputs are bit for bit where no row is split, and with rows split the
bounds stay within the contract's tolerance of the reference's cpu_omp
(test_power_law_vs_reference_semantics).
"""
import numpy as np
import pytest

import gdp
import gdpgen
import oracle
from gdp_testutil import (GOLDEN_CASES, REF_TEST_EPS, assert_bitexact, assert_bounds_close, bounds_close,
                          clamp_inf, eps_band_mip, load_golden, permute, row_infeasible_mip)

pytestmark = pytest.mark.gpu

SYNCS = [gdp.CPU_LOOP, gdp.GPU_LOOP, gdp.MEGAKERNEL]
TRM, TILE = 32, 1024  # library defaults
ALL_LTR = 1 << 20      # thread_row_max that keeps every test row on the left-to-right path


def gpu(mip, sync=gdp.CPU_LOOP, max_rounds=0, trm=0, tile=0, lb=None, ub=None, marking=-1):
    return gdp.propagate(mip, sync_type=sync, max_rounds=max_rounds, thread_row_max=trm, split_tile=tile, lb=lb,
                         ub=ub, use_marking=marking)


def check_vs_oracle(mip, sync=gdp.CPU_LOOP, max_rounds=0, trm=TRM, tile=TILE, marking=-1):
    lb, ub, st = gpu(mip, sync, max_rounds, trm, tile, marking=marking)
    ref = oracle.propagate(mip, oracle.JACOBI, max_rounds=max_rounds, split_len=trm, split_tile=tile, nthreads=8)
    assert st["rounds"] == ref.rounds
    assert bool(st["infeasible"]) == ref.infeasible
    if ref.infeasible:
        assert st["infeasible_var"] == ref.infeasible_var
        assert st["infeasible_row"] == ref.infeasible_row
    assert_bitexact(lb, ub, ref.lb, ref.ub, what=f"sync={sync} trm={trm} tile={tile}")
    if marking == 2 and np.all(np.diff(mip.row_ptr) > 0):
        # always-on marking processes exactly the rows the oracle's marking processes
        assert st["rows_processed"] == ref.rows_processed
        assert st["nnz_processed"] == ref.nnz_processed
        # every row test decided like the oracle's, whether the FP32 screen,
        # the screen's bounds of max |a|(ub - lb) or the sequential EPS-max
        # decided it on the GPU
        assert st["rows_go"] == ref.rows_go
    return st


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("sync", SYNCS)
def test_golden_vs_reference_cpu_omp(name, sync):
    """Bit-exact against the reference's own cpu_omp round function (rows unsplit)."""
    mip, g = load_golden(name)
    lb, ub, st = gpu(mip, sync, trm=ALL_LTR)
    assert st["rounds"] == int(g["rounds_omp"])
    assert st["infeasible"] == int(g["infeasible_omp"])
    assert_bitexact(lb, ub, g["lb_omp"], g["ub_omp"], what=name)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_default_layout_vs_oracle(name):
    """Library defaults (long rows split into warp tiles) against the oracle's GPU mode."""
    mip, _ = load_golden(name)
    check_vs_oracle(mip, gdp.MEGAKERNEL)


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES])
def test_golden_vs_reference_cpu_seq(name):
    """Final bounds against the reference's cpu_seq: exact for integer
    variables and within 1e-9 rel / 1e-12 abs for continuous ones, except the
    two fixtures whose fixpoint is only reached in the limit (TwoLines,
    ATMSynthetic): there both schedules stop where the last improvement falls
    below GDP_EPS, and the reference's own tolerance (1e-4) applies."""
    mip, g = load_golden(name)
    lb, ub, st = gpu(mip)
    assert st["infeasible"] == int(g["infeasible_seq"])
    if int(g["infeasible_seq"]):
        return
    if name in ("two_lines", "atm_synthetic_2000"):
        np.testing.assert_allclose(clamp_inf(lb), clamp_inf(g["lb_seq"]), atol=REF_TEST_EPS)
        np.testing.assert_allclose(clamp_inf(ub), clamp_inf(g["ub_seq"]), atol=REF_TEST_EPS)
    else:
        assert_bounds_close(lb, ub, g["lb_seq"], g["ub_seq"], mip.vartype)


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if "analytical" in np.load(
    __import__("gdp_testutil").GOLDEN / f"{c}.npz").files])
def test_golden_analytical(name):
    mip, g = load_golden(name)
    lb, ub, _ = gpu(mip, gdp.MEGAKERNEL)
    np.testing.assert_allclose(clamp_inf(ub), clamp_inf(g["ub_analytical"]), atol=REF_TEST_EPS)
    np.testing.assert_allclose(clamp_inf(lb), clamp_inf(g["lb_analytical"]), atol=REF_TEST_EPS)


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("sync", SYNCS)
def test_random_small_mip(seed, sync):
    check_vs_oracle(gdpgen.random_mip(0, seed=100 + seed), sync)
    check_vs_oracle(gdpgen.random_mip(0, seed=100 + seed), sync, marking=2)


@pytest.mark.parametrize("trm,tile", [(4, 3), (8, 5), (16, 1), (2, 256), (1, 33)])
def test_split_rows_bitexact(trm, tile):
    """Force rows through the split (warp-tile) path; the oracle emulates its tree."""
    mip = gdpgen.random_mip(0, seed=7)
    for sync in SYNCS:
        check_vs_oracle(mip, sync, trm=trm, tile=tile)


@pytest.mark.parametrize("sync", SYNCS)
def test_marking_equals_full_sweep(sync):
    """Processing only rows with a changed variable gives the full-sweep result bit for bit."""
    mip = gdpgen.random_mip(1, seed=9, m=40_000, n=30_000, len_max=3000, dense_len=6000, n_dense_rows=2)
    a = gpu(mip, sync, trm=256, tile=512, marking=2)
    b = gpu(mip, sync, trm=256, tile=512, marking=0)
    assert a[2]["rounds"] == b[2]["rounds"]
    assert a[2]["rows_processed"] < b[2]["rows_processed"]
    assert_bitexact(a[0], a[1], b[0], b[1])


@pytest.mark.parametrize("seed", [1, 2])
def test_power_law_scaled(seed):
    mip = gdpgen.random_mip(1, seed=seed, m=100_000, n=75_000, len_max=5000, dense_len=20_000, n_dense_rows=4)
    for sync in SYNCS:
        st = check_vs_oracle(mip, sync, trm=1024, tile=1024)
        assert st["rounds"] >= 2


def test_power_law_small_tiles_and_threshold():
    mip = gdpgen.random_mip(1, seed=5, m=30_000, n=20_000, len_max=3000, dense_len=8000, n_dense_rows=3)
    check_vs_oracle(mip, gdp.MEGAKERNEL, trm=64, tile=512)
    check_vs_oracle(mip, gdp.CPU_LOOP, trm=256, tile=1024)


@pytest.mark.parametrize("sync", [gdp.CPU_LOOP, gdp.MEGAKERNEL])
def test_row_tests_decided_like_oracle(sync):
    """Rows at or near equality (the largest |a|(ub - lb) within EPS of the
    slack) are where the screen's bounds cannot decide the reference's row
    test: with marking on every round, the GPU passes exactly the rows the
    oracle passes, round by round, on power-law, chain and cover instances."""
    mips = [gdpgen.random_mip(1, seed=7, m=40_000, n=30_000, len_max=2000, dense_len=5000, n_dense_rows=2),
            gdpgen.chains(8000, chain_max=300, seed=5, frac_int_vars=1.0),
            gdpgen.cover_knapsack(20_000, 2_000, 16_000, 2_000, seed=2)]
    for mip in mips:
        st = check_vs_oracle(mip, sync, max_rounds=2000, marking=2)
        assert st["rows_go"] > 0


def test_chains_many_rounds():
    mip = gdpgen.chains(6000, chain_max=400, seed=2)
    for sync in SYNCS:
        for marking in (0, 1, 2):
            st = check_vs_oracle(mip, sync, max_rounds=5000, marking=marking)
            assert st["rounds"] > 100


def test_chains_infeasible():
    mip = gdpgen.chains(6000, chain_max=400, infeasible=True, seed=3)
    for sync in SYNCS:
        st = check_vs_oracle(mip, sync, max_rounds=5000)
        assert st["infeasible"] == 1


def test_cover_knapsack():
    mip = gdpgen.cover_knapsack(20_000, 2_000, 16_000, 2_000, seed=1)
    for sync in SYNCS:
        check_vs_oracle(mip, sync)


def test_round_cap_and_not_converged():
    mip, _ = load_golden("two_lines")
    for sync in SYNCS:
        lb, ub, st = gpu(mip, sync, max_rounds=5)
        ref = oracle.propagate(mip, oracle.JACOBI, max_rounds=5)
        assert st["rounds"] == 5 and not st["converged"]
        assert_bitexact(lb, ub, ref.lb, ref.ub)


def test_initially_infeasible_bounds():
    mip, _ = load_golden("savelsbergh1")
    lb = mip.lb.copy()
    lb[0] = 2.0
    for sync in SYNCS:
        _, _, st = gpu(mip, sync, lb=lb)
        assert st["infeasible"] == 1 and st["rounds"] == 0 and st["infeasible_var"] == 0


def test_row_permutation_bitexact():
    mip = gdpgen.random_mip(0, seed=21)
    perm = np.random.default_rng(1).permutation(mip.m)
    a = gpu(mip)
    b = gpu(permute(mip, row_perm=perm))
    assert a[2]["rounds"] == b[2]["rounds"]
    assert_bitexact(a[0], a[1], b[0], b[1])


def test_column_permutation():
    """Metamorphic check as in the reference's permute_mip: a column
    permutation reorders the sums, so bounds agree within tolerance."""
    mip = gdpgen.random_mip(0, seed=22)
    cp = np.random.default_rng(2).permutation(mip.n)
    a = gpu(mip)
    b = gpu(permute(mip, col_perm=cp))
    assert_bounds_close(a[0][cp], a[1][cp], b[0], b[1], mip.vartype[cp], rel=1e-9, abs_=1e-9)


def test_context_reuse_branch_and_bound_nodes():
    """One upload, many node bound vectors (fixings), each equal to a fresh run."""
    mip = gdpgen.random_mip(0, seed=23)
    rng = np.random.default_rng(3)
    ints = np.flatnonzero(mip.vartype != 3)
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL) as ctx:
        for _ in range(5):
            lb, ub = mip.lb.copy(), mip.ub.copy()
            fix = rng.choice(ints, size=10, replace=False)
            v = np.floor(rng.uniform(lb[fix], ub[fix] + 1))
            lb[fix] = np.minimum(v, ub[fix])
            ub[fix] = lb[fix]
            glb, gub, st = ctx.propagate(lb, ub)
            ref = oracle.propagate(mip, oracle.JACOBI, lb=lb, ub=ub)
            assert st["rounds"] == ref.rounds and bool(st["infeasible"]) == ref.infeasible
            assert_bitexact(glb, gub, ref.lb, ref.ub)


def test_device_pointer_entry_point():
    torch = pytest.importorskip("torch")
    mip = gdpgen.random_mip(0, seed=24)
    dlb = torch.tensor(mip.lb, dtype=torch.float64, device="cuda")
    dub = torch.tensor(mip.ub, dtype=torch.float64, device="cuda")
    with gdp.Context(mip) as ctx:
        st = ctx.propagate_device(dlb.data_ptr(), dub.data_ptr(), torch.cuda.current_stream().cuda_stream)
    ref = oracle.propagate(mip, oracle.JACOBI)
    assert st["rounds"] == ref.rounds
    assert_bitexact(dlb.cpu().numpy(), dub.cpu().numpy(), ref.lb, ref.ub)


def test_reference_python_driver_mirror():
    """Same call shape as the reference's fileReader/GPUDomPropInterface.py."""
    mip, g = load_golden("achterberg")
    for synctype in (0, 1, 2):
        lbs, ubs = gdp.propagateGPUAtomic(mip.n, mip.m, mip.nnz, list(mip.col), list(mip.row_ptr), list(mip.val),
                                          list(mip.lhs), list(mip.rhs), list(mip.lb), list(mip.ub),
                                          list(mip.vartype), synctype=synctype)
        assert_bitexact(np.array(lbs), np.array(ubs), g["lb_omp"], g["ub_omp"])
    lbs, ubs = gdp.propagateGPUReduction(mip.n, mip.m, mip.nnz, mip.col, mip.row_ptr, mip.val, mip.lhs, mip.rhs,
                                         mip.lb, mip.ub, mip.vartype)  # Achterberg rows have <= 10 non-zeros
    assert_bitexact(np.array(lbs), np.array(ubs), g["lb_omp"], g["ub_omp"])


def test_infinite_bound_forms():
    """ex1 mixes 1e100 / DBL_MAX / 1e20 infinities (reference test_setups.cuh:614-660)."""
    mip, g = load_golden("ex1")
    for sync in SYNCS:
        lb, ub, st = gpu(mip, sync)
        assert_bitexact(lb, ub, g["lb_omp"], g["ub_omp"])


def test_single_row_and_empty_rows():
    mip = gdp.MIP(np.array([0, 0, 3, 3], np.int32), np.array([0, 1, 2], np.int32), np.array([1.0, 2.0, -1.5]),
                  np.array([-1e20, 1.0, -1e20]), np.array([1e20, 4.0, 1e20]), np.zeros(3), np.array([5.0, 5.0, 2.0]),
                  np.array([1, 3, 3], np.int32))
    for sync in SYNCS:
        lb, ub, st = gpu(mip, sync)
        ref = oracle.propagate(mip, oracle.JACOBI)
        assert st["rounds"] == ref.rounds
        assert_bitexact(lb, ub, ref.lb, ref.ub)


@pytest.mark.parametrize("bad,msg", [("col", "column index out of range at non-zero 1"),
                                     ("val", "non-finite coefficient at non-zero 2")])
def test_invalid_elements_rejected_on_device(bad, msg):
    """Column range and finite coefficients are checked over the uploaded CSR;
    the error names the first bad non-zero, and the library stays usable."""
    col, val = [0, 1, 1, 0], [1.0, 2.0, 3.0, 4.0]
    if bad == "col":
        col = [0, 7, 1, -1]
    else:
        val = [1.0, 2.0, np.inf, np.nan]
    args = ([0, 2, 4], [1.0, 2.0], [3.0, 8.0])
    with pytest.raises(gdp.GDPError, match=msg):
        gdp.propagateGPUAtomic(2, 2, 4, col, args[0], val, [-1e20, -1e20], args[2], [0.0, 0.0], [10.0, 10.0],
                               [3, 3])
    lb, ub = gdp.propagateGPUAtomic(2, 2, 4, [0, 1, 1, 0], args[0], args[1] + [3.0, 4.0], [-1e20, -1e20], args[2],
                                    [0.0, 0.0], [10.0, 10.0], [3, 3])
    mip = gdp.MIP(np.array([0, 2, 4], np.int32), np.array([0, 1, 1, 0], np.int32), np.array([1.0, 2.0, 3.0, 4.0]),
                  np.array([-1e20, -1e20]), np.array([3.0, 8.0]), np.zeros(2), np.full(2, 10.0),
                  np.array([3, 3], np.int32))
    ref = oracle.propagate(mip, oracle.JACOBI)
    assert_bitexact(np.array(lb), np.array(ub), ref.lb, ref.ub)


def test_cached_device_memory_reuse_and_release():
    """Contexts draw on the memory that destroyed ones left cached; results do
    not depend on what the reused blocks held, and the cache can be freed."""
    mip_a = gdpgen.random_mip(1, seed=5, m=30_000, n=25_000, len_max=3000, dense_len=8000, n_dense_rows=2)
    mip_b = gdpgen.random_mip(1, seed=6, m=20_000, n=18_000, len_max=2000, dense_len=5000, n_dense_rows=2)
    ref_a = oracle.propagate(mip_a, oracle.JACOBI, split_len=TRM, split_tile=TILE, nthreads=8)
    ref_b = oracle.propagate(mip_b, oracle.JACOBI, split_len=TRM, split_tile=TILE, nthreads=8)
    for mip, ref in [(mip_a, ref_a), (mip_b, ref_b), (mip_a, ref_a), (mip_a, ref_a), (mip_b, ref_b)]:
        for sync in SYNCS:
            lb, ub, st = gpu(mip, sync)
            assert st["rounds"] == ref.rounds
            assert_bitexact(lb, ub, ref.lb, ref.ub)
    gdp.release_cached_memory()
    lb, ub, st = gpu(mip_b, gdp.MEGAKERNEL)
    assert_bitexact(lb, ub, ref_b.lb, ref_b.ub)
    gdp.release_cached_memory()


def test_propagate_into_separate_and_aliased_outputs():
    """gdp_propagate_into leaves its inputs alone, and equals gdp_propagate
    (in place) when an output is its input."""
    mip = gdpgen.random_mip(0, seed=11)
    ref = oracle.propagate(mip, oracle.JACOBI, split_len=TRM, split_tile=TILE, nthreads=8)
    lib = gdp.load_library()
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL) as ctx:
        lb_in, ub_in = mip.lb.astype(np.float64).copy(), mip.ub.astype(np.float64).copy()
        keep_lb, keep_ub = lb_in.copy(), ub_in.copy()
        lbo, ubo = np.full_like(lb_in, np.nan), np.full_like(ub_in, np.nan)
        st = gdp.Stats()
        assert lib.gdp_propagate_into(ctx._h, gdp._pd(lb_in), gdp._pd(ub_in), gdp._pd(lbo), gdp._pd(ubo),
                                      None) == gdp.GDP_OKAY
        assert_bitexact(lbo, ubo, ref.lb, ref.ub)
        assert np.array_equal(lb_in, keep_lb) and np.array_equal(ub_in, keep_ub)
        assert lib.gdp_propagate_into(ctx._h, gdp._pd(lb_in), gdp._pd(ub_in), gdp._pd(lb_in), gdp._pd(ub_in),
                                      st) == gdp.GDP_OKAY
        assert_bitexact(lb_in, ub_in, ref.lb, ref.ub)
        assert st.rounds == ref.rounds


def test_stats_accounting():
    mip = gdpgen.random_mip(0, seed=25)
    _, _, st = gpu(mip, gdp.MEGAKERNEL, marking=0)
    assert st["rows_processed"] == st["rounds"] * mip.m
    assert st["nnz_processed"] == st["rounds"] * mip.nnz
    assert st["bytes_algorithmic"] == st["rounds"] * (12.0 * mip.nnz + 20.0 * mip.m + 36.0 * mip.n)
    assert st["device_ms"] > 0 and st["kernel_launches"] >= 2
    _, _, sm = gpu(mip, gdp.MEGAKERNEL, marking=2)
    # bytes of the rows read: split rows left unread on their drift bound are not
    assert sm["bytes_algorithmic"] == 12.0 * (sm["nnz_processed"] - sm["nnz_drift"]) + \
        20.0 * (sm["rows_processed"] - sm["rows_drift"]) + 36.0 * mip.n * sm["rounds"]


def test_gpu_loop_graph_reused_and_cap_changes():
    """The GPU_LOOP graph is built once per context and rebuilt when the round cap changes."""
    mip, _ = load_golden("two_lines")
    with gdp.Context(mip, sync_type=gdp.GPU_LOOP) as ctx:
        a = ctx.propagate()
        b = ctx.propagate()
        assert a[2]["rounds"] == b[2]["rounds"] == 61
        ctx.set_options(max_rounds=7, sync_type=gdp.GPU_LOOP)
        c = ctx.propagate()
        assert c[2]["rounds"] == 7 and not c[2]["converged"]


def _extreme_mip(seed, m=1500, n=4000, long_rows=6):
    """Rows whose FP32 screen is stressed: coefficients from 1e-30 to 1e30,
    bounds from subnormal to 1e19 and every infinity form, zero-slack
    equalities, exact cancellation pairs, and split-length rows."""
    rng = np.random.default_rng(seed)
    lens = np.concatenate([rng.integers(1, 40, m - long_rows), rng.integers(1100, 3000, long_rows)])
    rng.shuffle(lens)
    row_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    nnz = int(row_ptr[-1])
    col = np.concatenate([rng.choice(n, L, replace=False) for L in lens]).astype(np.int32)
    val = rng.choice([-1.0, 1.0], nnz) * 10.0 ** rng.uniform(-30, 30, nnz)
    small = rng.random(nnz) < 0.5
    val[small] = rng.choice([-1.0, 1.0], small.sum()) * rng.uniform(0.5, 10, small.sum())
    # cancellation pairs inside rows: a, -a
    for i in rng.choice(m, m // 10, replace=False):
        b, e = row_ptr[i], row_ptr[i + 1]
        if e - b >= 2:
            val[b + 1] = -val[b]
    kind = rng.integers(0, 8, n)
    lb = -rng.uniform(0, 100, n)
    ub = rng.uniform(0, 100, n)
    lb[kind == 1] = -1e20
    ub[kind == 2] = 1e100
    lb[kind == 3] = -np.inf
    ub[kind == 4] = 5e-320  # subnormal
    lb[kind == 4] = -0.0
    lb[kind == 5], ub[kind == 5] = -1e19, 1e19
    lb[kind == 6], ub[kind == 6] = 0.0, 0.0
    vt = np.where(rng.random(n) < 0.5, 1, 3).astype(np.int32)
    ilb, iub = np.ceil(lb), np.floor(ub)
    fin = np.isfinite(ilb) & (np.abs(ilb) < 1e20)
    lb = np.where((vt != 3) & fin, ilb, lb)
    fin = np.isfinite(iub) & (np.abs(iub) < 1e20)
    ub = np.where((vt != 3) & fin, iub, ub)
    ub = np.maximum(ub, lb)
    x0 = np.clip(np.zeros(n), np.maximum(lb, -1e6), np.minimum(ub, 1e6))
    rows = np.repeat(np.arange(m), lens)
    ax = np.bincount(rows, val * x0[col], m)
    form = rng.integers(0, 5, m)
    slack = np.abs(ax) * rng.uniform(0, 1e-3, m)
    lhs = np.where(form == 0, ax, ax - slack)
    rhs = np.where(form == 0, ax, ax + slack)
    lhs[form == 1] = -1e20
    rhs[form == 2] = np.inf
    lhs[form == 3], rhs[form == 3] = -1e100, 1e100
    return gdp.MIP(row_ptr, col, val, lhs, rhs, lb, ub, vt)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("sync", [gdp.CPU_LOOP, gdp.MEGAKERNEL])
def test_screen_extreme_magnitudes(seed, sync):
    """The FP32 screen only skips rows the exact rule skips: bit-exact with the
    oracle on magnitudes that overflow, underflow and cancel in FP32."""
    mip = _extreme_mip(seed)
    st = check_vs_oracle(mip, sync)
    assert st["nnz_exact"] <= st["nnz_processed"]
    st = check_vs_oracle(mip, sync, trm=4, tile=64, marking=2)


def test_screen_skips_work():
    """On the power-law instance the screen keeps most non-zeros away from the FP64 pass."""
    mip = gdpgen.random_mip(1, seed=3, m=60_000, n=45_000, n_dense_rows=2, dense_len=20_000)
    st = check_vs_oracle(mip, gdp.MEGAKERNEL)
    assert st["nnz_exact"] < 0.5 * st["nnz_processed"]


@pytest.mark.parametrize("sync", SYNCS)
def test_row_infeasible_without_variable_crossing(sync):
    """The row rule flags a row whose maximum activity is below its lhs while
    no variable crosses beyond its tolerance; the round completes as in the
    oracle (bounds equal), and the stats name the row."""
    mip = row_infeasible_mip()
    lb, ub, st = gpu(mip, sync)
    assert st["infeasible"] == 1 and st["rounds"] == 1 and st["converged"] == 1
    assert st["infeasible_row"] == 0 and st["infeasible_var"] == -1
    ref = oracle.propagate(mip, oracle.JACOBI)
    assert_bitexact(lb, ub, ref.lb, ref.ub)
    # the same row inside a larger instance, placed as a long split row
    big = gdpgen.random_mip(0, seed=31)
    check_vs_oracle(big, sync)


@pytest.mark.parametrize("blocker", [True, False])
@pytest.mark.parametrize("length,trm,tile", [(64, 32, 1024), (700, 32, 1024), (3000, 32, 1024), (64, 4, 16)])
def test_eps_band_rows_decided_like_reference(blocker, length, trm, tile):
    """Rows summed by several lanes (64 and 700 non-zeros) or in warp tiles
    (3000 non-zeros; 64 with 16-element tiles) whose largest |a|(ub-lb)
    exceeds the slack by 1.5e-9: only the reference's sequential EPS-max
    decides them (an element 0.8e-9 below the maximum, earlier in the row,
    makes the reference skip the row). The GPU computes that EPS-max and
    reaches the reference's result bit for bit (the reference harness's own
    cpu_omp round function agrees, tests/test_oracle.py)."""
    mip = eps_band_mip(length, blocker, q=3, p=length - 5)
    ref = oracle.propagate(mip, oracle.JACOBI)
    for sync in SYNCS:
        lb, ub, st = gpu(mip, sync, trm=trm, tile=tile, marking=0)
        assert st["rounds"] == ref.rounds
        assert_bitexact(lb, ub, ref.lb, ref.ub, what=f"blocker={blocker} len={length} sync={sync}")
        assert st["rows_seqmax"] >= 1
        assert ub[length - 5] == (1.0 + 1.5e-9 if blocker else 1.0)


def _deviation(a_lb, a_ub, b_lb, b_ub, vt):
    """Per variable: integer bounds unequal, continuous bounds beyond 1e-9 rel / 1e-12 abs."""
    is_int = vt != 3
    bad_int, bad_cont = np.zeros(len(vt), bool), np.zeros(len(vt), bool)
    for x, y in ((a_lb, b_lb), (a_ub, b_ub)):
        x, y = clamp_inf(x), clamp_inf(y)
        bad_int |= is_int & (x != y)
        bad_cont |= (~is_int) & ~(np.abs(x - y) <= 1e-12 + 1e-9 * np.abs(y))
    return bad_int, bad_cont


def test_power_law_vs_reference_semantics():
    """The library defaults (rows split into lane groups and warp tiles) on a
    300k-row power-law MIP (the large generator scaled down, 5.0M non-zeros)
    against the reference's own semantics, not the oracle's GPU mode:
      * the reference's cpu_omp round function (oracle JACOBI, left-to-right
        sums): the same round count and verdict, integer bounds bit for bit,
        continuous bounds within 1e-9 rel / 1e-12 abs;
      * the reference's cpu_seq (oracle SEQUENTIAL) on the same generator
        without equality rows: the same verdict and integer bounds bit for
        bit; the continuous bounds that differ by more than 1e-9 are exactly
        those where cpu_omp and cpu_seq themselves differ (Jacobi and
        Gauss-Seidel stop where their last improvement falls below GDP_EPS,
        at different points of a limit). With equality rows (tight at the
        generating point) cpu_seq amplifies rounding through coefficient
        ratios and can cut that point off; there cpu_omp is the reference
        schedule to compare with."""
    mip = gdpgen.random_mip(1, seed=11, m=300_000, n=225_000, len_max=5000, dense_len=20_000, n_dense_rows=4)
    lb, ub, st = gpu(mip, gdp.MEGAKERNEL)
    omp = oracle.propagate(mip, oracle.JACOBI, nthreads=8)
    assert st["rounds"] == omp.rounds and bool(st["infeasible"]) == omp.infeasible
    bi, bc = _deviation(lb, ub, omp.lb, omp.ub, mip.vartype)
    assert bi.sum() == 0 and bc.sum() == 0, (int(bi.sum()), int(bc.sum()))

    noeq = gdpgen.random_mip(1, seed=11, m=300_000, n=225_000, len_max=5000, dense_len=20_000, n_dense_rows=4,
                             frac_equality=0.0)
    lb, ub, st = gpu(noeq, gdp.MEGAKERNEL)
    omp = oracle.propagate(noeq, oracle.JACOBI, nthreads=8)
    seq = oracle.propagate(noeq, oracle.SEQUENTIAL)
    assert st["rounds"] == omp.rounds
    assert bool(st["infeasible"]) == seq.infeasible == omp.infeasible
    bi, bc = _deviation(lb, ub, omp.lb, omp.ub, noeq.vartype)
    assert bi.sum() == 0 and bc.sum() == 0
    bi, bc = _deviation(lb, ub, seq.lb, seq.ub, noeq.vartype)
    ri, rc = _deviation(omp.lb, omp.ub, seq.lb, seq.ub, noeq.vartype)
    assert bi.sum() == 0
    assert not np.any(bc & ~rc), "the GPU differs from cpu_seq where cpu_omp does not"


def test_drift_bound_skips_split_rows_bitexact():
    """Marked rounds leave a split row unread while the certified margin of its
    last screen covers every tightening of its variables since (the drift
    bound): on a power-law MIP with long rows such skips happen, and with
    marking on every round the result, the round count and the work counters
    (rows and non-zeros screened, rows through the row test) equal the
    oracle's, which screens every marked row."""
    mip = gdpgen.random_mip(1, seed=3, m=200_000, n=150_000, len_max=5000, dense_len=20_000, n_dense_rows=4)
    for sync in SYNCS:
        st = check_vs_oracle(mip, sync, trm=32, tile=1024, marking=2)
        assert st["rows_drift"] > 0 and st["nnz_drift"] > 1024 * st["rows_drift"], sync
    # the library defaults (adaptive marking) against the reference's cpu_omp semantics
    lb, ub, st = gpu(mip, gdp.MEGAKERNEL)
    omp = oracle.propagate(mip, oracle.JACOBI, nthreads=8)
    assert st["rounds"] == omp.rounds and st["rows_drift"] > 0
    bi, bc = _deviation(lb, ub, omp.lb, omp.ub, mip.vartype)
    assert bi.sum() == 0 and bc.sum() == 0


def test_barrier_wait_limit_returns_error_and_library_stays_usable():
    """A grid-barrier wait that runs out records a device error instead of
    waiting on: with a limit of 1,000 SM cycles (the first barrier of a round
    waits for the slowest CTA's phase work, tens of thousands of cycles on
    this instance) the first CTAs to arrive give up, every CTA leaves at its
    next barrier, and the call returns GDP_ERROR with the timeout message.
    The library stays usable: a fresh context then propagates correctly."""
    mip = gdpgen.random_mip(1, seed=7, m=40_000, n=30_000, len_max=2000, dense_len=5000, n_dense_rows=2)
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL, barrier_wait_kcycles=1) as ctx:
        with pytest.raises(gdp.GDPError, match="grid barrier wait exceeded its limit"):
            ctx.propagate()
    ref = oracle.propagate(mip, oracle.JACOBI, split_len=TRM, split_tile=TILE, nthreads=8)
    with gdp.Context(mip, sync_type=gdp.MEGAKERNEL) as ctx:
        lb, ub, st = ctx.propagate()
    assert st["rounds"] == ref.rounds and st["device_error"] == 0
    assert_bitexact(lb, ub, ref.lb, ref.ub)
