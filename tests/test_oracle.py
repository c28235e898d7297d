"""CPU tests of the oracle: known answers from the reference's unit tests,
the reference's analytical fixtures, and bit-exact agreement with the
reference's own round functions (golden outputs, and live where the reference
harness is built)."""
import ctypes as C

import numpy as np
import pytest

import gdpgen
import oracle
from gdp_testutil import (GOLDEN_CASES, REF_TEST_EPS, assert_bitexact, assert_bounds_close, clamp_inf,
                          load_golden, permute)

INF = 1e20


# ---- known-answer tests: reference test/testCases/test_propagator.cuh ----
def test_adjust_bounds_kat():  # :4-38
    o = oracle.lib()
    assert o.gdpo_adjust_upper(1, 3.7) == 3.7
    assert o.gdpo_adjust_upper(0, -3.7) == -4.0
    assert o.gdpo_adjust_lower(1, -3.7) == -3.7
    assert o.gdpo_adjust_lower(0, 3.7) == 4.0


def test_is_bound_better_kat():  # :40-100
    o = oracle.lib()
    assert o.gdpo_is_ub_better(-0.5, 3.0, 1.5)
    assert not o.gdpo_is_ub_better(-0.5, 3.0, 3.2)
    assert o.gdpo_is_ub_better(-0.5, 0.001, -0.001)
    assert o.gdpo_is_ub_better(-3.5, -1.0, -2.0)
    assert not o.gdpo_is_lb_better(-1.0, 1.0, -1.5)
    assert o.gdpo_is_lb_better(-1.0, 1.0, -0.5)
    assert o.gdpo_is_lb_better(-0.001, 1.0, 0.001)
    assert o.gdpo_is_lb_better(0.5, 1.0, 0.9)


def test_can_cons_be_tightened_kat():  # :102-117
    o = oracle.lib()
    assert not o.gdpo_can_cons_be_tightened(0.0, 10.8, 0, 0, 0.0, 9.1, 3.8)
    assert o.gdpo_can_cons_be_tightened(0.0, 3.8, 0, 0, 0.0, 2.0, 2.8)


def test_is_cons_infeasible_kat():  # :119-135
    o = oracle.lib()
    assert o.gdpo_is_cons_infeasible(9.1, 10.8, 3.2, 3.8)
    assert not o.gdpo_is_cons_infeasible(-2.0, 10.0, 3.2, -3.8)


def _tu(coeff, slack, surplus, ninf, lb, ub, cont):
    out = C.c_double()
    t = oracle.lib().gdpo_tighten_var_upper(coeff, slack, surplus, ninf, lb, ub, int(cont), C.byref(out))
    return bool(t), out.value


def _tl(coeff, slack, surplus, ninf, lb, ub, cont):
    out = C.c_double()
    t = oracle.lib().gdpo_tighten_var_lower(coeff, slack, surplus, ninf, lb, ub, int(cont), C.byref(out))
    return bool(t), out.value


def test_tighten_var_bounds_kat():  # :137-249
    assert _tu(1.0, 13.0, INF, 0, -10.0, 10.0, True) == (True, pytest.approx(3.0, abs=1e-6))
    assert _tu(-2.0, 45.0, -109.0, 0, 0.0, 100.0, False) == (True, pytest.approx(54.0, abs=1e-6))
    assert _tu(-2.0, 45.0, -109.0, 0, 0.0, 100.0, True) == (True, pytest.approx(54.5, abs=1e-6))
    assert _tl(1.0, INF, -5.1, 0, -100.0, 10.0, True) == (True, pytest.approx(4.9, abs=1e-6))
    assert _tl(1.0, INF, -5.1, 0, -100.0, 10.0, False) == (True, pytest.approx(5.0, abs=1e-6))
    assert _tl(-10.5, 10.5, 0.0, 0, -7.5, -3.0, True) == (True, pytest.approx(-4.0, abs=1e-6))
    assert _tl(-10.5, 10.5, 0.0, 0, -7.5, -3.0, False) == (True, pytest.approx(-4.0, abs=1e-6))


def test_infinity_forms():
    # ISPOSINF / ISNEGINF of the reference (src/def.h:78-79) are plain >= / <= 1e20 comparisons for
    # every double; the activity of a row sees 1e20, 1e100, DBL_MAX and inf alike.
    mip, _ = load_golden("ex1")
    a = oracle.activities(mip, 0)
    assert a["maxact_inf"] == 2 and a["minact_inf"] == 0


# ---- analytical fixtures (reference test/test_setups.cuh) ----
@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES])
@pytest.mark.parametrize("schedule", [oracle.JACOBI, oracle.SEQUENTIAL])
def test_oracle_matches_reference_golden(name, schedule):
    mip, g = load_golden(name)
    tag = "omp" if schedule == oracle.JACOBI else "seq"
    r = oracle.propagate(mip, schedule)
    assert r.rounds == int(g[f"rounds_{tag}"])
    assert r.infeasible == bool(g[f"infeasible_{tag}"])
    assert_bitexact(r.lb, r.ub, g[f"lb_{tag}"], g[f"ub_{tag}"], what=f"{name}/{tag}")


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if "analytical" in np.load(
    __import__("gdp_testutil").GOLDEN / f"{c}.npz").files])
def test_reference_analytical_solutions(name):
    mip, g = load_golden(name)
    for tag in ("omp", "seq"):
        np.testing.assert_allclose(clamp_inf(g[f"ub_{tag}"]), clamp_inf(g["ub_analytical"]), atol=REF_TEST_EPS)
        np.testing.assert_allclose(clamp_inf(g[f"lb_{tag}"]), clamp_inf(g["lb_analytical"]), atol=REF_TEST_EPS)


def test_jacobi_thread_count_independent():
    mip = gdpgen.random_mip(0, seed=11)
    r1 = oracle.propagate(mip, oracle.JACOBI, nthreads=1)
    r4 = oracle.propagate(mip, oracle.JACOBI, nthreads=4)
    assert r1.rounds == r4.rounds
    assert_bitexact(r1.lb, r1.ub, r4.lb, r4.ub)


def test_row_permutation_invariance():
    mip = gdpgen.random_mip(0, seed=12)
    perm = np.random.default_rng(5).permutation(mip.m)
    a = oracle.propagate(mip, oracle.JACOBI)
    b = oracle.propagate(permute(mip, row_perm=perm), oracle.JACOBI)
    assert a.rounds == b.rounds
    assert_bitexact(a.lb, a.ub, b.lb, b.ub)


def test_column_permutation_invariance():
    mip = gdpgen.random_mip(0, seed=13)
    cp = np.random.default_rng(6).permutation(mip.n)
    a = oracle.propagate(mip, oracle.JACOBI)
    b = oracle.propagate(permute(mip, col_perm=cp), oracle.JACOBI)
    assert_bounds_close(a.lb[cp], a.ub[cp], b.lb, b.ub, mip.vartype[cp], what="column permutation")


def test_infeasible_fixture_flagged():
    mip, g = load_golden("random_mip_infeasible")
    r = oracle.propagate(mip, oracle.JACOBI)
    assert r.infeasible and int(g["infeasible_omp"]) == 1
    assert r.infeasible_var >= 0


def test_initially_crossing_bounds_infeasible_in_round_zero():
    mip, _ = load_golden("savelsbergh1")
    lb = mip.lb.copy()
    lb[0] = 2.0  # ub is 1
    r = oracle.propagate(mip, oracle.JACOBI, lb=lb)
    assert r.infeasible and r.rounds == 0 and r.infeasible_var == 0


def test_round_cap():
    mip, g = load_golden("two_lines")
    r = oracle.propagate(mip, oracle.JACOBI, max_rounds=5)
    assert r.rounds == 5 and not r.converged


# ---- live comparison with the reference's own code (build container only) ----
needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built here")


@needs_ref
@pytest.mark.parametrize("seed", [21, 22, 23])
@pytest.mark.parametrize("schedule", [oracle.JACOBI, oracle.SEQUENTIAL])
def test_oracle_matches_reference_live(seed, schedule):
    mip = gdpgen.random_mip(0, seed=seed, m=3000, n=2000, len_max=40)
    r = oracle.propagate(mip, schedule)
    ref = oracle.ref_propagate(mip, schedule)
    assert r.rounds == ref.rounds and r.infeasible == ref.infeasible
    assert_bitexact(r.lb, r.ub, ref.lb, ref.ub)


@needs_ref
def test_oracle_matches_reference_live_power_law_sequential():
    mip = gdpgen.random_mip(1, seed=3, m=20000, n=15000, len_max=2000, dense_len=5000, n_dense_rows=2)
    r = oracle.propagate(mip, oracle.SEQUENTIAL)
    ref = oracle.ref_propagate(mip, oracle.SEQUENTIAL)
    assert r.rounds == ref.rounds and r.infeasible == ref.infeasible
    assert_bitexact(r.lb, r.ub, ref.lb, ref.ub)


# The reference's cpu_omp applies a variable's candidates in thread-arrival
# order and keeps the first of two candidates within GDP_EPS of each other, so
# on instances with equality rows (many near-ties) its own result varies from
# run to run; the oracle keeps the tighter candidate (order-independent). The
# JACOBI schedule is therefore compared live on instances without equality rows
# (test_oracle_matches_reference_live), and the deterministic SEQUENTIAL
# schedule on every family.


def test_split_order_emulation_changes_only_long_rows():
    # rows no longer than split_len keep the left-to-right order exactly
    mip = gdpgen.random_mip(0, seed=14)
    a = oracle.propagate(mip, oracle.JACOBI)
    b = oracle.propagate(mip, oracle.JACOBI, split_len=16, split_tile=4)
    assert a.rounds == b.rounds
    assert_bitexact(a.lb, a.ub, b.lb, b.ub)
    c = oracle.propagate(mip, oracle.JACOBI, split_len=4, split_tile=3)
    assert_bounds_close(a.lb, a.ub, c.lb, c.ub, mip.vartype, rel=1e-9, abs_=1e-9)


@needs_ref
def test_oracle_matches_reference_live_chains():
    mip = gdpgen.chains(4000, chain_max=300, seed=4)
    r = oracle.propagate(mip, oracle.JACOBI, max_rounds=2000)
    assert r.rounds > 100  # chains drive propagation past the reference's 100-round cap
    s = oracle.propagate(mip, oracle.SEQUENTIAL, max_rounds=2000)
    rs = oracle.ref_propagate(mip, oracle.SEQUENTIAL, max_rounds=2000)
    assert s.rounds == rs.rounds
    assert_bitexact(s.lb, s.ub, rs.lb, rs.ub)


@needs_ref
def test_infeasible_chain_detected_like_reference():
    mip = gdpgen.chains(4000, chain_max=300, infeasible=True, seed=4)
    r = oracle.propagate(mip, oracle.SEQUENTIAL, max_rounds=2000)
    ref = oracle.ref_propagate(mip, oracle.SEQUENTIAL, max_rounds=2000)
    assert r.infeasible and ref.infeasible and r.rounds == ref.rounds
    assert oracle.propagate(mip, oracle.JACOBI, max_rounds=2000).infeasible


# ---- the row rule and the EPS band of the row test -------------------------
def test_row_rule_flags_infeasible_row():
    """A row whose activities exclude its sides is infeasible even when no
    variable crosses beyond the variable rule's tolerance (both schedules,
    GPU mode, and the reference harness applying the same rule to the
    activities its own round functions computed)."""
    from gdp_testutil import row_infeasible_mip
    mip = row_infeasible_mip()
    for kw in (dict(schedule=oracle.JACOBI), dict(schedule=oracle.SEQUENTIAL),
               dict(schedule=oracle.JACOBI, split_len=1, split_tile=1)):
        r = oracle.propagate(mip, **kw)
        assert r.infeasible and r.rounds == 1, kw
        assert r.infeasible_row == 0 and r.infeasible_var == -1, kw
    o = oracle.lib()
    assert o.gdpo_row_infeasible(0.0, 0.0, 0, 0, 1e-3, 1e20)
    assert not o.gdpo_row_infeasible(0.0, 0.0, 0, 1, 1e-3, 1e20)  # an infinite contribution: no verdict
    assert not o.gdpo_row_infeasible(0.0, 0.0, 0, 0, 5e-7, 1e20)  # within the tolerance
    assert o.gdpo_row_infeasible(2.5, 9.0, 0, 0, -1e20, 2.0)
    if oracle.ref_available():
        for schedule in (oracle.JACOBI, oracle.SEQUENTIAL):
            r = oracle.ref_propagate(mip, schedule)
            assert r.infeasible and r.rounds == 1


@pytest.mark.parametrize("blocker", [True, False])
def test_eps_band_row_test(blocker):
    """The reference's sequential EPS-max decides the row test when the row's
    maximum |a|(ub-lb) exceeds the slack by EPS to 2 EPS: with an earlier
    element within EPS below the maximum the row is skipped, without it the
    maximum's variable tightens. The GPU mode (rows summed in lane groups or
    warp tiles) decides like the reference."""
    from gdp_testutil import eps_band_mip
    for length, trm, tile in ((64, 32, 1024), (3000, 32, 1024), (64, 4, 16)):
        mip = eps_band_mip(length, blocker, q=3, p=length - 5)
        ref = oracle.propagate(mip, oracle.JACOBI)
        gpu_mode = oracle.propagate(mip, oracle.JACOBI, split_len=trm, split_tile=tile)
        seq = oracle.propagate(mip, oracle.SEQUENTIAL)
        p = length - 5
        if blocker:
            assert ref.rounds == 1 and ref.ub[p] == 1.0 + 1.5e-9
        else:
            assert ref.rounds == 2 and ref.ub[p] == 1.0
        assert_bitexact(gpu_mode.lb, gpu_mode.ub, ref.lb, ref.ub)
        assert_bitexact(seq.lb, seq.ub, ref.lb, ref.ub)
        if oracle.ref_available():
            r = oracle.ref_propagate(mip, oracle.JACOBI)
            assert_bitexact(r.lb, r.ub, ref.lb, ref.ub)
