"""Learned row marking: the trace logger, the learned round loop and the
training pipeline. Whatever the model selects, a propagation ends only after a
full round that changes nothing, so its bounds are a fixpoint of the same
operator. On instances whose fixpoint does not depend on the processing order
(integer bounds; checked: the oracle's Jacobi and Gauss-Seidel schedules agree
on them) it is the plain propagation's fixpoint bit for bit."""
import numpy as np
import pytest

import gdp
import gdpgen
from gdp_testutil import assert_bitexact

pytestmark = pytest.mark.gpu


def _plain(mip):
    return gdp.propagate(mip, sync_type=gdp.MEGAKERNEL)


def _cover(seed, scale=1):
    return gdpgen.cover_knapsack(20_000 * scale, 2_000 * scale, 16_000 * scale, 2_000 * scale, seed=seed)


def _ctx(mip, model=None, threshold=0.0, max_rounds=0, min_len=0):
    c = gdp.Context(mip, sync_type=gdp.MEGAKERNEL, max_rounds=max_rounds)
    if model is not None:
        c.set_model(model, threshold, min_len)
    return c



def test_trace_logs_marked_rows_and_keeps_bounds():
    mip = gdpgen.chains(60_000, chain_max=90, seed=5, frac_int_vars=1.0)
    lb, ub, st = _plain(mip)
    assert st["converged"] and not st["infeasible"]
    c = _ctx(mip)
    x, y, tlb, tub, tst = c.trace(capacity=500_000)
    assert_bitexact(tlb, tub, lb, ub, what="trace bounds")
    assert tst["converged"] and tst["full_rounds"] >= 1  # the first round; a FULL or FLUSH round certifies
    assert len(x) > 0 and x.shape[1] == 16
    assert set(np.unique(y)) <= {0.0, 1.0} and 0 < y.mean() < 1
    assert np.all(np.isfinite(x)) and np.all(np.abs(x) <= 1.0 + 1e-6)
    # capacity caps the samples
    x2, y2, *_ = _ctx(mip).trace(capacity=100)
    assert len(x2) == 100


@pytest.mark.parametrize("threshold", [-1e30, 0.0, 1e30])
def test_learned_rounds_reach_plain_fixpoint(threshold):
    """Select all (exact marking), a random model, and defer all: the same fixpoint."""
    for mip in (_cover(1), gdpgen.chains(60_000, chain_max=90, seed=6, frac_int_vars=1.0)):
        lb, ub, st = _plain(mip)
        assert st["converged"] and not st["infeasible"]
        # deferring every marked row doubles the rounds of a chain: room for them
        c = _ctx(mip, gdp.Mlp(seed=3), threshold, max_rounds=1000)
        llb, lub, lst = c.propagate()
        assert lst["converged"] and not lst["infeasible"]
        assert_bitexact(llb, lub, lb, ub, what=f"threshold {threshold}")
        if threshold < -1e29:
            assert lst["rows_deferred"] == 0
        if threshold > 1e29:
            assert lst["rows_deferred"] > 0 or lst["rounds"] <= 2


def test_learned_rounds_on_fragile_instance():
    """On chain MIPs with continuous equality cycles the processing order decides
    whether rounding drift crosses the infeasibility tolerance: the reference's
    own cpu_seq reports this instance infeasible while the Jacobi schedule does
    not. Learned rounds must end certified either way (a full or flush round
    without change, or an infeasibility verdict), never at a round-cap surprise."""
    mip = gdpgen.chains(60_000, chain_max=90, seed=6)
    _, _, lst = _ctx(mip, gdp.Mlp(seed=4), 0.0, max_rounds=1000).propagate()
    assert lst["converged"]
    assert lst["infeasible"] or lst["full_rounds"] >= 1


def test_learned_infeasible_detected():
    mip = gdpgen.chains(20_000, chain_max=60, seed=4, infeasible=True)
    _, _, st = _plain(mip)
    _, _, lst = _ctx(mip, gdp.Mlp(seed=1), 0.0).propagate()
    assert st["infeasible"] and lst["infeasible"]


def test_train_on_traces_and_gain():
    """Trace -> train on the GPU -> learned marking on a held-out seed: the
    same certified fixpoint as plain propagation (bit for bit on this
    all-integer chain MIP), with less than half the non-zeros of the plain
    full sweep every round (the reference's GPU schedule). Against exact
    marking (the engine's own marking without the model) the learned rounds
    process about as many non-zeros on such chains: that comparison is
    printed, not asserted (bench.py reports it on the chain workload)."""
    import marking
    x, y = marking.collect_traces(gdpgen.chains(60_000, chain_max=90, seed=100 + s, frac_int_vars=1.0) for s in range(4))
    assert len(y) > 1000 and 0 < y.mean() < 1
    model, tau, info = marking.train_marking_model(x, y, epochs=4, batch=4096, seed=7, recall=0.98, min_len=8)
    assert info["loss"] < 0.69 and info["recall"] >= 0.97
    held = gdpgen.chains(60_000, chain_max=90, seed=999, frac_int_vars=1.0)
    lb, ub, st = _plain(held)
    _, _, _, _, exact_st = _ctx(held, max_rounds=1000).trace(capacity=0)
    c = _ctx(held, model, tau, max_rounds=1000, min_len=8)
    llb, lub, lst = c.propagate()
    print("learned", {k: lst[k] for k in ("rounds", "rows_processed", "nnz_processed", "rows_deferred",
                                          "full_rounds", "device_ms", "converged")},
          "exact", {k: exact_st[k] for k in ("rounds", "rows_processed", "nnz_processed", "device_ms")},
          "plain", {k: st[k] for k in ("rounds", "rows_processed", "nnz_processed", "device_ms")}, info)
    assert lst["converged"]
    assert_bitexact(llb, lub, lb, ub, what="held-out")
    assert lst["rows_deferred"] > 0
    full = gdp.propagate(held, sync_type=gdp.MEGAKERNEL, use_marking=0)[2]
    # against the plain full sweep every round (the reference's schedule)
    assert lst["nnz_processed"] < 0.5 * full["nnz_processed"]
    print("full sweep", {k: full[k] for k in ("rounds", "rows_processed", "nnz_processed", "device_ms")})


@pytest.mark.parametrize("threshold", [-1e30, 0.0, 1e30])
def test_learned_batch_equals_single_learned(threshold):
    """Learned marking inside an instance batch: every member takes exactly the
    rounds of its own single-problem learned propagation -- bounds bit for bit,
    round count, verdict, deferred rows and full rounds -- with an infeasible
    member and members of different sizes in the one launch."""
    mips = [gdpgen.chains(12_000 + 9_000 * s, chain_max=80, seed=60 + s, frac_int_vars=1.0) for s in range(3)]
    mips.append(gdpgen.chains(15_000, chain_max=60, seed=64, infeasible=True, frac_int_vars=1.0))
    mips.append(_cover(3))
    model = gdp.Mlp(seed=5)
    b = gdp.Batch.instances(mips, max_rounds=1000)
    b.set_model(model, threshold, 8)
    for _ in range(2):  # the second call replays the captured graph
        lbs, ubs, sts, tot = b.propagate([m.lb for m in mips], [m.ub for m in mips])
        for k, m in enumerate(mips):
            lb, ub, st = _ctx(m, model, threshold, max_rounds=1000, min_len=8).propagate()
            what = f"member {k}, threshold {threshold}"
            assert sts[k]["rounds"] == st["rounds"], what
            assert sts[k]["infeasible"] == st["infeasible"], what
            assert sts[k]["converged"] == st["converged"], what
            assert sts[k]["rows_deferred"] == st["rows_deferred"], what
            assert sts[k]["full_rounds"] == st["full_rounds"], what
            assert_bitexact(lbs[k], ubs[k], lb, ub, what=what)
        assert tot["infeasible"] >= 1
    if threshold > 1e29:
        assert tot["rows_deferred"] > 0


def test_learned_batch_model_off_equals_plain_batch():
    mips = [gdpgen.chains(10_000, chain_max=50, seed=70 + s, frac_int_vars=1.0) for s in range(2)]
    plain = gdp.Batch.instances(mips, max_rounds=1000)
    r0 = plain.propagate([m.lb for m in mips], [m.ub for m in mips])
    b = gdp.Batch.instances(mips, max_rounds=1000)
    b.set_model(gdp.Mlp(seed=1), 0.0, 8)
    b.set_model(None)
    r1 = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    for k in range(len(mips)):
        assert_bitexact(r0[0][k], r0[1][k], r1[0][k], r1[1][k])
        assert r0[2][k]["rounds"] == r1[2][k]["rounds"]
