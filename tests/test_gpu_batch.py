"""GPU parity of the batched engine: every batch member (instance or node)
must get exactly what a single-problem propagation of it returns -- bounds bit
for bit, round count, infeasibility verdict -- and that in turn is the
oracle's Jacobi result."""
import numpy as np
import pytest

import gdp
import gdpgen
import oracle
from gdp_testutil import assert_bitexact

pytestmark = pytest.mark.gpu


def _single(mip, lb=None, ub=None, marking=-1, max_rounds=0):
    return gdp.propagate(mip, sync_type=gdp.MEGAKERNEL, lb=lb, ub=ub, use_marking=marking, max_rounds=max_rounds)


def _check_member(lb, ub, st, ref_lb, ref_ub, ref_st, what):
    assert st["rounds"] == ref_st["rounds"], what
    assert st["infeasible"] == ref_st["infeasible"], what
    if ref_st["infeasible"]:
        assert st["infeasible_var"] == ref_st["infeasible_var"], what
    assert st["converged"] == ref_st["converged"], what
    assert_bitexact(lb, ub, ref_lb, ref_ub, what=what)


def _mixed_instances():
    mips = [gdpgen.random_mip(0, seed=s) for s in range(3)]
    mips.append(gdpgen.random_mip(1, seed=7, m=30_000, n=22_500, n_dense_rows=2, dense_len=5_000))
    mips.append(gdpgen.chains(20_000, chain_max=60, seed=3))
    mips.append(gdpgen.chains(20_000, chain_max=60, seed=4, infeasible=True))
    mips.append(gdpgen.cover_knapsack(3_000, 300, 2_400, 300, seed=5))
    return mips


@pytest.mark.parametrize("marking", [-1, 0, 2])
def test_instance_batch_equals_single(marking):
    mips = _mixed_instances()
    b = gdp.Batch.instances(mips, use_marking=marking)
    lbs, ubs, sts, tot = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    for k, m in enumerate(mips):
        lb, ub, st = _single(m, marking=marking)
        _check_member(lbs[k], ubs[k], sts[k], lb, ub, st, f"instance {k}")
    assert tot["rounds"] == max(s["rounds"] for s in sts)
    assert tot["infeasible"] == sum(s["infeasible"] for s in sts) >= 1


def test_instance_batch_matches_oracle():
    mips = _mixed_instances()[:4]
    b = gdp.Batch.instances(mips)
    lbs, ubs, sts, _ = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    for k, m in enumerate(mips):
        ref = oracle.propagate(m, oracle.JACOBI, split_len=32, split_tile=1024, nthreads=8)
        assert sts[k]["rounds"] == ref.rounds
        assert bool(sts[k]["infeasible"]) == ref.infeasible
        assert_bitexact(lbs[k], ubs[k], ref.lb, ref.ub, what=f"instance {k}")


def test_batch_in_place_call_equals_into_call():
    """gdp_batch_propagate (bounds in/out) and gdp_batch_propagate_into
    (separate outputs, inputs untouched) give the same members."""
    mips = _mixed_instances()[:4]
    b = gdp.Batch.instances(mips)
    lbs_in = [m.lb.astype(np.float64).copy() for m in mips]
    ubs_in = [m.ub.astype(np.float64).copy() for m in mips]
    r_into = b.propagate(lbs_in, ubs_in)
    for k, m in enumerate(mips):
        assert np.array_equal(lbs_in[k], m.lb) and np.array_equal(ubs_in[k], m.ub)
    k = len(mips)
    pl = (gdp._P_DBL * k)(*[gdp._pd(x) for x in lbs_in])
    pu = (gdp._P_DBL * k)(*[gdp._pd(x) for x in ubs_in])
    assert gdp.load_library().gdp_batch_propagate(b._h, pl, pu, None, None) == gdp.GDP_OKAY
    for i in range(k):
        assert_bitexact(lbs_in[i], ubs_in[i], r_into[0][i], r_into[1][i], what=f"member {i}")


def test_instance_batch_repeat_and_graph():
    """Replaying the captured graph gives the same result; new bounds are honoured."""
    mips = _mixed_instances()[:3]
    b = gdp.Batch.instances(mips)
    r1 = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    r2 = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    for k in range(len(mips)):
        assert_bitexact(r1[0][k], r1[1][k], r2[0][k], r2[1][k])
        assert r1[2][k]["rounds"] == r2[2][k]["rounds"]
    assert b.uses_graph in (True, False)
    ub2 = [m.ub.copy() for m in mips]
    ub2[1][:] = np.minimum(ub2[1], np.maximum(mips[1].lb, 0.0))
    lbs, ubs, sts, _ = b.propagate([m.lb for m in mips], ub2)
    lb, ub, st = _single(mips[1], ub=ub2[1])
    _check_member(lbs[1], ubs[1], sts[1], lb, ub, st, "changed bounds")


def _nodes_from(mip, root_lb, root_ub, n_nodes, seed, infeasible_every=0):
    rng = np.random.default_rng(seed)
    ints = np.flatnonzero((mip.vartype != 3) & np.isfinite(root_lb) & np.isfinite(root_ub)
                          & (root_ub - root_lb >= 1) & (np.abs(root_lb) < 1e19) & (np.abs(root_ub) < 1e19))
    lbs, ubs = [], []
    for k in range(n_nodes):
        lb, ub = root_lb.copy(), root_ub.copy()
        fix = rng.choice(ints, size=min(len(ints), int(rng.integers(1, 51))), replace=False)
        v = np.floor(lb[fix] + rng.random(len(fix)) * (ub[fix] - lb[fix] + 1))
        v = np.minimum(v, ub[fix])
        lb[fix] = v
        ub[fix] = v
        if infeasible_every and k % infeasible_every == 0:
            j = fix[0]
            lb[j], ub[j] = ub[j] + 1.0, ub[j]
        lbs.append(lb)
        ubs.append(ub)
    return lbs, ubs


@pytest.mark.parametrize("marking", [-1, 0, 2])
def test_node_batch_from_certified_root(marking):
    """Nodes = root fixpoint + fixings; round 1 starts from the marks of the
    fixed variables. Each node equals its own full propagation."""
    mip = gdpgen.random_mip(1, seed=11, m=40_000, n=30_000, n_dense_rows=2, dense_len=8_000)
    ctx = gdp.Context(mip, sync_type=gdp.MEGAKERNEL, use_marking=marking)
    rlb, rub, rst = ctx.propagate()
    assert rst["converged"] and not rst["infeasible"]
    lbs, ubs = _nodes_from(mip, rlb, rub, 24, seed=1, infeasible_every=7)
    b = gdp.Batch.nodes(ctx, len(lbs))
    blb, bub, sts, tot = b.propagate(lbs, ubs)
    for k in range(len(lbs)):
        lb, ub, st = _single(mip, lb=lbs[k], ub=ubs[k], marking=marking)
        _check_member(blb[k], bub[k], sts[k], lb, ub, st, f"node {k}")
    assert tot["infeasible"] >= 1
    if marking != 0:
        # the marked start processes far fewer rows than full first sweeps would
        assert tot["rows_processed"] < len(lbs) * mip.m


def test_node_batch_without_certified_root():
    """A context whose last propagation stopped at a round cap has no certified
    fixpoint: nodes then sweep every row in round 1 and still match."""
    mip = gdpgen.random_mip(1, seed=12, m=20_000, n=15_000, n_dense_rows=1, dense_len=4_000)
    ctx = gdp.Context(mip, sync_type=gdp.MEGAKERNEL, max_rounds=2)
    rlb, rub, rst = ctx.propagate()
    assert not rst["converged"]
    lbs, ubs = _nodes_from(mip, rlb, rub, 8, seed=2)
    b = gdp.Batch.nodes(ctx, len(lbs))
    blb, bub, sts, _ = b.propagate(lbs, ubs)
    for k in range(len(lbs)):
        lb, ub, st = _single(mip, lb=lbs[k], ub=ubs[k], max_rounds=2)
        _check_member(blb[k], bub[k], sts[k], lb, ub, st, f"node {k}")


def test_node_equal_to_root_converges_in_one_round():
    mip = gdpgen.random_mip(0, seed=13)
    ctx = gdp.Context(mip, sync_type=gdp.MEGAKERNEL)
    rlb, rub, _ = ctx.propagate()
    b = gdp.Batch.nodes(ctx, 3)
    blb, bub, sts, _ = b.propagate([rlb] * 3, [rub] * 3)
    for k in range(3):
        assert sts[k]["rounds"] == 1 and sts[k]["converged"] and not sts[k]["infeasible"]
        assert sts[k]["rows_processed"] == 0
        assert_bitexact(blb[k], bub[k], rlb, rub)


def test_batch_round_cap():
    mips = [gdpgen.chains(10_000, chain_max=300, seed=s) for s in (1, 2)]
    b = gdp.Batch.instances(mips, max_rounds=5)
    lbs, ubs, sts, _ = b.propagate([m.lb for m in mips], [m.ub for m in mips])
    for k, m in enumerate(mips):
        lb, ub, st = _single(m, max_rounds=5)
        _check_member(lbs[k], ubs[k], sts[k], lb, ub, st, f"capped {k}")
