"""The row test of rows summed by several lanes, restated on the CPU.

The reference decides canConsBeTightened (src/propagation_methods.cuh:136-154)
with its sequential EPS-max of |a|(ub-lb) (computeActivities :188-190: an
element replaces the running value m only if it exceeds m by more than EPS).
The GPU kernels sum such rows in lane groups and warp tiles, and decide the
row test from the row's first FP64 maximum (M, p) instead
(gdp_device.cuh:row_go_from_max), falling back to the recursion
m(E) = fl(M - m(p)) > EPS ? M : m(p) over prefix maxima
(gdp_round.cuh:seq_eps_max) when fl(M - slack) lies in (EPS, 2.00001e-9].

These tests restate that procedure in plain Python and check it against the
sequential definition on sequences built to stress it: values within EPS of
each other, long chains of near-equal values (deeper than the kernels' 32
stack levels), negative values (crossed bounds), infinities and NaN.
"""
import math
import random

import numpy as np
import pytest

EPS = 1e-9
INF = 1e20
GO_CLEAR = 2.00001e-9


def eps_gt(x, y):
    return (x - y) > EPS


def seq_eps_max(d):
    m = 0.0
    for x in d:
        if eps_gt(x, m):
            m = x
    return m


def first_max(d, e):
    """First maximum of d[0:e] with the leading 0.0 at index -1; NaN never counts."""
    best, p = 0.0, -1
    for k in range(e):
        x = d[k]
        if not math.isnan(x) and x > best:
            best, p = x, k
    return best, p


def eps_max_by_prefix_maxima(d, levels=32):
    """gdp_round.cuh:seq_eps_max restated: a stack of prefix maxima, one per
    level, a serial scan below the deepest level."""
    M, p = first_max(d, len(d))
    stack, E = [], len(d)
    while True:
        if p < 0:
            x = 0.0
            break
        if len(stack) == levels:
            x = seq_eps_max(d[:E])
            break
        stack.append(M)
        M2, p2 = first_max(d, p)
        if p2 >= 0 and eps_gt(M, M2):
            x = stack.pop()
            break
        E, M, p = p, M2, p2
    while stack:
        Mi = stack.pop()
        if eps_gt(Mi, x):
            x = Mi
    return x


def row_go_reference(m, mn):
    if m < INF:
        return not ((m - mn) <= EPS)
    return True


def row_go_from_max(d, mn):
    """gdp_device.cuh:row_go_from_max, completed by the prefix recursion."""
    M, _ = first_max(d, len(d))
    if M >= INF:
        return True
    v = M - mn
    if v <= EPS:
        return False
    if v > GO_CLEAR or v != v:
        return True
    return row_go_reference(eps_max_by_prefix_maxima(d), mn)


def _sequences(rng: random.Random):
    base = rng.choice([1e-9, 3e-9, 1.0, 7.5, 1e3, 1e6])
    n = rng.randint(1, 200)
    kind = rng.randrange(6)
    if kind == 0:  # values within a few EPS of each other
        return [base + rng.uniform(-3, 3) * EPS for _ in range(n)]
    if kind == 1:  # an increasing chain of steps just under EPS, shuffled in parts
        d = [base + i * 0.9 * EPS for i in range(n)]
        if rng.random() < 0.5:
            k = rng.randint(0, n)
            d[k:] = reversed(d[k:])
        return d
    if kind == 2:  # crossed bounds and zeros
        return [rng.choice([0.0, -0.0, -1.0, base, base + 0.5 * EPS, base + 1.5 * EPS]) for _ in range(n)]
    if kind == 3:  # infinities and huge values
        return [rng.choice([base, math.inf, 2e20, 1e20, base + EPS]) for _ in range(n)]
    if kind == 4:  # NaN terms (inf - inf) never count
        return [rng.choice([base, math.nan, base + 1.2 * EPS, base - 0.7 * EPS]) for _ in range(n)]
    return [rng.uniform(0, base) for _ in range(n)]


def test_prefix_maxima_equal_sequential_eps_max():
    rng = random.Random(1234)
    for _ in range(20_000):
        d = _sequences(rng)
        assert eps_max_by_prefix_maxima(d) == seq_eps_max(d) or (
            math.isnan(seq_eps_max(d)) and math.isnan(eps_max_by_prefix_maxima(d)))


def test_deep_chain_beyond_the_stack():
    # each element exceeds the previous by 0.9 EPS: the first maximum is the
    # last element, and every prefix level is within EPS of the next
    d = [1.0 + i * 0.9 * EPS for i in range(100)]
    assert eps_max_by_prefix_maxima(d, levels=32) == seq_eps_max(d)
    assert eps_max_by_prefix_maxima(d, levels=4) == seq_eps_max(d)


def test_row_decision_from_maximum_equals_reference():
    rng = random.Random(99)
    checked_band = 0
    for _ in range(20_000):
        d = _sequences(rng)
        M, _ = first_max(d, len(d))
        # slacks around the maximum, in and out of the (EPS, 2.00001e-9] band
        for mn in (M - rng.uniform(0, 3) * EPS, M - 1.5 * EPS, M, M + EPS, -1.0, math.inf, -math.inf,
                   math.nan):
            ref = row_go_reference(seq_eps_max(d), mn)
            assert row_go_from_max(d, mn) == ref, (d[:8], mn)
            v = M - mn
            checked_band += int(EPS < v <= GO_CLEAR)
    assert checked_band > 1000


def test_clear_margin_is_safe_across_magnitudes():
    """v = fl(M - mn) > 2.00001e-9 implies fl(m - mn) > EPS whatever m the
    prefix leaves (m >= M - EPS - ulp(EPS)/2)."""
    rng = np.random.default_rng(5)
    for scale in (1e-9, 1e-3, 1.0, 1e3, 1e7):
        for _ in range(2000):
            M = scale * (1 + rng.random())
            m = M - EPS * rng.random()  # the lowest m the sequential rule can leave
            mn = M - GO_CLEAR * (1 + rng.random() * 1e-3)
            if (M - mn) > GO_CLEAR:
                assert (m - mn) > EPS
