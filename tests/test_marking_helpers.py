"""Host-side helpers of learned marking (marking.py): the row length decoded
from feature 0, class-balanced sample weights, and the logit threshold that
keeps a requested recall of the productive rows."""
import numpy as np

import marking


def test_row_length_inverts_feature_0():
    lens = np.array([0, 1, 8, 33, 1000, 65535], np.float64)
    x = np.zeros((len(lens), 16), np.float32)
    x[:, 0] = (np.log2(1.0 + lens) / 16.0).astype(np.float32)
    assert np.array_equal(marking.row_length(x), lens)


def test_balanced_weights_give_each_class_half_the_mass():
    rng = np.random.default_rng(3)
    y = (rng.random(1000) < 0.1).astype(np.float32)
    w = marking.balanced_weights(y)
    assert np.isclose(w[y > 0.5].sum(), 500.0, rtol=1e-5)
    assert np.isclose(w[y <= 0.5].sum(), 500.0, rtol=1e-5)
    cost = rng.uniform(1.0, 50.0, 1000)
    wc = marking.balanced_weights(y, cost)
    assert np.isclose(wc[y > 0.5].sum(), wc[y <= 0.5].sum(), rtol=1e-5)
    # within a class, weights follow the cost
    pos = np.flatnonzero(y > 0.5)
    assert np.allclose(wc[pos] / wc[pos[0]], cost[pos] / cost[pos[0]], rtol=1e-5)


def test_balanced_weights_with_one_class_are_the_costs():
    y = np.zeros(10, np.float32)
    assert np.array_equal(marking.balanced_weights(y), np.ones(10, np.float32))


def test_recall_threshold_is_the_largest_meeting_the_recall():
    rng = np.random.default_rng(5)
    z = rng.normal(size=5000)
    y = (rng.random(5000) < 0.3).astype(np.float32)
    zp = np.sort(z[y > 0.5])
    for recall in (0.5, 0.9, 0.98, 0.999, 1.0):
        t = marking.recall_threshold(z, y, recall)
        kept = np.mean(zp >= t)
        assert kept >= recall - 1e-12
        larger = zp[zp > t]
        if larger.size:  # the next larger sample value would miss the recall
            assert np.mean(zp >= larger[0]) < recall


def test_recall_threshold_without_positives_is_zero():
    assert marking.recall_threshold(np.array([1.0, -2.0]), np.zeros(2, np.float32), 0.9) == 0.0
