"""The MLP's CUDA forward and gradient kernels against the numpy oracle (same
BF16 rounding points; tolerances cover FP32 accumulation order and the rare
BF16 tie that a different summation order rounds the other way), and GPU
training on a learnable synthetic task."""
import numpy as np
import pytest

import gdp
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, mo.IN)).astype(np.float32)
    y = (x[:, 0] + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3] > 0.2).astype(np.float32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return x, y, w


def _params(seed):
    rng = np.random.default_rng(seed)
    p = mo.init_params(seed)
    p[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.1, mo.H)
    p[mo.OFF_B2:mo.OFF_W3] = rng.normal(0, 0.1, mo.H)
    p[mo.OFF_B3] = 0.05
    return p.astype(np.float32)


@pytest.mark.parametrize("n", [1, 15, 16, 333, 5000])
def test_forward_matches_oracle(n):
    m = gdp.Mlp(seed=1)
    p = _params(3)
    m.params = p
    assert np.array_equal(m.params, p)
    x, _, _ = _data(n, 7)
    z = m.forward(x)
    z_ref, _ = mo.forward(p, x)
    scale = np.abs(z_ref).mean() + 1e-3
    err = np.abs(z - z_ref)
    assert np.median(err) <= 1e-3 * scale + 1e-5
    assert err.max() <= 0.05 * scale + 1e-3


@pytest.mark.parametrize("n", [16, 100, 4096])
def test_gradient_matches_oracle(n):
    m = gdp.Mlp(seed=2)
    p = _params(5)
    m.params = p
    x, y, w = _data(n, 11)
    loss, g = m.gradient(x, y, w)
    loss_ref, g_ref = mo.loss_and_grad(p, x, y, w)
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref) + 1e-5
    for name, a, b in (("W1", mo.OFF_W1, mo.OFF_B1), ("b1", mo.OFF_B1, mo.OFF_W2), ("W2", mo.OFF_W2, mo.OFF_B2),
                       ("b2", mo.OFF_B2, mo.OFF_W3), ("w3", mo.OFF_W3, mo.OFF_B3), ("b3", mo.OFF_B3, mo.N_PARAMS)):
        rel = np.linalg.norm(g[a:b] - g_ref[a:b]) / (np.linalg.norm(g_ref[a:b]) + 1e-12)
        assert rel < 2e-2, (name, rel)


def test_training_learns():
    x, y, w = _data(60_000, 13)
    xt, yt, _ = _data(10_000, 14)
    m = gdp.Mlp(seed=4)
    z0 = m.forward(xt)
    acc0 = np.mean((z0 > 0) == (yt > 0.5))
    final = m.train(x, y, w, epochs=8, batch=2048, lr=3e-3, seed=1)
    z = m.forward(xt)
    acc = np.mean((z > 0) == (yt > 0.5))
    assert final < 0.35
    assert acc > 0.9 and acc > acc0
    # the trained parameters give the same loss through the oracle
    loss_ref, _ = mo.loss_and_grad(m.params, x, y, w)
    loss_gpu, _ = m.gradient(x, y, w)
    assert abs(loss_gpu - loss_ref) <= 1e-2 * loss_ref + 1e-4
