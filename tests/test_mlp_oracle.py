"""The MLP oracle's gradient formulas against central finite differences (FP64,
no BF16 rounding): validates the restatement the GPU kernels are checked against."""
import numpy as np

from oracle import mlp_oracle as mo


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    p = mo.init_params(1).astype(np.float64)
    p[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.1, mo.H)
    p[mo.OFF_B2:mo.OFF_W3] = rng.normal(0, 0.1, mo.H)
    x = rng.normal(0, 1, (40, mo.IN))
    y = (rng.random(40) < 0.4).astype(float)
    w = rng.uniform(0.5, 2.0, 40)
    _, g = mo.loss_and_grad(p, x, y, w, bf16_round=False)
    idx = np.concatenate([rng.choice(np.arange(mo.OFF_W1, mo.OFF_B1), 20), rng.choice(np.arange(mo.OFF_B1, mo.OFF_W2), 8),
                          rng.choice(np.arange(mo.OFF_W2, mo.OFF_B2), 30), rng.choice(np.arange(mo.OFF_B2, mo.OFF_W3), 8),
                          np.arange(mo.OFF_W3, mo.OFF_W3 + 8), [mo.OFF_B3]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_and_grad(pp, x, y, w, False)[0] - mo.loss_and_grad(pm, x, y, w, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    # spacing at 1.0 is 2^-7; halfway cases round to the even mantissa
    v = np.array([1.0, 1 + 2 ** -8, 1 + 2 ** -9, 1 + 3 * 2 ** -8, 1 + 2 ** -8 + 2 ** -12, -3.14159, 0.0], np.float32)
    r = mo.bf16(v)
    assert list(r[:5]) == [1.0, 1.0, 1.0, 1.015625, 1.0078125]
    assert r[6] == 0.0
    assert abs(r[5] - v[5]) <= 2 ** -8 * abs(v[5])
