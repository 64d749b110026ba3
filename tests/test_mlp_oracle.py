"""The CPU restatement of the warm-start MLP (oracle/mlp_oracle.py): its
analytic gradient against central finite differences (float64, no BF16
rounding)."""
import numpy as np

from oracle import mlp_oracle as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(64 * 128 + 128 + 128 * 128 + 128 + 128 * 3 + 3) * 0.1
    X = rng.standard_normal((7, 64))
    T = rng.standard_normal((7, 3))
    loss, g = M.loss_grad(X, T, p, round_bf16=False)
    idx = rng.choice(p.size, 40, replace=False)
    idx = np.concatenate([idx, [p.size - 1, p.size - 4, 64 * 128 + 5]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = M.loss_grad(X, T, p + e, round_bf16=False)
        lm, _ = M.loss_grad(X, T, p - e, round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - (-3.140625)) < 1e-12 and r[4] == 0.0
