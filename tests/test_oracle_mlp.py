"""The picker network's CPU restatement: its analytic gradient matches
central finite differences (float64, no bf16 rounding)."""
import numpy as np

from oracle import mlp_ref as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, M.NPARAM)
    X = rng.normal(0, 1, (40, M.NF))
    y = rng.integers(0, 3, 40)
    _, g = M.loss_and_grad(p, X, y, bf16=False, dtype=np.float64)
    idx = rng.choice(M.NPARAM, 200, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = M.loss_and_grad(q, X, y, bf16=False, dtype=np.float64)
        q[i] -= 2 * eps
        lm, _ = M.loss_and_grad(q, X, y, bf16=False, dtype=np.float64)
        assert abs((lp - lm) / (2 * eps) - g[i]) < 1e-6 + 1e-4 * abs(g[i])


def test_bf16_round_ties_to_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 0.0], dtype=np.float32)
    r = M.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == -2.5 and r[4] == 0.0
