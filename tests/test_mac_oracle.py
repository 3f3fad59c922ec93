"""The CPU oracle of the learned-MAC MLP: its analytic gradient equals finite
differences of its loss (without the BF16 rounding, where the loss is smooth
almost everywhere), and the BF16 rounding helper rounds to nearest even."""
import numpy as np

from oracle import mac_oracle as M


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0 + 2 ** -7 or r[1] == 1.0  # tie to even
    assert r[1] == 1.0  # 1 + 2^-8 is halfway: even mantissa is 1.0
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, M.NPARAMS)
    x = rng.normal(0, 1, (64, M.F))
    t = rng.normal(-3, 1, 64)
    _, g = M.loss_grad(p, x, t, round_bf16=False)
    idx = rng.choice(M.NPARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = M.loss(q, x, t, round_bf16=False)
        q[i] -= 2 * h
        lm = M.loss(q, x, t, round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])
