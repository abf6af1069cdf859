"""CPU checks of the learned part's restatement (oracle/mlp_oracle.py): the
backward formulas against central finite differences, and bf16 rounding."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounds_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.3e-5], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even mantissa
    assert r[2] == np.float32(1.0 + 2 ** -6)  # tie -> even (up)
    assert r[3] == -2.5
    assert abs(r[4] - 3.3e-5) <= 3.3e-5 * 2 ** -8


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, M.NPARAM)
    x = rng.normal(0, 1, (64, M.NIN))
    y = rng.poisson(1.5, (64, M.NOUT)).astype(np.float64)
    _, g = M.loss_grad(p, x, y, round_bf16=False)
    idx = rng.choice(M.NPARAM, 60, replace=False)
    h = 1e-6
    for k in idx:
        e = np.zeros(M.NPARAM)
        e[k] = h
        fd = (M.loss_grad(p + e, x, y, False)[0] - M.loss_grad(p - e, x, y, False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, g[k])
