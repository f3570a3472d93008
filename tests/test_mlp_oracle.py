"""CPU checks of the NumPy restatement of the warm-start network: with the
BF16 rounding points switched off its gradient equals central finite
differences of its loss, and BF16 rounding matches round-to-nearest-even."""
import numpy as np

from oracle import mlp_oracle as MO


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 1e-30, 65504.0], dtype=np.float32)
    r = MO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125            # above the tie rounds up
    assert abs(r[3] - (-3.140625)) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_gradient_equals_finite_differences():
    rng = np.random.default_rng(0)
    shape = (7, 9, 6, 4)
    n = 9 * 7 + 9 + 6 * 9 + 6 + 4 * 6 + 4
    p = rng.standard_normal(n) * 0.5
    X = rng.standard_normal((5, 7))
    T = rng.standard_normal((5, 4))
    MO.EXACT = True
    try:
        _, g = MO.loss_and_gradient(p, shape, X, T)
        h = 1e-6
        for k in rng.choice(n, 25, replace=False):
            e = np.zeros(n)
            e[k] = h
            fd = (MO.loss_and_gradient(p + e, shape, X, T)[0] - MO.loss_and_gradient(p - e, shape, X, T)[0]) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])
    finally:
        MO.EXACT = False
