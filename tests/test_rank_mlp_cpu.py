"""The CPU restatement of the rank predictor (oracle/rank_mlp.py), which the GPU gradients are
checked against, is itself checked here: its hand-written backward pass against central finite
differences of its forward pass, and its BF16 rounding against round-to-nearest-even."""
import numpy as np

from oracle import rank_mlp as R


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(R.P) * 0.2
    X = rng.standard_normal((7, R.F))
    t = rng.standard_normal(7)
    g, _ = R.gradient(p, X, t, rounded=False)
    idx = rng.choice(R.P, size=60, replace=False)
    idx[:6] = [0, R.F * R.H, R.F * R.H + R.H + 5, R.P - 66, R.P - 2, R.P - 1]  # one in every block
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = np.mean((R.forward(pp, X, rounded=False)[0] - t) ** 2)
        lm = np.mean((R.forward(pm, X, rounded=False)[0] - t) ** 2)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5 + 2 ** -10, 3.1415926], dtype=np.float32)
    r = R.bf16_round(x)
    # 8 significant bits: 1 + 2^-8 is a tie -> even (1.0); 1 + 3 2^-9 rounds up to 1 + 2^-7
    np.testing.assert_array_equal(r[:3], [1.0, 1.0, 1.0 + 2 ** -7])
    assert abs(r[4] - 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)
