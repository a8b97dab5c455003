"""The NumPy network oracle's backpropagation against central finite
differences (no rounding, float64), so that the GPU gradient check rests on a
verified restatement."""
import numpy as np

from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    W = rng.uniform(-0.3, 0.3, (6, 64, 64))
    W[5][:, 3:] = 0
    x = rng.uniform(-1, 1, (8, 64))
    t = np.zeros((8, 4))
    t[:, :3] = rng.uniform(0, 1, (8, 3))
    loss, g = mlp_ref.loss_and_grad(W, x, t, "fp32")
    y0, _ = mlp_ref.forward(W, x, "fp32")
    den = y0.astype(np.float64) ** 2 + 0.01

    def surrogate(Wp):
        y, _ = mlp_ref.forward(Wp, x, "fp32")
        return np.sum((y - t[:, :3]) ** 2 / den) / len(x)

    h = 1e-6
    for (l, i, j) in [(0, 3, 5), (2, 10, 40), (4, 63, 0), (5, 7, 2), (5, 0, 0)]:
        Wp, Wm = W.copy(), W.copy()
        Wp[l, i, j] += h
        Wm[l, i, j] -= h
        num = (surrogate(Wp) - surrogate(Wm)) / (2 * h)
        assert abs(num - g[l, i, j]) <= 1e-5 * max(1.0, abs(num)), (l, i, j, num, g[l, i, j])
    assert abs(loss / len(x) - surrogate(W)) < 1e-9
