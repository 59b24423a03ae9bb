"""The CPU reference of the selector network: gradients against central
differences (no GPU)."""
import numpy as np

from oracle import mlp as ref


def _data(n=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, ref.IN)).astype(np.float32) * 3 + 1
    Y = rng.normal(size=(n, ref.OUT)).astype(np.float32)
    p = ref.init_params(X, seed)
    return X, Y, p


def test_gradient_finite_difference_cpu():
    """The numpy reference gradient itself against central differences."""
    X, Y, p = _data(n=64, seed=2)
    p = p.astype(np.float64)
    _, g = ref.loss_and_grad(p, X.astype(np.float64), Y.astype(np.float64))
    rng = np.random.default_rng(3)
    o = ref.offsets()
    for name in ("W1", "W3", "b4"):
        a, n = o[name]
        for k in rng.choice(n, 5, replace=False):
            e = np.zeros_like(p)
            e[a + k] = 1e-6
            lp, _ = ref.loss_and_grad(p + e, X, Y)
            lm, _ = ref.loss_and_grad(p - e, X, Y)
            assert abs((lp - lm) / 2e-6 - g[a + k]) <= 1e-5 + 1e-4 * abs(g[a + k])
