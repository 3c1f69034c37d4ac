"""The FP64 restatement of the warm-start network (oracle/mlp_oracle.py) checked against
finite differences, so that it can serve as the checker of the GPU gradients."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = M.n_params()
    p = rng.normal(size=n) * 0.05
    X = M.encode(rng.uniform(-1, 1, (7, 3)))
    C = rng.normal(size=(7, 3))
    T = rng.normal(size=(7, 5)) * 0.1
    _, g, _ = M.loss_and_grad(p, X, C, T)
    for i in rng.choice(n, 40, replace=False):
        e = np.zeros(n)
        e[i] = 1e-6
        fd = (M.loss_and_grad(p + e, X, C, T)[0] - M.loss_and_grad(p - e, X, C, T)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-5 * abs(g[i]) + 1e-10


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.0e-3, 65504.0])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert abs(r[3] - x[3]) <= 2 ** -8 * abs(x[3])  # half an ulp of an 8-bit significand
    assert abs(r[4] - x[4]) <= 2 ** -8 * x[4]
