"""The CPU oracle of the learned-proposal network, pinned by central finite
differences of its own loss (the network has no counterpart in the
reference)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp  # noqa: E402


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    theta = rng.normal(0.0, 0.3, mlp.N_PARAMS)
    X = rng.normal(0.0, 1.0, (24, mlp.LF))
    T = rng.normal(0.0, 1.0, 24)
    _, g = mlp.loss_grad(theta, X, T)
    idx = rng.choice(mlp.N_PARAMS, size=60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(mlp.N_PARAMS)
        e[i] = h
        fd = (mlp.loss_grad(theta + e, X, T)[0] - mlp.loss_grad(theta - e, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
