"""CPU oracle of the learned-proposal network (test infrastructure only).

The proposal network of the library's learned SGMA form -- 8 features ->
128 -> 128 -> 1 with ReLU, parameters flattened as W1 [128][8], b1 [128],
W2 [128][128], b2 [128], W3 [1][128], b3 [1] -- restated in numpy (float64)
with its mean-squared-error gradient, so that tests can check the GPU forward
and backward kernels. The reference has no such network: it is part of the
the benchmark spec's learned form, not of the reference's algorithm, so this oracle
is pinned against central finite differences of its own loss instead of
against reference outputs.
"""
import numpy as np

LF, LH = 8, 128
SIZES = [("W1", (LH, LF)), ("b1", (LH,)), ("W2", (LH, LH)), ("b2", (LH,)), ("W3", (1, LH)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(theta):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(theta[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(parts):
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).ravel() for name, _ in SIZES])


def forward(theta, X):
    p = unpack(theta)
    A1 = np.maximum(X @ p["W1"].T + p["b1"], 0.0)
    A2 = np.maximum(A1 @ p["W2"].T + p["b2"], 0.0)
    P = (A2 @ p["W3"].T + p["b3"])[:, 0]
    return P, (A1, A2)


def loss_grad(theta, X, T):
    """Mean squared error of forward(theta, X) against T and its gradient in
    the flattened layout."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    p = unpack(theta)
    P, (A1, A2) = forward(theta, X)
    n = X.shape[0]
    e = P - T
    dP = 2.0 * e / n
    g = {"W3": dP[None, :] @ A2, "b3": np.array([dP.sum()])}
    dA2 = (dP[:, None] @ p["W3"]) * (A2 > 0)
    g["W2"] = dA2.T @ A1
    g["b2"] = dA2.sum(0)
    dA1 = (dA2 @ p["W2"]) * (A1 > 0)
    g["W1"] = dA1.T @ X
    g["b1"] = dA1.sum(0)
    return float((e * e).mean()), pack(g)
