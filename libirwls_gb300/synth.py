"""Seeded synthetic workloads for tests and benchmarks.

The reference's only public benchmark input is the a9a set that its demo
downloads; it is not available offline, so these seeded generators stand in
for it with the shapes and value distributions of the workloads the library
is measured on. Every generator returns CSR arrays with 1-based feature
indices (what a libsvm file holds) plus labels in {+1, -1}; ``write_libsvm``
writes them with 17 significant digits so any libsvm reader recovers the same
doubles.
"""
from __future__ import annotations

import numpy as np


class Sparse:
    """CSR rows with 1-based feature indices (libsvm convention)."""

    def __init__(self, indptr, indices, values, y, d):
        self.indptr = np.asarray(indptr, dtype=np.int64)
        self.indices = np.asarray(indices, dtype=np.int32)
        self.values = np.asarray(values, dtype=np.float64)
        self.y = np.asarray(y, dtype=np.float64)
        self.d = int(d)

    @property
    def n(self) -> int:
        return len(self.indptr) - 1

    def dense(self) -> np.ndarray:
        X = np.zeros((self.n, self.d + 1))
        rows = np.repeat(np.arange(self.n), np.diff(self.indptr))
        X[rows, self.indices] = self.values
        return X[:, 1:]


def from_dense(X: np.ndarray, y: np.ndarray, keep_zeros: bool) -> Sparse:
    """Rows of X as libsvm entries; ``keep_zeros`` writes every feature (the
    reader then flags the set as dense), else zeros are omitted."""
    n, d = X.shape
    mask = np.ones_like(X, dtype=bool) if keep_zeros else (X != 0.0)
    counts = mask.sum(axis=1)
    indptr = np.concatenate([[0], np.cumsum(counts)])
    rr, cc = np.nonzero(mask)
    return Sparse(indptr, cc + 1, X[rr, cc], y, d)


def two_gaussians(n: int, d: int, seed: int, shift: float = 0.5, flip: float = 0.10):
    """Two isotropic unit-variance Gaussian classes with means +-shift*1 and a
    fraction ``flip`` of labels flipped."""
    rng = np.random.default_rng(seed)
    y = np.where(rng.random(n) < 0.5, 1.0, -1.0)
    X = rng.standard_normal((n, d)) + shift * y[:, None]
    flipped = rng.random(n) < flip
    y = np.where(flipped, -y, y)
    return X, y


def full_dense_workload(n_train=4000, n_test=1000, d=20, seed=20240601):
    """Dense full-IRWLS workload: every feature written (sparse == 0)."""
    X, y = two_gaussians(n_train + n_test, d, seed)
    tr = from_dense(X[:n_train], y[:n_train], keep_zeros=True)
    te = from_dense(X[n_train:], y[n_train:], keep_zeros=True)
    return tr, te


def mixed_onehot(n: int, seed: int, n_cont=10, groups=(4, 40), hidden=16, flip=0.05, label_seed=None):
    """n_cont N(0,1) features plus one-hot groups; labels from the sign of a
    seeded random 2-layer tanh network, with a fraction ``flip`` flipped.
    Zeros are omitted, so the reader flags the set as sparse. The network is
    drawn from ``label_seed`` when given (so that a test set drawn with
    another ``seed`` shares the training set's labelling function), else from
    the same stream as the rows."""
    rng = np.random.default_rng(seed)
    d = n_cont + sum(groups)
    X = np.zeros((n, d))
    X[:, :n_cont] = rng.standard_normal((n, n_cont))
    off = n_cont
    for g in groups:
        X[np.arange(n), off + rng.integers(0, g, n)] = 1.0
        off += g
    frng = rng if label_seed is None else np.random.default_rng(label_seed)
    W1 = frng.standard_normal((d, hidden)) / np.sqrt(d)
    w2 = frng.standard_normal(hidden)
    s = np.tanh(X @ W1 * 2.0) @ w2
    y = np.where(s >= (np.median(s) if label_seed is None else 0.0), 1.0, -1.0)
    y = np.where(rng.random(n) < flip, -y, y)
    return from_dense(X, y, keep_zeros=False)


def budgeted_workload(n=200_000, seed=20240602, label_seed=20240603):
    """Budgeted-IRWLS workload: 10 continuous + one-hot(4) + one-hot(40)."""
    return mixed_onehot(n, seed, label_seed=label_seed)


def budgeted_test_set(n=20_000, seed=20240604, label_seed=20240603):
    """Held-out rows labelled by the same network as budgeted_workload()."""
    return mixed_onehot(n, seed, label_seed=label_seed)


def write_libsvm(path: str, data: Sparse, labeled: bool = True) -> None:
    with open(path, "w") as f:
        ip, ix, vv = data.indptr, data.indices, data.values
        for i in range(data.n):
            parts = []
            if labeled:
                parts.append("%d" % int(data.y[i]))
            for k in range(ip[i], ip[i + 1]):
                parts.append("%d:%.17g" % (ix[k], vv[k]))
            f.write(" ".join(parts) + "\n")
