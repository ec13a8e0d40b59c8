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


def proto_digits(n: int, seed: int, proto_seed: int = 20240605, d: int = 784, n_proto: int = 10,
                 support: float = 0.2, keep: float = 0.9, extra: float = 0.015):
    """Sparse-valued dense rows from seeded prototype patterns: prototype k
    lights a random ``support`` fraction of the d pixels with base
    intensities U(0.3, 1); a sample of class k keeps each lit pixel with
    probability ``keep`` (intensity x (1 + 0.25 N(0, 1))), lights each other
    pixel with probability ``extra`` (U(0, 0.5)), and is quantised to 8-bit
    integers / 255 (about 19 % nonzero). Label +1 for prototypes 0-4, -1 for
    5-9. The prototypes come from ``proto_seed`` so that sets drawn with
    different ``seed`` share them. Returns the dense (n, d) matrix and labels."""
    prng = np.random.default_rng(proto_seed)
    lit = np.zeros((n_proto, d), dtype=bool)
    base = np.zeros((n_proto, d))
    for k in range(n_proto):
        idx = prng.choice(d, size=int(round(support * d)), replace=False)
        lit[k, idx] = True
        base[k, idx] = prng.uniform(0.3, 1.0, size=idx.size)
    rng = np.random.default_rng(seed)
    cls = rng.integers(0, n_proto, n)
    X = np.zeros((n, d), dtype=np.float32)
    chunk = 8192
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        k = cls[a:b]
        on = lit[k] & (rng.random((b - a, d)) < keep)
        val = base[k] * (1.0 + 0.25 * rng.standard_normal((b - a, d)))
        ex = (~lit[k]) & (rng.random((b - a, d)) < extra)
        val = np.where(ex, rng.uniform(0.0, 0.5, (b - a, d)), np.where(on, val, 0.0))
        X[a:b] = np.rint(np.clip(val, 0.0, 1.0) * 255.0)
    y = np.where(cls < n_proto // 2, 1.0, -1.0)
    return X.astype(np.float64) / 255.0, y


def precision_full_workload(n_train=100_000, n_test=10_000, seed=20240606):
    """Full-IRWLS workload of the precision form: 784 features, 8-bit values,
    about 19 % nonzero, prototypes 0-4 against 5-9 (zeros omitted, so the
    reader flags the set as sparse)."""
    Xtr, ytr = proto_digits(n_train, seed)
    Xte, yte = proto_digits(n_test, seed + 1)
    return from_dense(Xtr, ytr, keep_zeros=False), from_dense(Xte, yte, keep_zeros=False)


def sparse_linear_pool(n: int = 50_000, d: int = 300, density: float = 0.03, seed: int = 20240607,
                       rule_nnz: int = 100, flip: float = 0.08) -> Sparse:
    """CSR rows over d features at the given density: even features are
    binary (1.0), odd ones U(0, 1). Labels are the sign of a seeded sparse
    linear rule (rule_nnz N(0, 1) weights, centred at its median), with a
    fraction ``flip`` flipped."""
    rng = np.random.default_rng(seed)
    mask = rng.random((n, d)) < density
    vals = np.where(np.arange(d) % 2 == 0, 1.0, rng.random((n, d)))
    X = np.where(mask, vals, 0.0)
    w = np.zeros(d)
    w[rng.choice(d, size=rule_nnz, replace=False)] = rng.standard_normal(rule_nnz)
    s = X @ w
    y = np.where(s >= np.median(s), 1.0, -1.0)
    y = np.where(rng.random(n) < flip, -y, y)
    return from_dense(X, y, keep_zeros=False)


def subset(data: Sparse, rows) -> Sparse:
    """The given rows of a CSR set, in the given order."""
    rows = np.asarray(rows)
    counts = np.diff(data.indptr)[rows]
    indptr = np.concatenate([[0], np.cumsum(counts)])
    take = np.concatenate([np.arange(data.indptr[r], data.indptr[r + 1]) for r in rows]) if len(rows) else []
    take = np.asarray(take, dtype=np.int64)
    return Sparse(indptr, data.indices[take], data.values[take], data.y[rows], data.d)


def batch_workload(seed: int = 20240608, n_min: int = 2000, n_max: int = 50_000, linear: int = 8):
    """SVMs of the batching form: an 8 x 8 grid of C in logspace(-1, 3, 8) x
    gamma in logspace(-3, 0, 8) (RBF) plus ``linear`` linear-kernel SVMs over
    the C grid, each on its own random subset of the pool with a size drawn
    log-uniform in [n_min, n_max]. Returns (pool, [(rows, kernel, C, gamma)])."""
    pool = sparse_linear_pool()
    rng = np.random.default_rng(seed)
    Cs, gammas = np.logspace(-1, 3, 8), np.logspace(-3, 0, 8)
    specs = [(1, c, g) for c in Cs for g in gammas] + [(0, Cs[k % 8], 1.0) for k in range(linear)]
    jobs = []
    for kern, c, g in specs:
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        rows = np.sort(rng.choice(pool.n, size=n, replace=False))
        jobs.append((rows, kern, float(c), float(g)))
    return pool, jobs


def gauss_mixture(n: int, seed: int, family_seed: int = 20240609, k: int = 50, d: int = 32, flip: float = 0.03,
                  mean_scale: float = 0.6, spread=(0.08, 0.22)):
    """Dense rows from a mixture of k seeded Gaussians with random
    covariances (x = mu_j + s_j R_j z, R_j with N(0, 1/d) entries, s_j drawn
    from ``spread``); label +1 for even components and -1 for odd ones, with a
    fraction ``flip`` flipped. ``family_seed`` draws the mixture, ``seed`` the
    rows. Values are rounded to FP32. Returns (X, y)."""
    frng = np.random.default_rng(family_seed)
    mu = frng.normal(0.0, mean_scale, (k, d))
    R = frng.normal(0.0, 1.0 / np.sqrt(d), (k, d, d)) * frng.uniform(spread[0], spread[1], (k, 1, 1))
    rng = np.random.default_rng(seed)
    comp = rng.integers(0, k, n)
    X = np.empty((n, d))
    for a in range(0, n, 65536):
        b = min(n, a + 65536)
        z = rng.standard_normal((b - a, d))
        X[a:b] = mu[comp[a:b]] + np.einsum("nij,nj->ni", R[comp[a:b]], z)
    y = np.where(comp % 2 == 0, 1.0, -1.0)
    y = np.where(rng.random(n) < flip, -y, y)
    return X.astype(np.float32).astype(np.float64), y


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


def dataset_digest(hd) -> str:
    """SHA-256 of a dataset exactly as the library reads it: the feature
    array (index/value pairs with their -1 terminators, class-mean rows
    included), every row's offset, the labels, the norms and the header
    fields. Two machines that rebuild a seeded workload agree on it only if
    every number the training sees is the same."""
    import hashlib

    h = hashlib.sha256()
    h.update(np.array([hd.l, hd.sparse, hd.maxdim, hd.n_rows], dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(hd.features).tobytes())
    h.update(np.ascontiguousarray(hd.row_start, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(hd.y, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(hd.q, dtype=np.float64).tobytes())
    return h.hexdigest()
