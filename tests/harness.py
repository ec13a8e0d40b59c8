"""Shared helpers of the tests: golden fixtures, dataset construction and
runners that drive any library exporting the reference API (the GPU library
or the CPU oracle) through the same C ABI."""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

from libirwls_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
PORT_PATH = os.path.join(ROOT, "oracle", "_build", "libirwls_port.so")
LIBC = C.CDLL(None)

FULL_CASES = ["full_dense", "full_sparse", "full_linear", "full_smallws", "full_cfg1"]
BUDGET_CASES = ["budget_sgma", "budget_sgma_dense", "budget_random", "budget_linear", "budget_cfg2_reduced"]

# Parity bar: identical index sets / labels, weights within 1e-9 relative
# (relative to the largest weight magnitude of the reference run).
REL_TOL = 1e-9


def golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: z[k] for k in z.files}


def params(g):
    return json.loads(str(g["params"]))


def datasets(g):
    tr = _abi.build_dataset(g["train_indptr"], g["train_indices"], g["train_values"], g["train_y"])
    te = _abi.build_dataset(g["test_indptr"], g["test_indices"], g["test_values"], g["test_y"], with_means=False)
    return tr, te


_port = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
        _port = _abi.load_library(PORT_PATH)
    return _port


def arr(ptr, n, dtype=np.float64):
    assert ptr, "entry point returned NULL"
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype).copy()


def run_full(lib, hd, p):
    """trainFULL with the full-train CLI's seed (srand(0))."""
    prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], working_set=p["w"])
    lib.initMemory(1, p["w"] + 1)
    LIBC.srand(0)
    ptr = lib.trainFULL(hd.struct, prop)
    return arr(ptr, hd.l + 1), ptr, prop


def run_budget(lib, hd, p):
    """SGMA or random centroids then IRWLSpar, with glibc's default seed."""
    prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=p["size"],
                                algorithm=p["algorithm"])
    lib.initMemory(1, p["size"])
    LIBC.srand(1)
    c = lib.SGMA(hd.struct, prop) if p["algorithm"] == 1 else lib.randomCentroids(hd.struct, prop)
    cent = arr(c, p["size"], np.int32)
    w = lib.IRWLSpar(hd.struct, c, prop)
    return cent, arr(w, p["size"]), c, w, prop


def predict(lib, ht, mdl, soft):
    pp = _abi.make_predict_properties(labels=0, soft=soft)
    f = lib.softTest if soft else lib.test
    return arr(f(ht.struct, mdl, pp), ht.l)


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def dual_objective(hd, beta, gamma, kernel):
    """D(beta) = sum_i y_i beta_i - 1/2 beta^T K beta over the training rows
    (beta_i = alpha_i y_i), in FP64 on the host; K in the reference's kernel
    form for the dataset (dense raw form when sparse == 0)."""
    rows, y, q = _abi.dataset_rows(hd.struct, hd.l)
    d = max([int(r[0].max()) for r in rows if len(r[0])] + [0]) + 1
    X = np.zeros((hd.l, d))
    for i, (ix, v) in enumerate(rows):
        X[i, ix] = v
    b = beta[:hd.l]
    sv = np.nonzero(b)[0]
    Xs = X[sv]
    if kernel == 0:
        K = Xs @ Xs.T
    else:
        sq = (Xs * Xs).sum(1)
        K = np.exp(-gamma * np.maximum(sq[:, None] + sq[None, :] - 2 * Xs @ Xs.T, 0.0))
    bs = b[sv]
    return float((y[sv] * bs).sum() - 0.5 * bs @ K @ bs)


def budget_primal(hd, cent, w, gamma, cost, kernel):
    """Budgeted primal 1/2 w^T (K_mm + 1e-5 I) w + C sum_i max(0, 1 - y_i f_i),
    f = K_nm w over the training rows, in FP64 on the host (centroid indices
    may name the class-mean rows l and l+1)."""
    rows, y, q = _abi.dataset_rows(hd.struct, hd.n_rows)
    d = max([int(r[0].max()) for r in rows if len(r[0])] + [0]) + 1
    X = np.zeros((hd.n_rows, d))
    for i, (ix, v) in enumerate(rows):
        X[i, ix] = v
    Xc = X[np.asarray(cent)]
    if kernel == 0:
        Kmm, Knm = Xc @ Xc.T, X[:hd.l] @ Xc.T
    else:
        qc = q[np.asarray(cent)]
        Kmm = np.exp(-gamma * (qc[:, None] + qc[None, :] - 2.0 * Xc @ Xc.T))
        Knm = np.exp(-gamma * (q[:hd.l, None] + qc[None, :] - 2.0 * X[:hd.l] @ Xc.T))
    w = np.asarray(w)
    f = Knm @ w
    return float(0.5 * w @ (Kmm + 1e-5 * np.eye(len(w))) @ w + cost * np.maximum(0.0, 1.0 - y[:hd.l] * f).sum())
