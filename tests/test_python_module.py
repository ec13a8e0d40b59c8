"""The Python-3 LIBIRWLS module (libirwls_gb300.LIBIRWLS): dataset builders
against a restatement of the reference module's numpy conversion, model
save/load on the CPU, and training/prediction on the GPU against the CPU
oracle fed with the same datasets."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import LIBIRWLS, _abi, load

PD = C.POINTER(C.c_double)


def _numpy2dataset_rows(X):
    """pythonmodule.c:213-263: every non-zero value is feature j+1."""
    rows = []
    for r in X:
        nz = np.nonzero(r)[0]
        rows.append((nz + 1, r[nz]))
    return rows


def _data(n=300, d=6, seed=9, zeros=True):
    X, y = __import__("libirwls_gb300.synth", fromlist=["x"]).two_gaussians(n, d, seed)
    if zeros:
        X[np.abs(X) < 0.3] = 0.0
    return np.ascontiguousarray(X), y


def test_dense_builder_matches_module_conversion():
    lib = load()
    X, y = _data()
    ds = lib.irwls_dataset_from_dense(X.ctypes.data_as(PD), y.ctypes.data_as(PD), X.shape[0], X.shape[1])
    rows, yy, q = _abi.dataset_rows(ds, X.shape[0])
    want = _numpy2dataset_rows(X)
    for (i1, v1), (i2, v2) in zip(rows, want):
        assert np.array_equal(i1, i2) and np.array_equal(v1, v2)
    assert np.array_equal(yy, y)
    assert ds.sparse == 1 and ds.maxdim == X.shape[1]
    for k in range(X.shape[0]):
        acc = 0.0
        for v in want[k][1]:
            acc = acc + v * v
        assert q[k] == acc
    lib.freeDataset(ds)


def test_mean_rows_builder_reproduces_module_layout():
    """pythonmodule.c:277-355: the positive mean row lists features 1..d plus a
    trailing index-0 entry, the negative mean row is empty, and the two mean
    "norms" are plain sums of the mean values."""
    lib = load()
    X, y = _data()
    n, d = X.shape
    ds = lib.irwls_dataset_from_dense_with_means(X.ctypes.data_as(PD), y.ctypes.data_as(PD), n, d)
    rows, yy, q = _abi.dataset_rows(ds, n + 2)
    pos = y == 1.0
    mean_p = np.zeros(d)
    for i in range(n):
        if pos[i]:
            for j in np.nonzero(X[i])[0]:
                mean_p[j] += X[i, j] / pos.sum()
    idx_p, val_p = rows[n]
    assert list(idx_p) == list(range(1, d + 1)) + [0]
    assert np.allclose(val_p[:d], mean_p, rtol=0, atol=1e-15) and val_p[d] == 0.0
    assert len(rows[n + 1][0]) == 0
    assert yy[n] == 1.0 and yy[n + 1] == -1.0
    assert abs(q[n] - val_p.sum()) < 1e-12
    lib.freeDataset(ds)


def test_save_load_roundtrip_of_a_reference_model():
    g = H.golden("full_dense")
    with tempfile.NamedTemporaryFile(delete=False) as f:
        f.write(g["model_bytes"].tobytes())
        path = f.name
    try:
        clf = LIBIRWLS.load(path)
        path2 = path + ".2"
        LIBIRWLS.save(clf, path2)
        assert open(path2, "rb").read() == g["model_bytes"].tobytes()
        os.unlink(path2)
    finally:
        os.unlink(path)


@pytest.mark.gpu
def test_module_training_matches_oracle():
    lib = load()
    port = H.port()
    X, y = _data(n=400, d=6)
    n, d = X.shape
    # full training through the module vs the oracle on the module's dataset
    H.LIBC.srand(0)
    clf = LIBIRWLS.full_train(X, y, gamma=0.5, C=2.0, workingSet=60, verbose=0)
    ds = lib.irwls_dataset_from_dense(X.ctypes.data_as(PD), y.ctypes.data_as(PD), n, d)
    p = _abi.make_properties(gamma=0.5, C_=2.0, working_set=60)
    port.initMemory(1, 61)
    H.LIBC.srand(0)
    ref_beta = H.arr(port.trainFULL(ds, p), n + 1)
    nz = ref_beta[:-1] != 0
    assert clf.nSVs == int(nz.sum())
    assert H.rel_err(clf.weights(), ref_beta[:-1][nz]) < 1e-9
    soft = LIBIRWLS.predict(clf, X, Soft=1, verbose=0)
    hard = LIBIRWLS.predict(clf, X, verbose=0)
    assert np.array_equal(hard, np.where(soft >= 0, 1.0, -1.0))
    lib.freeDataset(ds)
    # budgeted training with SGMA through the module vs the oracle
    H.LIBC.srand(1)
    bclf = LIBIRWLS.budgeted_train(X, y, gamma=0.5, C=2.0, size=12, algorithm=1, verbose=0)
    dsm = lib.irwls_dataset_from_dense_with_means(X.ctypes.data_as(PD), y.ctypes.data_as(PD), n, d)
    pb = _abi.make_properties(gamma=0.5, C_=2.0, size=12, algorithm=1)
    port.initMemory(1, 12)
    H.LIBC.srand(1)
    c = port.SGMA(dsm, pb)
    w = H.arr(port.IRWLSpar(dsm, c, pb), 12)
    assert H.rel_err(bclf.weights(), w) < 1e-9
    lib.freeDataset(dsm)


def test_precision_switch():
    assert LIBIRWLS.get_precision() == "fp64"
    LIBIRWLS.set_precision("mixed")
    try:
        assert LIBIRWLS.get_precision() == "mixed"
        assert load().irwls_get_precision() == 1
    finally:
        LIBIRWLS.set_precision("fp64")
    with pytest.raises(ValueError):
        LIBIRWLS.set_precision("fp16")
