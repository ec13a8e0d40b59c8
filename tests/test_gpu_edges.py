"""Edge cases of the precision, batching and learned forms: budgets of 1-3,
sets smaller than one 128-row tile, tiny working sets, empty and single-SVM
batches, a proposer under a linear kernel (random candidates stay), and
trace requests that must fail cleanly."""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, learned, load, synth

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)


def _small(n, seed, d=5, kernel=1):
    X, y = synth.two_gaussians(n, d, seed)
    return _abi.build_dataset(*_csr(X, y))


def _csr(X, y):
    s = synth.from_dense(X, y, keep_zeros=True)
    return s.indptr, s.indices, s.values, s.y


def _budget(lib, hd, p, precision):
    lib.irwls_set_precision(precision)
    try:
        lib.initMemory(1, p.size)
        H.LIBC.srand(1)
        c = lib.SGMA(hd.struct, p) if p.algorithm == 1 else lib.randomCentroids(hd.struct, p)
        assert c, lib.irwls_last_error_message()
        w = lib.IRWLSpar(hd.struct, c, p)
        assert w, lib.irwls_last_error_message()
        return H.arr(c, p.size, np.int32), H.arr(w, p.size)
    finally:
        lib.irwls_set_precision(0)


@pytest.mark.parametrize("m", [1, 2, 3])
def test_precision_budgeted_tiny_budgets_and_sets(m):
    lib = load()
    hd = _small(50, 3)
    p = _abi.make_properties(gamma=0.2, C_=5.0, size=m, algorithm=1)
    c0, w0 = _budget(lib, hd, p, 0)
    c1, w1 = _budget(lib, hd, p, 1)
    assert np.array_equal(c0, c1)
    assert H.rel_err(w1, w0) < 1e-6


def test_precision_full_tiny_set_and_working_set():
    lib = load()
    hd = _small(40, 5)
    p = {"gamma": 0.3, "C": 2.0, "w": 8, "kernel": 1}
    b0, _, _ = H.run_full(lib, hd, p)
    lib.irwls_set_precision(1)
    try:
        b1, _, _ = H.run_full(lib, hd, p)
    finally:
        lib.irwls_set_precision(0)
    assert np.array_equal(b0[:-1] != 0, b1[:-1] != 0)
    d0, d1 = H.dual_objective(hd, b0, 0.3, 1), H.dual_objective(hd, b1, 0.3, 1)
    assert abs(d1 - d0) <= 1e-9 * abs(d0)


def test_batch_of_zero_and_one():
    lib = load()
    hd = _small(300, 7)
    p = _abi.make_properties(gamma=0.2, C_=1.0, working_set=40)
    assert lib.irwls_full_train_batch(None, None, None, 0, 4, None) == 0
    dss = (_abi.SvmDataset * 1)(hd.struct)
    prs = (_abi.Properties * 1)(p)
    seeds = (C.c_uint * 1)(9)
    out = (PD * 1)()
    assert lib.irwls_full_train_batch(dss, prs, seeds, 1, 4, out) == 0
    lib.initMemory(1, 41)
    H.LIBC.srand(9)
    ref = H.arr(lib.trainFULL(hd.struct, p), hd.l + 1)
    assert np.array_equal(np.ctypeslib.as_array(out[0], shape=(hd.l + 1,)), ref)


def test_proposer_leaves_linear_kernels_on_random_candidates():
    lib = load()
    hd = _small(600, 11)
    p = _abi.make_properties(gamma=1.0, C_=1.0, kernel=0, size=10, algorithm=1)
    c0, w0 = _budget(lib, hd, p, 1)
    net = learned.Proposer(seed=1)
    net.install(pool=256)
    try:
        c1, w1 = _budget(lib, hd, p, 1)
    finally:
        net.close()
    assert np.array_equal(c0, c1)
    assert np.array_equal(w0, w1)


def test_traces_reject_small_budgets():
    lib = load()
    hd = _small(200, 13)
    p = _abi.make_properties(gamma=0.5, C_=1.0, size=2, algorithm=1)
    with pytest.raises(RuntimeError):
        learned.traces(hd, p)
    p_lin = _abi.make_properties(gamma=0.5, C_=1.0, kernel=0, size=10, algorithm=1)
    with pytest.raises(RuntimeError):
        learned.traces(hd, p_lin)
