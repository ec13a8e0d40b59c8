"""Batching form (irwls_full_train_batch / irwls_budgeted_train_batch): SVMs
of different sizes, kernels, C, gamma and seeds trained concurrently on
separate streams must give bit for bit what the single-call API gives after
srand(seed), whatever the worker count."""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load, synth

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)


def _jobs():
    jobs = []
    for k, (n, kern, cost, gamma, ws) in enumerate([(900, 1, 10.0, 0.05, 120), (400, 1, 1.0, 0.5, 60),
                                                    (1500, 1, 100.0, 0.1, 200), (650, 0, 1.0, 1.0, 80),
                                                    (300, 1, 1.0, 0.5, 7), (1200, 1, 10.0, 0.2, 150)]):
        d = synth.mixed_onehot(n, seed=100 + k) if k % 2 else synth.from_dense(
            *synth.two_gaussians(n, 6, 200 + k), keep_zeros=True)
        hd = _abi.build_dataset(d.indptr, d.indices, d.values, d.y)
        p = _abi.make_properties(gamma=gamma, C_=cost, kernel=kern, working_set=ws, size=12 + 3 * k,
                                 algorithm=1 if k % 3 else 0)
        jobs.append((hd, p, 11 + 7 * k))
    return jobs


@pytest.mark.parametrize("workers", [1, 3, 8])
def test_full_batch_equals_sequential(workers):
    lib = load()
    jobs = _jobs()
    ref = []
    for hd, p, seed in jobs:
        lib.initMemory(1, p.MaxSize + 1)
        H.LIBC.srand(seed)
        ref.append(H.arr(lib.trainFULL(hd.struct, p), hd.l + 1))
    n = len(jobs)
    dss = (_abi.SvmDataset * n)(*[j[0].struct for j in jobs])
    prs = (_abi.Properties * n)(*[j[1] for j in jobs])
    seeds = (C.c_uint * n)(*[j[2] for j in jobs])
    out = (PD * n)()
    assert lib.irwls_full_train_batch(dss, prs, seeds, n, workers, out) == 0
    for i, (hd, _, _) in enumerate(jobs):
        got = np.ctypeslib.as_array(out[i], shape=(hd.l + 1,)).copy()
        assert np.array_equal(got, ref[i]), "SVM %d differs from its single-call training" % i


def test_budgeted_batch_equals_sequential():
    lib = load()
    jobs = _jobs()
    ref = []
    for hd, p, seed in jobs:
        lib.initMemory(1, p.size)
        H.LIBC.srand(seed)
        c = lib.SGMA(hd.struct, p) if p.algorithm == 1 else lib.randomCentroids(hd.struct, p)
        cent = H.arr(c, p.size, np.int32)
        ref.append((cent, H.arr(lib.IRWLSpar(hd.struct, c, p), p.size)))
    n = len(jobs)
    dss = (_abi.SvmDataset * n)(*[j[0].struct for j in jobs])
    prs = (_abi.Properties * n)(*[j[1] for j in jobs])
    seeds = (C.c_uint * n)(*[j[2] for j in jobs])
    cents, weights = (PI * n)(), (PD * n)()
    assert lib.irwls_budgeted_train_batch(dss, prs, seeds, n, 4, cents, weights) == 0
    for i, (_, p, _) in enumerate(jobs):
        assert np.array_equal(np.ctypeslib.as_array(cents[i], shape=(p.size,)), ref[i][0])
        assert np.array_equal(np.ctypeslib.as_array(weights[i], shape=(p.size,)), ref[i][1])


def test_batch_reports_a_failing_svm():
    lib = load()
    jobs = _jobs()[:3]
    bad = _abi.make_properties(gamma=0.1, C_=1.0, working_set=0)  # working set must be positive
    n = len(jobs)
    dss = (_abi.SvmDataset * n)(*[j[0].struct for j in jobs])
    prs = (_abi.Properties * n)(jobs[0][1], bad, jobs[2][1])
    out = (PD * n)()
    assert lib.irwls_full_train_batch(dss, prs, None, n, 2, out) != 0
    assert b"working-set size" in lib.irwls_last_error_message()
    assert not out[1]
    assert out[0] and out[2]
