"""The precision form's full-IRWLS error update (the persistent tcgen05
kernel of dev_tc.cu) in both operand forms, checked through whole trainings
against the CPU oracle (the restatement of the reference, FP64):

- one exact bf16 piece when the data are 8-bit values k / 255 or binary
  (the products are exact; only the FP32 accumulation rounds);
- three pieces (hi + mid + lo of the FP32 value) otherwise.

On the integer-valued sets the rows that decide the support vectors (the
exact set, the working set, G13) take the exact-integer mode: dot products
exact on the tensor cores, exp and sums in FP64.

Bars (the precision form's contract): the support-vector set of the oracle,
the dual objective within 1e-5 relative, >= 99.9 % of the held-out labels.
Prediction in the precision form (the same engine, f = b + sum w k) is
checked against the library's FP64 prediction. Also: the kernel's bounded
waits, made to run out with the test hook
irwls_debug_tc_wait (no MMA issued, so nothing is in flight), fail the
training with -13 and leave the library usable."""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load, synth

pytestmark = pytest.mark.gpu

DUAL_TOL = 1e-5


def _sets(kind, n, n_test, seed):
    if kind == "digits":
        X, y = synth.proto_digits(n + n_test, seed, d=196, n_proto=10)
        tr = synth.from_dense(X[:n], y[:n], keep_zeros=False)
        te = synth.from_dense(X[n:], y[n:], keep_zeros=False)
    elif kind == "binary":
        tr = synth.mixed_onehot(n, seed, n_cont=0, groups=(4, 12, 40), label_seed=seed + 1)
        te = synth.mixed_onehot(n_test, seed + 7, n_cont=0, groups=(4, 12, 40), label_seed=seed + 1)
    else:
        tr = synth.mixed_onehot(n, seed, label_seed=seed + 1)
        te = synth.mixed_onehot(n_test, seed + 7, label_seed=seed + 1)
    hd = _abi.build_dataset(tr.indptr, tr.indices, tr.values, tr.y)
    ht = _abi.build_dataset(te.indptr, te.indices, te.values, te.y, with_means=False)
    return hd, ht


def _debug_wait(lib, limit, stall):
    lib.irwls_debug_tc_wait.argtypes = [C.c_longlong, C.c_int]
    lib.irwls_debug_tc_wait.restype = None
    lib.irwls_debug_tc_wait(limit, stall)


def _mixed_full(lib, hd, p):
    lib.irwls_set_precision(1)
    try:
        return H.run_full(lib, hd, p)
    finally:
        lib.irwls_set_precision(0)


@pytest.mark.parametrize("kind,pieces,gamma", [("digits", 1, 0.05), ("binary", 1, 0.1), ("gauss", 3, 0.1)])
def test_precision_full_operand_forms_match_oracle(kind, pieces, gamma):
    lib = load()
    lib.irwls_tc_exact_calls.argtypes = [C.c_int]
    lib.irwls_tc_exact_calls.restype = C.c_longlong
    hd, ht = _sets(kind, 3000, 600, 91)
    p = {"gamma": gamma, "C": 10.0, "w": 300, "kernel": 1}
    lib.irwls_tc_exact_calls(1)
    beta, ptr, prop = _mixed_full(lib, hd, p)
    exact_calls = lib.irwls_tc_exact_calls(1)
    assert lib.irwls_tc_status() == 0
    assert lib.irwls_last_tc_pieces() == pieces
    # integer-valued data (8-bit / 255, binary) take the exact-integer mode for
    # the exact rows, the working-set updates and G13; FP32-split data do not
    assert (exact_calls > 0) == (pieces == 1), exact_calls
    ref, rptr, _ = H.run_full(H.port(), hd, p)
    same_sv = np.array_equal(np.nonzero(beta[:-1])[0], np.nonzero(ref[:-1])[0])
    d_ref = H.dual_objective(hd, ref, p["gamma"], 1)
    d_got = H.dual_objective(hd, beta, p["gamma"], 1)
    print("%s: %d SVs, beta rel err %.3g, dual rel err %.3g" % (kind, int((ref[:-1] != 0).sum()),
                                                              H.rel_err(beta, ref), abs(d_got - d_ref) / abs(d_ref)))
    assert same_sv
    assert abs(d_got - d_ref) <= DUAL_TOL * abs(d_ref)
    mdl = lib.calculateFULLModel(prop, hd.struct, ptr)
    try:
        labels = H.predict(lib, ht, mdl, 0)
    finally:
        lib.freeModel(mdl)
    # the oracle's weights packed by the library's host C model packing
    mref = lib.calculateFULLModel(prop, hd.struct, rptr)
    try:
        want = H.predict(H.port(), ht, mref, 0)
    finally:
        lib.freeModel(mref)
    assert float((labels == want).mean()) >= 0.999


def test_precision_full_wait_timeout_is_reported_and_recovers():
    lib = load()
    hd, _ = _sets("digits", 1500, 10, 93)
    p = {"gamma": 0.05, "C": 10.0, "w": 200, "kernel": 1}
    good, _, _ = _mixed_full(lib, hd, p)
    assert lib.irwls_tc_status() == 0
    _debug_wait(lib, 2000, 1)
    try:
        lib.irwls_set_precision(1)
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=1, working_set=p["w"])
        lib.initMemory(1, p["w"] + 1)
        H.LIBC.srand(0)
        ptr = lib.trainFULL(hd.struct, prop)
    finally:
        _debug_wait(lib, 0, 0)
        lib.irwls_set_precision(0)
    assert not ptr
    assert lib.irwls_last_error() == -13
    assert b"ran out" in lib.irwls_last_error_message()
    assert lib.irwls_tc_status() == 0  # the failed training read and cleared it
    again, _, _ = _mixed_full(lib, hd, p)
    assert lib.irwls_tc_status() == 0
    assert np.array_equal(again, good)


@pytest.mark.parametrize("kind", ["digits", "gauss"])
def test_precision_prediction_matches_fp64(kind):
    lib = load()
    hd, ht = _sets(kind, 3000, 2500, 95)
    p = {"gamma": 0.05, "C": 10.0, "w": 300, "kernel": 1}
    beta, ptr, prop = H.run_full(lib, hd, p)
    mdl = lib.calculateFULLModel(prop, hd.struct, ptr)
    try:
        soft64 = H.predict(lib, ht, mdl, 1)
        hard64 = H.predict(lib, ht, mdl, 0)
        lib.irwls_set_precision(1)
        try:
            soft = H.predict(lib, ht, mdl, 1)
            hard = H.predict(lib, ht, mdl, 0)
        finally:
            lib.irwls_set_precision(0)
    finally:
        lib.freeModel(mdl)
    assert lib.irwls_tc_status() == 0
    err = float(np.abs(soft - soft64).max() / np.abs(soft64).max())
    print("%s: %d SVs, decision values rel err %.3g" % (kind, int((beta[:-1] != 0).sum()), err))
    assert err <= 1e-5
    assert np.array_equal(hard, np.where(soft >= 0, 1.0, -1.0))
    assert float((hard == hard64).mean()) >= 0.999
