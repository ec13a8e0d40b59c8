"""Failure paths of the library, made on the host (no GPU fault is caused):

- an allocation that fails (injected through irwls_debug_fail_alloc at every
  position of a training's allocation sequence) makes the call return NULL
  with error -3, and the next call trains normally, equal to the reference's
  golden result;
- a non-finite feature value or label makes training and prediction return
  NULL with error -4 before any device work;
- a system whose Cholesky meets a pivot that is not positive is solved as
  the reference's LAPACK call leaves it (src/ParallelAlgorithms.c:277-282 and
  :383 ignore dpotrf's info), and the condition is reported through
  irwls_last_error as the warning IRWLS_WARN_PIVOT.
"""
import ctypes as C

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load

pytestmark = pytest.mark.gpu

PD = C.POINTER(C.c_double)
WARN_PIVOT = 1


def _lib():
    lib = load()
    assert lib.irwls_gpu_available(), lib.irwls_last_error_message()
    lib.irwls_debug_fail_alloc.argtypes = [C.c_longlong]
    lib.irwls_debug_fail_alloc.restype = None
    return lib


@pytest.mark.parametrize("k", [1, 2, 3, 4, 6, 9, 14, 20])
def test_injected_allocation_failure_full(k):
    lib = _lib()
    g = H.golden("full_sparse")
    p = H.params(g)
    hd, _ = H.datasets(g)
    lib.irwls_debug_fail_alloc(k)
    try:
        prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], working_set=p["w"])
        lib.initMemory(1, p["w"] + 1)
        H.LIBC.srand(0)
        ptr = lib.trainFULL(hd.struct, prop)
    finally:
        lib.irwls_debug_fail_alloc(0)
    if ptr:
        # the training made fewer than k allocations: nothing failed
        assert lib.irwls_last_error() == 0
    else:
        assert lib.irwls_last_error() == -3
        assert b"injected" in lib.irwls_last_error_message()
    beta, _, _ = H.run_full(lib, hd, p)
    assert np.array_equal(beta[:-1] != 0, g["beta"][:-1] != 0)
    assert H.rel_err(beta, g["beta"]) <= H.REL_TOL


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 12, 18])
def test_injected_allocation_failure_budgeted(k):
    lib = _lib()
    g = H.golden("budget_sgma")
    p = H.params(g)
    hd, _ = H.datasets(g)
    prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=p["size"],
                                algorithm=p["algorithm"])
    lib.initMemory(1, p["size"])
    H.LIBC.srand(1)
    c = lib.SGMA(hd.struct, prop)
    assert c, lib.irwls_last_error_message()
    lib.irwls_debug_fail_alloc(k)
    try:
        w = lib.IRWLSpar(hd.struct, c, prop)
    finally:
        lib.irwls_debug_fail_alloc(0)
    if not w:
        assert lib.irwls_last_error() == -3
        assert b"injected" in lib.irwls_last_error_message()
    cent, w2, _, _, _ = H.run_budget(lib, hd, p)
    assert np.array_equal(cent, g["centroids"])
    assert H.rel_err(w2, g["weights"]) <= H.REL_TOL


def _with_value(g, row, value=None, label=None):
    ip, ix, vv, y = g["train_indptr"], g["train_indices"], g["train_values"].copy(), g["train_y"].copy()
    if value is not None:
        vv[ip[row]] = value
    if label is not None:
        y[row] = label
    return _abi.build_dataset(ip, ix, vv, y)


@pytest.mark.parametrize("bad", [dict(value=np.nan), dict(value=np.inf), dict(label=np.nan), dict(label=-np.inf)])
def test_non_finite_input_is_rejected(bad):
    lib = _lib()
    g = H.golden("full_sparse")
    p = H.params(g)
    hd = _with_value(g, 17, **bad)
    prop = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], working_set=p["w"])
    lib.initMemory(1, p["w"] + 1)
    H.LIBC.srand(0)
    assert not lib.trainFULL(hd.struct, prop)
    assert lib.irwls_last_error() == -4
    assert b"non-finite" in lib.irwls_last_error_message()
    bp = _abi.make_properties(gamma=p["gamma"], C_=p["C"], kernel=p["kernel"], size=8, algorithm=1)
    H.LIBC.srand(1)
    assert not lib.SGMA(hd.struct, bp)
    assert lib.irwls_last_error() == -4
    # the library stays usable
    hd_ok, _ = H.datasets(g)
    beta, _, _ = H.run_full(lib, hd_ok, p)
    assert H.rel_err(beta, g["beta"]) <= H.REL_TOL


def test_non_finite_test_value_is_rejected_by_prediction():
    lib = _lib()
    g = H.golden("full_sparse")
    p = H.params(g)
    hd, _ = H.datasets(g)
    beta, ptr, prop = H.run_full(lib, hd, p)
    mdl = lib.calculateFULLModel(prop, hd.struct, ptr)
    te = g["test_values"].copy()
    te[3] = np.nan
    ht = _abi.build_dataset(g["test_indptr"], g["test_indices"], te, g["test_y"], with_means=False)
    assert not lib.softTest(ht.struct, mdl, _abi.make_predict_properties(soft=1))
    assert lib.irwls_last_error() == -4
    lib.freeModel(mdl)


def _solve(lib, A, b):
    n = len(b)
    M = np.asfortranarray(A).ravel(order="F").copy()
    x = np.zeros(n)
    lib.ParallelLinearSystem(M.ctypes.data_as(PD), n, n, 0, 0, b.ctypes.data_as(PD), n, 1, 0, 0, n, 1,
                             x.ctypes.data_as(PD), n, 1, 0, 0, 1)
    return x


def test_failed_pivot_is_reported_as_a_warning():
    lib = _lib()
    z = np.load(H.GOLDEN + "/solver.npz")
    # SPD: no warning
    A, b = z["solve_200_spd_A"], z["solve_200_spd_b"]
    x = _solve(lib, A, b)
    assert lib.irwls_last_error() == 0
    assert H.rel_err(x, z["solve_200_spd_x"]) <= 1e-10
    # bordered system of full IRWLS: its last pivot fails by construction; the
    # reference's solution stands and the failed pivot is reported
    A, b = z["solve_251_bordered_A"], z["solve_251_bordered_b"]
    x = _solve(lib, A, b)
    assert lib.irwls_last_error() == WARN_PIVOT
    assert b"pivot 251 " in lib.irwls_last_error_message()
    assert H.rel_err(x, z["solve_251_bordered_x"]) <= 1e-10
    # an indefinite matrix: the first failed pivot is the one reported
    rng = np.random.default_rng(5)
    Q = rng.standard_normal((40, 40))
    S = Q @ Q.T + 40 * np.eye(40)
    S[6, 6] = -1.0
    _solve(lib, S, rng.standard_normal(40))
    assert lib.irwls_last_error() == WARN_PIVOT
    assert b"pivot 7 " in lib.irwls_last_error_message()
    # the next call starts clean
    _solve(lib, z["solve_200_spd_A"], z["solve_200_spd_b"])
    assert lib.irwls_last_error() == 0
